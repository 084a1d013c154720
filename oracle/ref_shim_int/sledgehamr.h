/* ORACLE (test infrastructure only).
 *
 * Stand-in for source/sledgehamr.h when the reference's integrators are
 * compiled unchanged (oracle/ref_integrators.cpp): the members of
 * Sledgehamr they use (nghost, with_gravitational_waves, FillRhs,
 * FillAddRhs, level_synchronizer->FillIntermediatePatch), to be provided by
 * the test driver.
 */
#ifndef SH_REF_SHIM_INT_SLEDGEHAMR_H_
#define SH_REF_SHIM_INT_SLEDGEHAMR_H_

#include "AMReX_MultiFab.H"

namespace sledgehamr {

class LevelSynchronizer {
  public:
    virtual ~LevelSynchronizer() = default;
    virtual void FillIntermediatePatch(int lev, double time, amrex::MultiFab &mf) = 0;
};

class Sledgehamr {
  public:
    virtual ~Sledgehamr() = default;
    virtual void FillRhs(amrex::MultiFab &rhs, const amrex::MultiFab &state, double time,
                         int lev, double dt, double dx) = 0;
    virtual void FillAddRhs(amrex::MultiFab &rhs, const amrex::MultiFab &state, double time,
                            int lev, double dt, double dx, double weight) = 0;
    int nghost = 0;
    bool with_gravitational_waves = false;
    LevelSynchronizer *level_synchronizer = nullptr;
};

} // namespace sledgehamr

#endif // SH_REF_SHIM_INT_SLEDGEHAMR_H_
