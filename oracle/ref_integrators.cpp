/* ORACLE (test infrastructure only): oracle/_ref/libshref_int.so.
 *
 * The reference's own integrators - source/integrators/rkn.cpp (RKN4,
 * RKN5), lsssprk3.cpp and leapfrog.cpp, compiled unchanged from the
 * sledgehamr sources - run on a periodic single-box level of the AMReX
 * stand-in (oracle/ref_shim_int), with the Rhs of the reference's own
 * per-cell project headers (ref_fill_rhs of oracle/_ref/libshref.so) and
 * periodic ghost fills as FillIntermediatePatch.  Each step is
 * Integrator::Advance for a periodic level (integrator.cpp:11-31): swap,
 * ghost fill of the old state at its time, Integrate, t_new = t_old + dt.
 * Built by oracle/build_ref.sh; compared with the oracle's integrator
 * drivers by tests/test_oracle_ref.py.  Also the reference's header-only
 * gw_GetProjection / gw_GetLambda (source/gravitational_waves.h), tabled by
 * ref_gw_lambda_table.
 */
#include <cstring>

#include "leapfrog.h"
#include "lsssprk3.h"
#include "rkn.h"

/* gravitational_waves.h includes the sibling sledgehamr.h by quotes, which
 * would find the reference's full header (AMReX's AmrCore): its include
 * guard is taken here, the stand-in already declared what the GW header
 * needs */
#define SLEDGEHAMR_SLEDGEHAMR_H_
#include "gravitational_waves.h"

extern "C" int ref_fill_rhs(int project, int N, int nghost, int ncomp, int with_gw,
                            const double *state_in, double *rhs_out, double time, int lev,
                            double dt, double dx, const double *params,
                            const double *gw_params, int ko_order, const double *ko_strength);

/* Integrator::Advance lives in integrator.cpp with the AMR level storage;
 * the loop of ref_int_evolve below does its work for one periodic level. */
void sledgehamr::Integrator::Advance(const int) {
    throw std::runtime_error("Integrator::Advance is replaced by ref_int_evolve");
}

namespace {

using amrex::MultiFab;

struct PeriodicSync : sledgehamr::LevelSynchronizer {
    void FillIntermediatePatch(int, double, MultiFab &mf) override { mf.FillBoundaryPeriodic(); }
};

/* valid cells to / from the canonical layout (ncomp, N, N, N), x fastest */
void gather(const MultiFab &mf, std::vector<double> &out) {
    const int N = mf.size(), nc = mf.nComp();
    out.resize((size_t)nc * N * N * N);
    size_t q = 0;
    for (int n = 0; n < nc; ++n)
        for (int k = 0; k < N; ++k)
            for (int j = 0; j < N; ++j)
                for (int i = 0; i < N; ++i) out[q++] = mf.at(i, j, k, n);
}
void scatter(const std::vector<double> &in, MultiFab &mf) {
    const int N = mf.size(), nc = mf.nComp();
    size_t q = 0;
    for (int n = 0; n < nc; ++n)
        for (int k = 0; k < N; ++k)
            for (int j = 0; j < N; ++j)
                for (int i = 0; i < N; ++i) mf.at(i, j, k, n) = in[q++];
}

struct Sim : sledgehamr::Sledgehamr {
    int project = 0;
    std::vector<double> params, gw_params;
    void FillRhs(MultiFab &rhs, const MultiFab &state, double time, int lev, double dt,
                 double dx) override {
        std::vector<double> s, r;
        gather(state, s);
        r.assign(s.size(), 0.);
        if (ref_fill_rhs(project, state.size(), nghost, state.nComp(), with_gravitational_waves,
                         s.data(), r.data(), time, lev, dt, dx, params.data(), gw_params.data(),
                         0, nullptr) != 0)
            throw std::runtime_error("ref_fill_rhs failed");
        scatter(r, rhs);
    }
    /* SLEDGEHAMR_PRJ_FILL_ADD_RHS (macros.h:392-485): rhs = f(state) +
     * weight * rhs, per cell */
    void FillAddRhs(MultiFab &rhs, const MultiFab &state, double time, int lev, double dt,
                    double dx, double weight) override {
        std::vector<double> old, f;
        gather(rhs, old);
        MultiFab tmp(rhs.boxArray(), amrex::DistributionMapping{}, rhs.nComp(), rhs.nGrow());
        FillRhs(tmp, state, time, lev, dt, dx);
        gather(tmp, f);
        for (size_t q = 0; q < f.size(); ++q) f[q] += weight * old[q];
        scatter(f, rhs);
    }
};

template <class I>
struct Runner : I {
    using I::I;
    void integrate(sledgehamr::LevelData &o, sledgehamr::LevelData &n, double dt, double dx) {
        this->Integrate(o, n, 0, dt, dx);
    }
};

} // namespace

/* nsteps steps of a periodic N^3 level (canonical arrays in and out) with
 * integrator.type `integrator` (11, 10, 21 or 22) of the reference. */
extern "C" int ref_int_evolve(int project, int integrator, int N, int nghost, int ncomp,
                              int with_gw, const double *state_in, double *state_out, double t0,
                              double dt, double dx, int nsteps, const double *params,
                              int nparams, const double *gw_params, int ngw) {
    try {
        Sim sim;
        PeriodicSync sync;
        sim.project = project;
        sim.nghost = nghost;
        sim.with_gravitational_waves = with_gw != 0;
        sim.level_synchronizer = &sync;
        sim.params.assign(params, params + nparams);
        sim.params.push_back(0.);
        sim.gw_params.assign(gw_params, gw_params + ngw);
        sim.gw_params.push_back(0.);
        amrex::BoxArray ba;
        ba.box.hi = amrex::Dim3{N - 1, N - 1, N - 1};
        sledgehamr::LevelData a(ba, amrex::DistributionMapping{}, ncomp, nghost, t0);
        sledgehamr::LevelData b(ba, amrex::DistributionMapping{}, ncomp, nghost, -DBL_MAX);
        scatter(std::vector<double>(state_in, state_in + (size_t)ncomp * N * N * N), a);
        sledgehamr::LevelData *nw = &a, *od = &b;
        auto step = [&](auto &integ) {
            for (int s = 0; s < nsteps; ++s) {
                std::swap(nw, od);                 /* grid_old <-> grid_new */
                od->FillBoundaryPeriodic();        /* FillPatch(lev, t_old) */
                integ.integrate(*od, *nw, dt, dx);
                nw->t = od->t + dt;
                nw->istep = od->istep + 1;
            }
        };
        if (integrator == sledgehamr::Rkn4 || integrator == sledgehamr::Rkn5) {
            Runner<sledgehamr::IntegratorRkn> r(&sim, (sledgehamr::IntegratorType)integrator);
            step(r);
        } else if (integrator == sledgehamr::Lsssprk3) {
            Runner<sledgehamr::IntegratorLsssprk3> r(&sim);
            step(r);
        } else if (integrator == sledgehamr::Leapfrog) {
            Runner<sledgehamr::IntegratorLeapfrog> r(&sim);
            step(r);
        } else {
            return -1;
        }
        std::vector<double> out;
        gather(*nw, out);
        std::memcpy(state_out, out.data(), out.size() * sizeof(double));
        return 0;
    } catch (const std::exception &) {
        return -3;
    }
}

/* The reference's gw_GetLambda (source/gravitational_waves.h:101-133) for
 * every k-cell of a P^3 R2C grid, 81 per cell in (i, j, l, m) order, with
 * the k-map index_to_k (P values). */
extern "C" int ref_gw_lambda_table(int P, const double *index_to_k, double *out) {
    const int H = P / 2 + 1;
    size_t q = 0;
    for (int c = 0; c < P; ++c)
        for (int b = 0; b < P; ++b)
            for (int a = 0; a < H; ++a) {
                int abc[3] = {a, b, c};
                for (int i = 0; i < 3; ++i)
                    for (int j = 0; j < 3; ++j)
                        for (int l = 0; l < 3; ++l)
                            for (int m = 0; m < 3; ++m)
                                out[q++] = sledgehamr::gw_GetLambda(i, j, l, m, abc, index_to_k);
            }
    return 0;
}
