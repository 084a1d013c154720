/* The sledgehamr project plugin surface, re-implemented without Boost or
 * AMReX so that project kernel headers written for sledgehamr compile
 * unchanged (with nvcc for sm_103a and with g++) against this library.
 *
 * A project declares its fields with
 *     SLEDGEHAMR_ADD_SCALARS(Psi1, Psi2)
 *     SLEDGEHAMR_ADD_CONJUGATE_MOMENTA(Pi1, Pi2)
 * which creates, inside the project namespace,
 *   - Scalar::<name> component indices (fields first, then momenta) and
 *     Scalar::NScalars,
 *   - the Gw enum of the 12 gravitational-wave tensor components that follow
 *     the user fields (u_xx, u_yy, u_zz, u_xy, u_xz, u_yz, du_xx ... du_yz),
 *   - default (no-op) hook templates TruncationModifier<n>,
 *     TagCellForRefinement<bool>, GravitationalWavesRhs<bool> and
 *     GravitationalWavesBackreaction<bool> that the project may specialise.
 * The project then writes its per-cell Rhs(...) and specialisations and ends
 * with SLEDGEHAMR_FINISH_SETUP, which here collects the hooks into the
 * struct ShHooks that the GPU kernels are instantiated with
 * (SH_INSTANTIATE_PROJECT in sledgehamr_gb300/csrc/).
 *
 * Reference interface: source/macros.h:39-181 (field and hook macros),
 * :247-249 (SLEDGEHAMR_FINISH_SETUP), :690-697 (SLEDGEHAMR_INITIALIZE_PROJECT);
 * source/scalars.h:10-44 (ScalarField); source/sledgehamr.h:248-337 (host
 * hooks of the project class).
 */
#ifndef SLEDGEHAMR_SHIM_SLEDGEHAMR_H_
#define SLEDGEHAMR_SHIM_SLEDGEHAMR_H_

#include <string>
#include <vector>

#include "kernels.h"
#include "sh_amrex.h"
#include "sledgehamr_utils.h"

/* ---- variadic for-each (up to 16 names) --------------------------------- */
#define SH_PP_CAT(a, b) SH_PP_CAT_I(a, b)
#define SH_PP_CAT_I(a, b) a##b
#define SH_PP_NARG(...)                                                        \
    SH_PP_NARG_I(__VA_ARGS__, 16, 15, 14, 13, 12, 11, 10, 9, 8, 7, 6, 5, 4, 3, \
                 2, 1, 0)
#define SH_PP_NARG_I(_1, _2, _3, _4, _5, _6, _7, _8, _9, _10, _11, _12, _13,  \
                     _14, _15, _16, N, ...)                                    \
    N
#define SH_PP_FOR_EACH(M, ...)                                                 \
    SH_PP_CAT(SH_PP_FE_, SH_PP_NARG(__VA_ARGS__))(M, __VA_ARGS__)
#define SH_PP_FE_1(M, a) M(a)
#define SH_PP_FE_2(M, a, ...) M(a) SH_PP_FE_1(M, __VA_ARGS__)
#define SH_PP_FE_3(M, a, ...) M(a) SH_PP_FE_2(M, __VA_ARGS__)
#define SH_PP_FE_4(M, a, ...) M(a) SH_PP_FE_3(M, __VA_ARGS__)
#define SH_PP_FE_5(M, a, ...) M(a) SH_PP_FE_4(M, __VA_ARGS__)
#define SH_PP_FE_6(M, a, ...) M(a) SH_PP_FE_5(M, __VA_ARGS__)
#define SH_PP_FE_7(M, a, ...) M(a) SH_PP_FE_6(M, __VA_ARGS__)
#define SH_PP_FE_8(M, a, ...) M(a) SH_PP_FE_7(M, __VA_ARGS__)
#define SH_PP_FE_9(M, a, ...) M(a) SH_PP_FE_8(M, __VA_ARGS__)
#define SH_PP_FE_10(M, a, ...) M(a) SH_PP_FE_9(M, __VA_ARGS__)
#define SH_PP_FE_11(M, a, ...) M(a) SH_PP_FE_10(M, __VA_ARGS__)
#define SH_PP_FE_12(M, a, ...) M(a) SH_PP_FE_11(M, __VA_ARGS__)
#define SH_PP_FE_13(M, a, ...) M(a) SH_PP_FE_12(M, __VA_ARGS__)
#define SH_PP_FE_14(M, a, ...) M(a) SH_PP_FE_13(M, __VA_ARGS__)
#define SH_PP_FE_15(M, a, ...) M(a) SH_PP_FE_14(M, __VA_ARGS__)
#define SH_PP_FE_16(M, a, ...) M(a) SH_PP_FE_15(M, __VA_ARGS__)

namespace sledgehamr {

/* A named field component; registers itself in the project's field list and
 * takes its position there as component id. */
class ScalarField {
  public:
    ScalarField(std::string str, std::vector<ScalarField *> &sfv,
                bool is_momentum)
        : name(std::move(str)), id(static_cast<int>(sfv.size())),
          is_conjugate_momentum(is_momentum) {
        sfv.push_back(this);
    }
    operator int() const { return id; }
    std::string name;
    const int id;
    bool is_conjugate_momentum;
};

/* Host-side hooks of a project class.  The time stepper of this library
 * asks them for the parameter vectors that are handed to the device hooks,
 * exactly where sledgehamr's framework does. */
class Sledgehamr {
  public:
    virtual ~Sledgehamr() = default;
    virtual void Init() {}
    virtual void SetParamsRhs(std::vector<double> &params, const double time,
                              const int lev) {}
    virtual void SetParamsGravitationalWaveRhs(std::vector<double> &params,
                                               const double time,
                                               const int lev) {}
    virtual void SetParamsTagCellForRefinement(std::vector<double> &params,
                                               const double time,
                                               const int lev) {}
    virtual void SetParamsTruncationModifier(std::vector<double> &params,
                                             const double time,
                                             const int lev) {}
    virtual void BeforeTimestep(const double time) {}
    virtual bool CreateLevelIf(const int lev, const double time) {
        return true;
    }
    virtual bool StopRunning(const double time) { return false; }

    std::vector<ScalarField *> scalar_fields;
};

} // namespace sledgehamr

/* ---- field declaration macros ------------------------------------------ */
#define SH_SCALAR_ENUM_ENTRY(f) f,
#define SH_ADD_ONE_SCALAR(f)                                                   \
    static sledgehamr::ScalarField SH_PP_CAT(_s_, f) = {#f, l_scalar_fields,   \
                                                        false};                \
    namespace Scalar {                                                         \
    constexpr int f = _Scalar::f;                                              \
    }
#define SH_ADD_ONE_MOMENTUM(f)                                                 \
    static sledgehamr::ScalarField SH_PP_CAT(_s_, f) = {#f, l_scalar_fields,   \
                                                        true};                 \
    namespace Scalar {                                                         \
    constexpr int f = _Momentum::f + _Scalar::NScalarFields;                   \
    }

#define SLEDGEHAMR_ADD_SCALARS(...)                                            \
    enum _Scalar { SH_PP_FOR_EACH(SH_SCALAR_ENUM_ENTRY, __VA_ARGS__)           \
                       NScalarFields };                                        \
    static std::vector<sledgehamr::ScalarField *> l_scalar_fields;             \
    SH_PP_FOR_EACH(SH_ADD_ONE_SCALAR, __VA_ARGS__)

#define SLEDGEHAMR_GW_ENUM                                                     \
    enum Gw {                                                                  \
        u_xx = Scalar::NScalars,                                               \
        u_yy,                                                                  \
        u_zz,                                                                  \
        u_xy,                                                                  \
        u_xz,                                                                  \
        u_yz,                                                                  \
        du_xx,                                                                 \
        du_yy,                                                                 \
        du_zz,                                                                 \
        du_xy,                                                                 \
        du_xz,                                                                 \
        du_yz,                                                                 \
        NGwScalars                                                             \
    };

#define SLEDGEHAMR_DEFAULT_HOOKS                                               \
    template <int>                                                             \
    AMREX_GPU_HOST_DEVICE AMREX_FORCE_INLINE double TruncationModifier(        \
        const amrex::Array4<const double> &state, const int i, const int j,    \
        const int k, const int lev, const double time, const double dt,        \
        const double dx, const double truncation_error,                        \
        const double *params) {                                                \
        return truncation_error;                                               \
    }                                                                          \
    template <bool>                                                            \
    AMREX_GPU_HOST_DEVICE AMREX_FORCE_INLINE bool TagCellForRefinement(        \
        const amrex::Array4<const double> &state, const int i, const int j,    \
        const int k, const int lev, const double time, const double dt,        \
        const double dx, const double *params) {                               \
        return false;                                                          \
    }                                                                          \
    template <bool>                                                            \
    AMREX_GPU_HOST_DEVICE AMREX_FORCE_INLINE void GravitationalWavesRhs(       \
        const amrex::Array4<double> &rhs,                                      \
        const amrex::Array4<const double> &state, const int i, const int j,    \
        const int k, const int lev, const double time, const double dt,        \
        const double dx, const double *params) {}                              \
    template <bool>                                                            \
    AMREX_GPU_HOST_DEVICE AMREX_FORCE_INLINE void                              \
    GravitationalWavesBackreaction(                                            \
        const amrex::Array4<double> &rhs,                                      \
        const amrex::Array4<const double> &state, const int i, const int j,    \
        const int k, const int lev, const double time, const double dt,        \
        const double dx, const double *params_scalars,                         \
        const double *params_gw) {}

#define SLEDGEHAMR_ADD_CONJUGATE_MOMENTA(...)                                  \
    enum _Momentum { SH_PP_FOR_EACH(SH_SCALAR_ENUM_ENTRY, __VA_ARGS__)         \
                         NMomentumFields };                                    \
    SH_PP_FOR_EACH(SH_ADD_ONE_MOMENTUM, __VA_ARGS__)                           \
    namespace Scalar {                                                         \
    constexpr int NScalars =                                                   \
        _Scalar::NScalarFields + _Momentum::NMomentumFields;                   \
    }                                                                          \
    SLEDGEHAMR_GW_ENUM                                                         \
    SLEDGEHAMR_DEFAULT_HOOKS

/* Collects the project's device hooks (free functions and specialisations
 * found by unqualified lookup inside the project namespace) into one type. */
#define SLEDGEHAMR_FINISH_SETUP                                                \
    struct ShHooks {                                                           \
        static constexpr int kNScalars = Scalar::NScalars;                     \
        static constexpr int kNFields = _Scalar::NScalarFields;                \
        static constexpr int kNMomenta = _Momentum::NMomentumFields;           \
        static std::vector<sledgehamr::ScalarField *> &fields() {              \
            return l_scalar_fields;                                            \
        }                                                                      \
        AMREX_GPU_DEVICE AMREX_FORCE_INLINE static void                        \
        rhs(const amrex::Array4<double> &r,                                    \
            const amrex::Array4<const double> &s, int i, int j, int k,         \
            int lev, double t, double dt, double dx, const double *p) {        \
            Rhs(r, s, i, j, k, lev, t, dt, dx, p);                             \
        }                                                                      \
        AMREX_GPU_DEVICE AMREX_FORCE_INLINE static void                        \
        gw_rhs(const amrex::Array4<double> &r,                                 \
               const amrex::Array4<const double> &s, int i, int j, int k,      \
               int lev, double t, double dt, double dx, const double *p) {     \
            GravitationalWavesRhs<true>(r, s, i, j, k, lev, t, dt, dx, p);     \
        }                                                                      \
        AMREX_GPU_DEVICE AMREX_FORCE_INLINE static void                        \
        gw_backreaction(const amrex::Array4<double> &r,                        \
                        const amrex::Array4<const double> &s, int i, int j,    \
                        int k, int lev, double t, double dt, double dx,        \
                        const double *ps, const double *pg) {                  \
            GravitationalWavesBackreaction<true>(r, s, i, j, k, lev, t, dt,    \
                                                 dx, ps, pg);                  \
        }                                                                      \
        AMREX_GPU_HOST_DEVICE AMREX_FORCE_INLINE static bool                   \
        tag(const amrex::Array4<const double> &s, int i, int j, int k,         \
            int lev, double t, double dt, double dx, const double *p) {        \
            return TagCellForRefinement<true>(s, i, j, k, lev, t, dt, dx, p);  \
        }                                                                      \
        template <int N>                                                       \
        AMREX_GPU_HOST_DEVICE AMREX_FORCE_INLINE static double                 \
        te_modifier(const amrex::Array4<const double> &s, int i, int j, int k, \
                    int lev, double t, double dt, double dx, double te,        \
                    const double *p) {                                         \
            return TruncationModifier<N>(s, i, j, k, lev, t, dt, dx, te, p);   \
        }                                                                      \
    };

/* Inside a project class deriving from sledgehamr::Sledgehamr. */
#define SLEDGEHAMR_INITIALIZE_PROJECT(prj)                                     \
    prj() { scalar_fields = l_scalar_fields; }

#endif // SLEDGEHAMR_SHIM_SLEDGEHAMR_H_
