/* ORACLE (test infrastructure only): oracle/_ref/libshref.so.
 *
 * The reference's own per-cell code, compiled from the sledgehamr sources
 * where they lie (source/utils/sledgehamr_utils.h, source/kernels.h,
 * projects/{AxionStrings,FirstOrderPhaseTransition,MinimalExample,
 * NextToMinimalExample}), wrapped as hook policies and driven by the same
 * drivers as the oracle (capi_body.h).  Its entry points carry the prefix
 * ref_ instead of orc_.  Built by oracle/build_ref.sh.
 */
#include <sledgehamr.h>

#include <AxionStrings/setup.h>
#include <AxionStrings/kernels_rhs.h>
#include <AxionStrings/kernels_tagging.h>
#include <AxionStrings/kernels_energy_densities.h>
#include <FirstOrderPhaseTransition/setup.h>
#include <FirstOrderPhaseTransition/kernels_rhs.h>
#include <FirstOrderPhaseTransition/kernels_tagging.h>
#include <FirstOrderPhaseTransition/kernels_misc.h>
#include <MinimalExample/MinimalExample.h>

#include "oracle_core.h"

namespace refp {
using orc::A4;
using R4 = A4<double>;
using S4 = A4<const double>;

template <class T>
inline amrex::Array4<T> conv(const A4<T> &a) {
    return amrex::Array4<T>(a.p, a.js, a.ks, a.ns, amrex::Dim3{a.b.x, a.b.y, a.b.z}, a.nc);
}

#define REF_TE_CASE(NS, N)                                                     \
    case N:                                                                    \
        return NS::TruncationModifier<N>(conv(s), i, j, k, lev, t, dt, dx, te, p);
#define REF_POLICY(NAME, NS, NSCAL, NFIELD)                                    \
    struct NAME {                                                              \
        static constexpr int NScalars = NSCAL, NFields = NFIELD;               \
        static void rhs(const R4 &r, const S4 &s, int i, int j, int k, int lev, double t, \
                        double dt, double dx, const double *p) {               \
            NS::Rhs(conv(r), conv(s), i, j, k, lev, t, dt, dx, p);             \
        }                                                                      \
        static void gw_rhs(const R4 &r, const S4 &s, int i, int j, int k, int lev, double t, \
                           double dt, double dx, const double *p) {            \
            NS::GravitationalWavesRhs<true>(conv(r), conv(s), i, j, k, lev, t, dt, dx, p); \
        }                                                                      \
        static void gw_backreaction(const R4 &r, const S4 &s, int i, int j, int k, int lev, \
                                    double t, double dt, double dx, const double *ps, \
                                    const double *pg) {                        \
            NS::GravitationalWavesBackreaction<true>(conv(r), conv(s), i, j, k, lev, t, dt, \
                                                     dx, ps, pg);              \
        }                                                                      \
        static bool tag(const S4 &s, int i, int j, int k, int lev, double t, double dt, \
                        double dx, const double *p) {                          \
            return NS::TagCellForRefinement<true>(conv(s), i, j, k, lev, t, dt, dx, p); \
        }                                                                      \
        static double te_modifier(int n, const S4 &s, int i, int j, int k, int lev, double t, \
                                  double dt, double dx, double te, const double *p) { \
            switch (n) {                                                       \
                REF_TE_CASE(NS, 0) REF_TE_CASE(NS, 1) REF_TE_CASE(NS, 2)       \
                REF_TE_CASE(NS, 3) REF_TE_CASE(NS, 4) REF_TE_CASE(NS, 5)       \
                REF_TE_CASE(NS, 6) REF_TE_CASE(NS, 7) REF_TE_CASE(NS, 8)       \
                REF_TE_CASE(NS, 9) REF_TE_CASE(NS, 10) REF_TE_CASE(NS, 11)     \
                REF_TE_CASE(NS, 12) REF_TE_CASE(NS, 13) REF_TE_CASE(NS, 14)    \
                REF_TE_CASE(NS, 15)                                            \
            default: return te;                                                \
            }                                                                  \
        }                                                                      \
        static double ko(int order, const S4 &s, int i, int j, int k, int n, double dx, \
                         double str) {                                         \
            return order == 2                                                  \
                       ? sledgehamr::kernels::KreissOligerDissipation<2>(conv(s), i, j, k, n, \
                                                                         dx, str) \
                       : sledgehamr::kernels::KreissOligerDissipation<3>(conv(s), i, j, k, n, \
                                                                         dx, str); \
        }                                                                      \
    };

REF_POLICY(AxionStrings, ::AxionStrings, 4, 2)
REF_POLICY(MinimalExample, ::MinimalExample, 4, 2)
REF_POLICY(FirstOrderPhaseTransition, ::FirstOrderPhaseTransition, 2, 1)
} // namespace refp

#define ORC_API(name) ref_##name
#define ORC_PROJECTS(X)                                                        \
    X(0, refp::AxionStrings)                                                   \
    X(1, refp::MinimalExample)                                                 \
    X(3, refp::FirstOrderPhaseTransition)
#include "capi_body.h"

/* The reference's own AverageDownWithTruncationError on one coarse cell,
 * for comparison with the oracle's restatement. */
extern "C" int ref_avgdown_te_kernel(int ncomp, int Nc, const double *fine, double *crse,
                                     double *te) {
    const int Nf = 2 * Nc;
    amrex::Array4<const double> f(fine, Nf, (long long)Nf * Nf, (long long)Nf * Nf * Nf,
                                  amrex::Dim3{0, 0, 0}, ncomp);
    amrex::Array4<double> c(crse, Nc, (long long)Nc * Nc, (long long)Nc * Nc * Nc,
                            amrex::Dim3{0, 0, 0}, ncomp);
    amrex::Array4<double> t(te, Nf, (long long)Nf * Nf, (long long)Nf * Nf * Nf,
                            amrex::Dim3{0, 0, 0}, ncomp);
    for (int k = 0; k < Nc; ++k)
        for (int j = 0; j < Nc; ++j)
            for (int i = 0; i < Nc; ++i)
                sledgehamr::kernels::AverageDownWithTruncationError(i, j, k, ncomp, c, f, t);
    return 0;
}

/* The reference's Laplacian<order> and Gradient<order> on a periodic N^3
 * component with `ghost` wrap (one component, canonical layout). */
extern "C" int ref_stencil(int kind, int order, int N, const double *field, double dx,
                           double *out) {
    const int g = 3, M = N + 2 * g;
    std::vector<double> pad((size_t)M * M * M);
    for (int k = 0; k < M; ++k)
        for (int j = 0; j < M; ++j)
            for (int i = 0; i < M; ++i) {
                int si = (i - g + N) % N, sj = (j - g + N) % N, sk = (k - g + N) % N;
                pad[((size_t)k * M + j) * M + i] = field[((size_t)sk * N + sj) * N + si];
            }
    amrex::Array4<const double> a(pad.data(), M, (long long)M * M, (long long)M * M * M,
                                  amrex::Dim3{-g, -g, -g}, 1);
    for (int k = 0; k < N; ++k)
        for (int j = 0; j < N; ++j)
            for (int i = 0; i < N; ++i) {
                double v = 0;
                const char ax = "xyz"[kind % 3];
                if (kind < 3) {
                    if (order == 1) v = sledgehamr::utils::Gradient<1>(a, i, j, k, 0, dx, ax);
                    if (order == 2) v = sledgehamr::utils::Gradient<2>(a, i, j, k, 0, dx, ax);
                    if (order == 3) v = sledgehamr::utils::Gradient<3>(a, i, j, k, 0, dx, ax);
                } else {
                    if (order == 1) v = sledgehamr::utils::Laplacian<1>(a, i, j, k, 0, dx * dx);
                    if (order == 2) v = sledgehamr::utils::Laplacian<2>(a, i, j, k, 0, dx * dx);
                    if (order == 3) v = sledgehamr::utils::Laplacian<3>(a, i, j, k, 0, dx * dx);
                }
                out[((size_t)k * N + j) * N + i] = v;
            }
    return 0;
}

/* The reference's AddBubble (projects/FirstOrderPhaseTransition/
 * kernels_misc.h:27-52) over every cell of a periodic N^3 canonical array,
 * bubbles inner, as AddBubbleValues (FirstOrderPhaseTransition.cpp:459-483).
 * Components: Scalar::Phi and Scalar::dPhi of the project. */
extern "C" int ref_add_bubbles(int N, int ncomp, double *state, int nb, const double *xyz,
                               const double *profile, int nbins, double inv_dx, double Lcut,
                               double dx) {
    using FirstOrderPhaseTransition::Bubble;
    std::vector<Bubble> bubbles(nb);
    for (int b = 0; b < nb; ++b) {
        Bubble &B = bubbles[b];
        B.x = xyz[3 * b];
        B.y = xyz[3 * b + 1];
        B.z = xyz[3 * b + 2];
        B.t = 0.;
        B.profile.assign(2, std::vector<double>(nbins));
        for (int r = 0; r < 2; ++r)
            for (int q = 0; q < nbins; ++q) B.profile[r][q] = profile[(size_t)r * nbins + q];
        B.inv_dx = inv_dx;
        B.L = Lcut;
        B.finest_level = 0;
        B.p_bubble = &B;
    }
    const long long n3 = (long long)N * N * N;
    amrex::Array4<double> fab(state, N, (long long)N * N, n3, amrex::Dim3{0, 0, 0}, ncomp);
    const double L = N * dx;
    for (int k = 0; k < N; ++k)
        for (int j = 0; j < N; ++j)
            for (int i = 0; i < N; ++i)
                for (int b = 0; b < nb; ++b)
                    FirstOrderPhaseTransition::AddBubble(i, j, k, dx, L, fab, bubbles[b]);
    return 0;
}

/* The reference's per-cell output functions on every cell of a canonical
 * state: fn 1 with comp 1 = FirstOrderPhaseTransition dPhi2
 * (kernels_misc.h:10-18), 2 = AxionStrings a_prime2, 3 = a_prime_screened,
 * 4 = r_prime2 (kernels_energy_densities.h). */
extern "C" int ref_out_function(const double *state, int N, int ncomp, int fn, double *out) {
    const long long n3 = (long long)N * N * N;
    amrex::Array4<double const> a(state, N, (long long)N * N, n3, amrex::Dim3{0, 0, 0}, ncomp);
    std::vector<double> params;
    for (int k = 0; k < N; ++k)
        for (int j = 0; j < N; ++j)
            for (int i = 0; i < N; ++i) {
                double v = 0;
                if (fn == 1) v = FirstOrderPhaseTransition::dPhi2(a, i, j, k, 0, 0., 0., 0., params);
                else if (fn == 2) v = AxionStrings::a_prime2(a, i, j, k, 0, 0., 0., 0., params);
                else if (fn == 3) v = AxionStrings::a_prime_screened(a, i, j, k, 0, 0., 0., 0., params);
                else if (fn == 4) v = AxionStrings::r_prime2(a, i, j, k, 0, 0., 0., 0., params);
                else return -1;
                out[((long long)k * N + j) * N + i] = v;
            }
    return 0;
}
