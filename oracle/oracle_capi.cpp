/* ORACLE (test infrastructure only): liboracle.so, the CPU restatement of the
 * reference's per-cell hooks (oracle_projects.h) behind the shared drivers
 * and extern "C" entry points of capi_body.h.
 *
 * Project ids: 0 AxionStrings, 1 MinimalExample, 2 NextToMinimalExample,
 * 3 FirstOrderPhaseTransition, 4/5/6 AxionStringsLap1/2/3.
 */
#include "oracle_projects.h"

#define ORC_API(name) orc_##name
#define ORC_PROJECTS(X)                                                        \
    X(0, orc::AxionStrings)                                                    \
    X(1, orc::MinimalExample)                                                  \
    X(2, orc::NextToMinimalExample)                                            \
    X(3, orc::FirstOrderPhaseTransition)                                       \
    X(4, orc::AxionStringsLap<1>)                                              \
    X(5, orc::AxionStringsLap<2>)                                              \
    X(6, orc::AxionStringsLap<3>)
#include "capi_body.h"

/* Laplacian (kind 3) or Gradient along x/y/z (kind 0/1/2) of order 1..3 on a
 * periodic N^3 component (canonical layout), restated stencils. */
extern "C" int orc_stencil(int kind, int order, int N, const double *field, double dx,
                           double *out) {
    using namespace orc;
    if (N <= 0 || order < 1 || order > 3 || kind < 0 || kind > 3) return -1;
    const int g = 3, M = N + 2 * g;
    std::vector<double> pad((size_t)M * M * M);
    for (int k = 0; k < M; ++k)
        for (int j = 0; j < M; ++j)
            for (int i = 0; i < M; ++i) {
                int si = (i - g + N) % N, sj = (j - g + N) % N, sk = (k - g + N) % N;
                pad[((size_t)k * M + j) * M + i] = field[((size_t)sk * N + sj) * N + si];
            }
    S4 a;
    a.p = pad.data(); a.js = M; a.ks = (long long)M * M; a.ns = (long long)M * M * M;
    a.b = IV{-g, -g, -g}; a.nc = 1;
    for (int k = 0; k < N; ++k)
        for (int j = 0; j < N; ++j)
            for (int i = 0; i < N; ++i) {
                double v = 0;
                if (kind < 3) {
                    if (order == 1) v = grad<1>(a, i, j, k, 0, dx, kind);
                    if (order == 2) v = grad<2>(a, i, j, k, 0, dx, kind);
                    if (order == 3) v = grad<3>(a, i, j, k, 0, dx, kind);
                } else {
                    if (order == 1) v = lap<1>(a, i, j, k, 0, dx * dx);
                    if (order == 2) v = lap<2>(a, i, j, k, 0, dx * dx);
                    if (order == 3) v = lap<3>(a, i, j, k, 0, dx * dx);
                }
                out[((size_t)k * N + j) * N + i] = v;
            }
    return 0;
}

/* Bubble injection of FirstOrderPhaseTransition on a periodic N^3 level in
 * the canonical layout (ncomp components): every cell (i, j, k) at
 * position (i dx, j dx, k dx) takes, for every bubble b in order, the
 * profile value at its periodic distance D from the bubble centre,
 * linearly interpolated in bins of width 1/inv_dx, added to component
 * comp_phi (profile row 0) and comp_dphi (row 1); cells with D >= Lcut are
 * left alone.  Restates projects/FirstOrderPhaseTransition/
 * kernels_misc.h:21-52 (Distance, AddBubble), bubbles.h:8-19 (GetPos,
 * GetVal) and FirstOrderPhaseTransition.cpp:459-483 (AddBubbleValues: cells
 * outer, bubbles inner). */
extern "C" int orc_add_bubbles(int N, int ncomp, double *state, int comp_phi, int comp_dphi,
                               int nb, const double *xyz, const double *profile, int nbins,
                               double inv_dx, double Lcut, double dx) {
    if (N <= 0 || nb < 0 || nbins < 2 || comp_phi < 0 || comp_phi >= ncomp || comp_dphi < 0 ||
        comp_dphi >= ncomp)
        return -1;
    if ((long long)(Lcut * inv_dx) + 2 > nbins) return -1;
    const double L = N * dx;
    auto distance = [&](double a, double b) {
        const double d = std::fabs(a - b);
        return d < L / 2. ? d : L - d;
    };
    const size_t n3 = (size_t)N * N * N;
    for (int k = 0; k < N; ++k)
        for (int j = 0; j < N; ++j)
            for (int i = 0; i < N; ++i) {
                const size_t c = ((size_t)k * N + j) * N + i;
                for (int b = 0; b < nb; ++b) {
                    const double Dx = distance(i * dx, xyz[3 * b + 0]);
                    const double Dy = distance(j * dx, xyz[3 * b + 1]);
                    const double Dz = distance(k * dx, xyz[3 * b + 2]);
                    const double D = std::sqrt(Dx * Dx + Dy * Dy + Dz * Dz);
                    if (D >= Lcut) continue;
                    const double pos = D * inv_dx;
                    const int ind = (int)pos;
                    const double frac = pos - (double)ind;
                    for (int r = 0; r < 2; ++r) {
                        const double *p = profile + (size_t)r * nbins;
                        const double val = p[ind] * (1. - frac) + p[ind + 1] * frac;
                        state[(size_t)(r == 0 ? comp_phi : comp_dphi) * n3 + c] += val;
                    }
                }
            }
    return 0;
}

/* Spectrum::Compute on a periodic N^3 canonical state (orc::scalar_spectrum). */
extern "C" int orc_scalar_spectrum(const double *state, int N, int ncomp, int fn, int comp,
                                   double L, double t, double *bins_out, long long *ks_out,
                                   int max_bins, int *nbins) {
    if (N <= 0 || fn < 0 || fn > 4 || (fn <= 1 && (comp < 0 || comp >= ncomp)) ||
        (fn >= 2 && ncomp < 4))
        return -1;
    std::vector<long long> ks;
    std::vector<double> s = orc::scalar_spectrum(state, N, ncomp, fn, comp, L, t, ks);
    *nbins = (int)s.size();
    if ((int)s.size() > max_bins) return -1;
    std::copy(s.begin(), s.end(), bins_out);
    if (ks_out) std::copy(ks.begin(), ks.end(), ks_out);
    return 0;
}

/* The per-cell output function on every cell of a canonical state. */
extern "C" int orc_out_function(const double *state, int N, int ncomp, int fn, int comp,
                                double *out) {
    if (N <= 0 || fn < 0 || fn > 4) return -1;
    const long long n3 = (long long)N * N * N;
    for (long long q = 0; q < n3; ++q) out[q] = orc::out_function(fn, comp, state + q, n3);
    (void)ncomp;
    return 0;
}
