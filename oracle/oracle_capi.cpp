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
