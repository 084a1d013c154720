/* Plaquette winding test of the axion-string projects.
 * A cell is pierced by a string when, walking the four edges of one of the
 * three plaquettes that have the cell as their lower corner (xy, xz, yz),
 * the signed Psi2 zero crossings do not cancel: an edge a -> b whose
 * endpoints have Psi2 of opposite sign contributes the sign of
 * Psi2(a) Psi1(b) - Psi1(a) Psi2(b).
 * Reference: projects/AxionStrings/kernels_tagging.h:16-108.
 *
 * The products of the sign test are rounded separately (no fused
 * multiply-add), so that the result depends only on the field values and
 * matches a CPU evaluation bit for bit.
 */
#ifndef SH_PROJECTS_STRING_WINDING_H_
#define SH_PROJECTS_STRING_WINDING_H_

#include <sh_amrex.h>

namespace sh_strings {

AMREX_GPU_HOST_DEVICE AMREX_FORCE_INLINE double mul_rn(double a, double b) {
#if defined(__CUDA_ARCH__)
    return __dmul_rn(a, b);
#else
    return a * b;
#endif
}

/* Signed crossing of the edge a -> b (0 if Psi2 keeps its sign). */
AMREX_GPU_HOST_DEVICE AMREX_FORCE_INLINE int EdgeCrossing(double a1, double a2, double b1,
                                                          double b2) {
    if (mul_rn(a2, b2) >= 0) return 0;
    const double cross = mul_rn(a2, b1) - mul_rn(a1, b2);
    return cross > 0 ? 1 : -1;
}

/* Winding around the plaquette spanned by unit steps p and q at (i,j,k). */
template <int C1, int C2>
AMREX_GPU_HOST_DEVICE AMREX_FORCE_INLINE int
PlaquetteWinding(const amrex::Array4<const double> &s, int i, int j, int k, int pi, int pj,
                 int pk, int qi, int qj, int qk) {
    const double c1[4] = {s(i, j, k, C1), s(i + pi, j + pj, k + pk, C1),
                          s(i + pi + qi, j + pj + qj, k + pk + qk, C1),
                          s(i + qi, j + qj, k + qk, C1)};
    const double c2[4] = {s(i, j, k, C2), s(i + pi, j + pj, k + pk, C2),
                          s(i + pi + qi, j + pj + qj, k + pk + qk, C2),
                          s(i + qi, j + qj, k + qk, C2)};
    int w = 0;
#pragma unroll
    for (int e = 0; e < 4; ++e) w += EdgeCrossing(c1[e], c2[e], c1[(e + 1) & 3], c2[(e + 1) & 3]);
    return w;
}

/* True if any of the xy, xz, yz plaquettes at (i,j,k) is pierced. */
template <int C1, int C2>
AMREX_GPU_HOST_DEVICE AMREX_FORCE_INLINE bool Pierced(const amrex::Array4<const double> &s,
                                                      int i, int j, int k) {
    if (PlaquetteWinding<C1, C2>(s, i, j, k, 1, 0, 0, 0, 1, 0) != 0) return true;
    if (PlaquetteWinding<C1, C2>(s, i, j, k, 1, 0, 0, 0, 0, 1) != 0) return true;
    if (PlaquetteWinding<C1, C2>(s, i, j, k, 0, 1, 0, 0, 0, 1) != 0) return true;
    return false;
}

} // namespace sh_strings

/* Inside a project namespace with fields Psi1, Psi2, Pi1, Pi2: the string
 * tagging criterion and the dt scaling of momentum truncation errors
 * (projects/AxionStrings/kernels_tagging.h:97-131). */
#define SH_AXION_TE_TIMES_DT(c)                                                \
    template <>                                                                \
    AMREX_GPU_HOST_DEVICE AMREX_FORCE_INLINE double TruncationModifier<c>(     \
        const amrex::Array4<const double> &state, const int i, const int j,    \
        const int k, const int lev, const double time, const double dt,        \
        const double dx, const double truncation_error, const double *params) { \
        return truncation_error * dt;                                          \
    }
#define SH_AXION_STRING_TAGGING                                                \
    template <>                                                                \
    AMREX_GPU_HOST_DEVICE AMREX_FORCE_INLINE bool TagCellForRefinement<true>(  \
        const amrex::Array4<const double> &state, const int i, const int j,    \
        const int k, const int lev, const double time, const double dt,        \
        const double dx, const double *params) {                               \
        return sh_strings::Pierced<Scalar::Psi1, Scalar::Psi2>(state, i, j, k); \
    }                                                                          \
    SH_AXION_TE_TIMES_DT(Scalar::Pi1)                                          \
    SH_AXION_TE_TIMES_DT(Scalar::Pi2)                                          \
    SH_AXION_TE_TIMES_DT(Gw::du_xx)                                            \
    SH_AXION_TE_TIMES_DT(Gw::du_yy)                                            \
    SH_AXION_TE_TIMES_DT(Gw::du_zz)                                            \
    SH_AXION_TE_TIMES_DT(Gw::du_xy)                                            \
    SH_AXION_TE_TIMES_DT(Gw::du_xz)                                            \
    SH_AXION_TE_TIMES_DT(Gw::du_yz)

#endif
