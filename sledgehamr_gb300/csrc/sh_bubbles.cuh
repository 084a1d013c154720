/* Bubble injection of FirstOrderPhaseTransition (device side): the profile
 * values of a list of bubbles added to the field and its momentum at one
 * cell, in bubble order, with separately rounded products and sums so that
 * the result equals a CPU evaluation bit for bit.
 * Reference: projects/FirstOrderPhaseTransition/kernels_misc.h:21-52
 * (Distance, AddBubble), bubbles.h:8-19 (GetPos, GetVal),
 * FirstOrderPhaseTransition.cpp:459-483 (AddBubbleValues). */
#ifndef SH_BUBBLES_CUH_
#define SH_BUBBLES_CUH_

#include <cuda_runtime.h>

namespace sh {

/* Bubbles of one injection: centres xyz[3 b + d], one profile of nbins bins
 * of width 1/inv_dx for the field (row 0) and its momentum (row 1), cut off
 * at distance Lcut. */
struct BubbleList {
    const double *xyz;
    const double *profile;
    int nb, nbins;
    double inv_dx, Lcut;
};

__device__ __forceinline__ double bubble_distance(double a, double b, double L) {
    const double d = fabs(__dadd_rn(a, -b));
    return d < L / 2. ? d : __dadd_rn(L, -d);
}

/* phi += sum_b P0(D_b), dphi += sum_b P1(D_b), sequentially in b, for the
 * cell (i, j, k) of a periodic cube of side L and spacing dx. */
__device__ __forceinline__ void add_bubbles_at(const BubbleList &bl, int i, int j, int k,
                                               double dx, double L, double &phi,
                                               double &dphi) {
    const double x = __dmul_rn((double)i, dx), y = __dmul_rn((double)j, dx),
                 z = __dmul_rn((double)k, dx);
    for (int b = 0; b < bl.nb; ++b) {
        const double Dx = bubble_distance(x, bl.xyz[3 * b + 0], L);
        const double Dy = bubble_distance(y, bl.xyz[3 * b + 1], L);
        const double Dz = bubble_distance(z, bl.xyz[3 * b + 2], L);
        const double D =
            sqrt(__dadd_rn(__dadd_rn(__dmul_rn(Dx, Dx), __dmul_rn(Dy, Dy)), __dmul_rn(Dz, Dz)));
        if (D >= bl.Lcut) continue;
        const double pos = __dmul_rn(D, bl.inv_dx);
        const int ind = (int)pos;
        if (ind + 1 >= bl.nbins) continue; /* excluded by the host's size check */
        const double frac = __dadd_rn(pos, -(double)ind);
        const double w0 = __dadd_rn(1., -frac);
        const double *p0 = bl.profile, *p1 = bl.profile + bl.nbins;
        phi = __dadd_rn(phi, __dadd_rn(__dmul_rn(p0[ind], w0), __dmul_rn(p0[ind + 1], frac)));
        dphi = __dadd_rn(dphi, __dadd_rn(__dmul_rn(p1[ind], w0), __dmul_rn(p1[ind + 1], frac)));
    }
}

} // namespace sh

#endif
