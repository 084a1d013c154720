/* RKN4 stage kernels of FP32 levels (the precision form on levels and AMR
 * hierarchies) for the axion-string projects of this library
 * (AxionStringsLap1 / AxionStringsLap2):
 *   Psi' = Pi,
 *   Pi'  = -2 Pi / eta + lap_N(Psi) - lambda Psi [eta^2 (|Psi|^2 - 1) + c]
 * with lambda = params[0], c = params[1], written against the equations in
 * FP32 (the plugin hooks compute in FP64, which runs at 1/64 of the FP32
 * rate on GB300).
 *
 * Same schedule as the FP64 stage kernel (sh_stage.cuh) with the RKN4
 * tableau of source/integrators/rkn.cpp:130-139 (c = {0, 1/2, 1},
 * a_21 = 1/8, a_32 = 1/2, a_31 = 0, bbar = {1/6, 1/3, 0},
 * b = {1/6, 2/3, 1/6}; every stage uses the step's initial momenta,
 * rkn.cpp:55-117):
 *   STAGE 0: K0 = accel(y0);  Y1 = y0 + h/2 y0' + h^2/8 K0
 *   STAGE 1: K1 = accel(Y1);  Y2 = y0 + h y0' + h^2/2 K1
 *   STAGE 2: K2 = accel(Y2);  y1 = y0 + h y0' + h^2 (K0/6 + K1/3),
 *                             y1' = y0' + h ((K0 + K2)/6 + 2 K1/3)
 * The stage buffers hold the positions Y_i only (every stage reads the
 * momenta y0' of the step's initial state), and only their two position
 * components get ghost cells at the stage times.  The last stage adds the
 * increments with Kahan compensation (the value y and its compensation c
 * stand for y - c; the compensations of the new state are written beside
 * it).
 *
 * The arithmetic is the explicitly rounded FP32 of the ensemble kernels
 * (sh_f32.cuh): Laplacian, potential, acceleration, stage positions and
 * increments round exactly as there.
 */
#ifndef SH_STAGE32_CUH_
#define SH_STAGE32_CUH_

#include "sh_f32.cuh"
#include "sh_internal.h"

namespace sh {

struct Stage32Args {
    const TileDev *tiles;
    const BoxDev *boxes;
    const float *state; /* Y_i, positions with filled ghost cells (stage 0: y0) */
    const float *y0;    /* the step's initial state (positions and momenta) */
    float *out;         /* stages 0, 1: Y_{i+1} (positions); stage 2: y1 */
    const float *k0, *k1; /* K buffers, two components each (box layout) */
    float *kout;
    const float *c_old;   /* compensations of y0 */
    float *c_new;         /* compensations of y1 */
    float h, cm, ck;      /* dt; stage position coefficients of y0' and K */
    float h2;             /* dt^2 */
    float inv;            /* 1/dx^2 (7 points) or 1/(12 dx^2) (13 points) */
    float lam, cst;       /* params[0], params[1] */
    float friction, eta2; /* -2/eta and eta^2 at the stage time */
};

/* Each thread walks its z-column keeping the 2 ORDER + 1 values of the two
 * position components along z in registers (one new plane value per step
 * instead of 2 ORDER + 1 loads), with restrict-qualified pointers (every
 * buffer of a stage is distinct) so that the next plane's loads can be
 * issued ahead of the current plane's stores.  The sums are formed in the
 * order of the ensemble kernels (x+, x-, y+, y-, z+, z-). */
template <int ORDER, int STAGE>
__global__ void __launch_bounds__(kThreads) stage32_axion_kernel(const __grid_constant__ Stage32Args a) {
    constexpr int R = ORDER; /* stencil reach */
    const TileDev t = a.tiles[blockIdx.x];
    const BoxDev b = a.boxes[t.box];
    const int tid = threadIdx.x + kTileX * threadIdx.y;
    const int ty = tid / t.nx;
    const int i = t.x0 + (tid - ty * t.nx);
    const int j = t.y0 + ty;
    if (ty >= kThreads / t.nx || i > b.hi[0] || j > b.hi[1]) return;
    const int kend = min(t.z0 + t.nz - 1, b.hi[2]);
    const long long gx = b.gdim[0], gxy = gx * b.gdim[1], gvol = b.gvol;
    const float *__restrict__ st = a.state;
    const float *__restrict__ y0 = a.y0;
    const float *__restrict__ k0 = a.k0;
    const float *__restrict__ k1 = a.k1;
    const float *__restrict__ c_old = a.c_old;
    float *__restrict__ out = a.out;
    float *__restrict__ kout = a.kout;
    float *__restrict__ c_new = a.c_new;
    const long long col =
        b.off * 4 + (i - b.glo[0]) + (long long)(j - b.glo[1]) * gx; /* component 0, z = glo */
    const long long kcol = b.off * 2 + (i - b.glo[0]) + (long long)(j - b.glo[1]) * gx;
    /* z-window of the two positions: w[c][d] = value at plane k - R + d */
    float w[2][2 * R + 1];
#pragma unroll
    for (int c = 0; c < 2; ++c)
#pragma unroll
        for (int d = 0; d < 2 * R; ++d)
            w[c][d] = st[col + c * gvol + (long long)(t.z0 - R + d - b.glo[2]) * gxy];
    for (int k = t.z0; k <= kend; ++k) {
        const long long lz = (long long)(k - b.glo[2]) * gxy;
        const long long sb = col + lz;  /* component 0 of the cell */
        const long long kb = kcol + lz; /* K component 0 of the cell */
        /* the next cell's y0 (and, in the last stage, K and compensations)
         * asked into L1 while this cell is computed */
        if (k < kend) {
#pragma unroll
            for (int c = 0; c < 4; ++c)
                asm volatile("prefetch.global.L1 [%0];" ::"l"(y0 + sb + gxy + c * gvol));
            if constexpr (STAGE == 2) {
#pragma unroll
                for (int c = 0; c < 2; ++c) {
                    asm volatile("prefetch.global.L1 [%0];" ::"l"(k0 + kb + gxy + c * gvol));
                    asm volatile("prefetch.global.L1 [%0];" ::"l"(k1 + kb + gxy + c * gvol));
                }
#pragma unroll
                for (int c = 0; c < 4; ++c)
                    asm volatile("prefetch.global.L1 [%0];" ::"l"(c_old + sb + gxy + c * gvol));
            }
        }
        float lap[2];
#pragma unroll
        for (int c = 0; c < 2; ++c) {
            const float *s = st + sb + c * gvol;
            w[c][2 * R] = s[R * gxy];
            if constexpr (ORDER == 1) {
                lap[c] = f32::lap7(w[c][1], s[1], s[-1], s[gx], s[-gx], w[c][2], w[c][0], a.inv);
            } else {
                const float s1 = f32::ring(s[1], s[-1], s[gx], s[-gx], w[c][3], w[c][1]);
                const float s2 = f32::ring(s[2], s[-2], s[2 * gx], s[-2 * gx], w[c][4], w[c][0]);
                lap[c] = f32::lap13(w[c][2], s1, s2, a.inv);
            }
        }
        const float p0 = w[0][R], p1 = w[1][R];
        const float q0 = y0[sb + 2 * gvol], q1 = y0[sb + 3 * gvol];
        const float v = f32::potential(p0, p1, a.lam, a.eta2, a.cst);
        const float kq[2] = {f32::accel(q0, lap[0], p0, v, a.friction),
                             f32::accel(q1, lap[1], p1, v, a.friction)};
        const float q[2] = {q0, q1};
        if constexpr (STAGE < 2) {
#pragma unroll
            for (int c = 0; c < 2; ++c) {
                kout[kb + c * gvol] = kq[c];
                const float y = y0[sb + c * gvol];
                out[sb + c * gvol] = f32::stage_pos(y, q[c], kq[c], a.cm, a.ck);
            }
        } else {
#pragma unroll
            for (int c = 0; c < 2; ++c) {
                const float ka = k0[kb + c * gvol], kbv = k1[kb + c * gvol];
                float y = y0[sb + c * gvol], cy = c_old[sb + c * gvol];
                float m = q[c], cmo = c_old[sb + (2 + c) * gvol];
                f32::kahan(y, f32::dpos(q[c], ka, kbv, a.h, a.h2), cy);
                f32::kahan(m, f32::dmom(ka, kbv, kq[c], a.h), cmo);
                out[sb + c * gvol] = y;
                out[sb + (2 + c) * gvol] = m;
                c_new[sb + c * gvol] = cy;
                c_new[sb + (2 + c) * gvol] = cmo;
            }
        }
#pragma unroll
        for (int c = 0; c < 2; ++c)
#pragma unroll
            for (int d = 0; d < 2 * R; ++d) w[c][d] = w[c][d + 1];
    }
}

/* Kick-drift-kick leapfrog stages of FP32 levels of FirstOrderPhaseTransition
 * with the pure potential (params[0] = 0), with or without the GW tensor:
 *   Phi'' = lap Phi + q2 Phi + q3 Phi^2 + q4 Phi^3,
 *   u_ij'' = lap u_ij + d_i Phi d_j Phi
 * (4th-order Laplacian and gradient; projects/FirstOrderPhaseTransition/
 * kernels_rhs.h:20-109), the schedule of source/integrators/leapfrog.cpp:13-57
 * (both kicks with the acceleration of the positions they see):
 *   STAGE 0: a = f(x0);  vh = v0 + dt/2 a;  x1 = x0 + dt vh
 *   STAGE 1: a = f(x1);  v1 = vh + dt/2 a
 * with Kahan-compensated updates: vh and its compensation go to the K
 * buffer, x1 and v1 with theirs to the new state.  The arithmetic is that of
 * the FP32 ensemble kernel of the same equations (sh_fast.cu). */
struct Stage32FoptArgs {
    const TileDev *tiles;
    const BoxDev *boxes;
    const float *state; /* positions read by the stencils (stage 0: x0, 1: x1) */
    const float *y0;    /* the step's initial state */
    const float *c_old; /* its compensations */
    float *out;         /* the new state */
    float *c_new;       /* its compensations */
    float *kv, *kc;     /* vh and its compensation (np components each) */
    float inv12dx2, inv12dx, hdt, dt, q2, q3, q4;
};

template <int STAGE, bool GW>
__global__ void __launch_bounds__(kThreads)
    stage32_fopt_kernel(const __grid_constant__ Stage32FoptArgs a) {
    constexpr int NP = GW ? 7 : 1, NC = 2 * NP;
    const TileDev t = a.tiles[blockIdx.x];
    const BoxDev b = a.boxes[t.box];
    const int tid = threadIdx.x + kTileX * threadIdx.y;
    const int ty = tid / t.nx;
    const int i = t.x0 + (tid - ty * t.nx);
    const int j = t.y0 + ty;
    if (ty >= kThreads / t.nx || i > b.hi[0] || j > b.hi[1]) return;
    const int kend = min(t.z0 + t.nz - 1, b.hi[2]);
    const long long gx = b.gdim[0], gxy = gx * b.gdim[1], gvol = b.gvol;
    /* position q: Phi, u_xx, u_yy, u_zz, u_xy, u_xz, u_yz; momentum: dPhi,
     * du_xx, ... (the level's component order) */
    auto pos = [](int q) { return q == 0 ? 0 : 1 + q; };
    auto mom = [](int q) { return q == 0 ? 1 : NP + q; };
    for (int k = t.z0; k <= kend; ++k) {
        const long long lc =
            (i - b.glo[0]) + (long long)(j - b.glo[1]) * gx + (long long)(k - b.glo[2]) * gxy;
        const long long sb = b.off * NC + lc;
        const long long kb = b.off * NP + lc;
        float acc[NP];
#pragma unroll
        for (int q = 0; q < NP; ++q) {
            const float *s = a.state + sb + pos(q) * gvol;
            float s1 = s[1] + s[-1];
            s1 += s[gx] + s[-gx];
            s1 += s[gxy] + s[-gxy];
            float s2 = s[2] + s[-2];
            s2 += s[2 * gx] + s[-2 * gx];
            s2 += s[2 * gxy] + s[-2 * gxy];
            acc[q] = (16.f * s1 - s2 - 90.f * s[0]) * a.inv12dx2;
        }
        const float *ph = a.state + sb;
        const float phi = ph[0];
        acc[0] += phi * (a.q2 + phi * (a.q3 + phi * a.q4));
        if constexpr (GW) {
            float g[3];
            g[0] = (8.f * (ph[1] - ph[-1]) - (ph[2] - ph[-2])) * a.inv12dx;
            g[1] = (8.f * (ph[gx] - ph[-gx]) - (ph[2 * gx] - ph[-2 * gx])) * a.inv12dx;
            g[2] = (8.f * (ph[gxy] - ph[-gxy]) - (ph[2 * gxy] - ph[-2 * gxy])) * a.inv12dx;
            acc[1] += g[0] * g[0];
            acc[2] += g[1] * g[1];
            acc[3] += g[2] * g[2];
            acc[4] += g[0] * g[1];
            acc[5] += g[0] * g[2];
            acc[6] += g[1] * g[2];
        }
#pragma unroll
        for (int q = 0; q < NP; ++q) {
            if constexpr (STAGE == 0) {
                float v = a.y0[sb + mom(q) * gvol], cv = a.c_old[sb + mom(q) * gvol];
                f32::kahan(v, a.hdt * acc[q], cv);
                a.kv[kb + q * gvol] = v;
                a.kc[kb + q * gvol] = cv;
                float x = a.y0[sb + pos(q) * gvol], cx = a.c_old[sb + pos(q) * gvol];
                f32::kahan(x, a.dt * v, cx);
                a.out[sb + pos(q) * gvol] = x;
                a.c_new[sb + pos(q) * gvol] = cx;
            } else {
                float v = a.kv[kb + q * gvol], cv = a.kc[kb + q * gvol];
                f32::kahan(v, a.hdt * acc[q], cv);
                a.out[sb + mom(q) * gvol] = v;
                a.c_new[sb + mom(q) * gvol] = cv;
            }
        }
    }
}

} // namespace sh

#endif
