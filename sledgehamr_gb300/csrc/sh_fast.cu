/* Batched periodic levels ("ensembles") with fused, shared-memory-tiled
 * stage kernels in FP32 with Kahan-compensated updates, or in FP64.
 *
 * These are the chosen precision and batching forms of the hot path for the
 * two physics families of the configured workloads, written against the
 * equations directly rather than through the double-typed plugin hooks:
 *
 *   axion strings (AxionStringsLap1/2, NextToMinimalExample form):
 *     Psi' = Pi,  Pi' = -2 Pi/eta + lap_N(Psi) - lambda Psi [eta^2 (|Psi|^2-1) + c]
 *     integrated with RKN4 (source/integrators/rkn.cpp:25-120, tableau
 *     :130-139; every stage uses the step's initial momenta).
 *   first-order phase transition + GW tensor (FirstOrderPhaseTransition):
 *     Phi'' = lap Phi + q2 Phi + q3 Phi^2 + q4 Phi^3,
 *     u_ij'' = lap u_ij + d_i Phi d_j Phi  (4th-order Laplacian and gradient)
 *     integrated with the kick-drift-kick leapfrog (leapfrog.cpp:13-57).
 *
 * Layout: every realisation r of an ensemble is one periodic cube of N_r^3
 * cells with no ghost cells (neighbours are wrapped in the kernel); each
 * component is one array with all realisations concatenated.  A thread
 * block owns a 32 x 8 column tile of one realisation and marches in z,
 * keeping the (2R+1) planes the stencil needs in a shared-memory ring; the
 * stage positions Y_i = y0 + c h y0' + h^2 sum a K_j are rebuilt while a
 * plane is loaded (so each stage reads y0, y0' and the earlier K once,
 * halos coming from L2), and the last stage writes the new state with
 * compensated summation: t = y + (d - c); c = (t - y) - (d - c); y = t.
 * Algorithmic HBM traffic per cell-update (4 components, RKN4): 26 words
 * plus 8 compensation words; (14 components, leapfrog): 49 words plus 42.
 */
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "sh_bubbles.cuh"
#include "sh_f32.cuh"
#include "sh_fixed_stencil.h"
#include "sh_internal.h"
#include "sledgehamr_gb300.h"

namespace sh {
namespace fast {

constexpr int TX = 32, TY = 8;

struct RealDesc {
    long long off; /* first cell of the realisation in every array */
    int N;
    int active;    /* 0: a released slot of a pool (no tiles) */
    double dx;     /* grid spacing */
    double dt;     /* own step of a pool member (leapfrog; 0: the step's dt) */
    double p[4];   /* physics parameters (lambda, c) or (q2, q3, q4, -) */
};

struct FastTile {
    int r;
    int x0, y0, z0, nz;
};

template <class R>
struct AxionArgs {
    const RealDesc *desc;
    const FastTile *tiles;
    const R *y0[2], *m0[2]; /* state in */
    R *y1[2], *m1[2];       /* state out */
    R *cy[2], *cm[2];       /* compensations (in place) */
    R *K[2][2];             /* K_0, K_1 (two components each) */
    double *time;           /* two slots; the step reads slot `slot` and the */
    int slot;               /* last stage writes slot 1 - slot = t + h */
    double h;
};

__device__ __forceinline__ int wrap(int a, int N) { return a < 0 ? a + N : (a >= N ? a - N : a); }


template <class R>
__device__ __forceinline__ void kahan_add(R &y, R d, R &c) {
    if constexpr (sizeof(R) == 4) {
        f32::kahan(y, d, c);
    } else {
        const R v = d - c;
        const R t = y + v;
        c = (t - y) - v;
        y = t;
    }
}

/* RKN4 stage kernel for the axion family.  ORDER: Laplacian order (1: 7
 * points, 2: 13 points).  STAGE 0 and 1 write K_STAGE; STAGE 2 writes the
 * new state.
 *
 * Software pipeline: the loads of the next plane (y0, y0', K) are issued
 * into registers before the current plane is computed and are combined
 * into the stage positions and stored into the ring at the start of the
 * next iteration; the centre values the epilogue needs are issued before
 * the barrier.  The ring has one slot more than the stencil reads, so one
 * barrier per plane suffices (a thread storing plane z+1 overwrites plane
 * z-2H-1, which no thread still reads once all passed the barrier of z).
 * The per-block constants (stage time, friction, couplings, 1/dx^2) are
 * formed once in FP64 by one thread: FP64 work per thread would run on
 * GB300's narrow FP64 pipe. */
template <class R, int ORDER, int STAGE, bool KAHAN>
__global__ void __launch_bounds__(TX *TY, sizeof(R) == 4 ? 5 : 1) axion_rkn4_kernel(const __grid_constant__ AxionArgs<R> a) {
    constexpr int H = ORDER;             /* halo */
    constexpr int RING = 2 * H + 2;
    constexpr int W = TX + 2 * H, HH = TY + 2 * H;
    constexpr int NT = TX * TY;
    constexpr int NPL = (W * HH + NT - 1) / NT; /* plane elements per thread */
    __shared__ R ring[RING][2][HH][W];
    __shared__ R kc[10];

    const FastTile tl = a.tiles[blockIdx.x];
    const RealDesc d = a.desc[tl.r];
    const int N = d.N;
    const long long off = d.off;
    const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * TX + tx;
    const int x = tl.x0 + tx, y = tl.y0 + ty;
    const bool active = x < N && y < N;

    /* RKN4 tableau (rkn.cpp:130-139): c = {0, 1/2, 1}; a21 = 1/8; a32 = 1/2;
     * bbar = {1/6, 1/3, 0}; b = {1/6, 2/3, 1/6}. */
    if (tid == 0) {
        const double hh = a.h * a.h;
        const double t0 = a.time[a.slot];
        const double ts = t0 + a.h * (STAGE == 0 ? 0. : (STAGE == 1 ? 0.5 : 1.));
        if (STAGE == 2 && blockIdx.x == 0) a.time[1 - a.slot] = t0 + a.h;
        kc[0] = (R)(STAGE == 0 ? 0. : (STAGE == 1 ? 0.5 * a.h : a.h)); /* cm */
        kc[1] = (R)(STAGE == 1 ? hh / 8. : (STAGE == 2 ? hh / 2. : 0.)); /* ck */
        kc[2] = (R)(-2. / ts);                                            /* friction */
        kc[3] = (R)d.p[0];                                                /* lambda */
        kc[4] = (R)d.p[1];                                                /* c */
        kc[5] = (R)(ts * ts);                                             /* eta^2 */
        const R inv_dx2 = (R)(1. / (d.dx * d.dx));
        kc[6] = inv_dx2;
        kc[7] = inv_dx2 / (R)12;
        kc[8] = (R)a.h;
        kc[9] = (R)hh;
    }
    __syncthreads();
    const R cm = kc[0], ck = kc[1], friction = kc[2], lam = kc[3], cst = kc[4], eta2 = kc[5];
    const R inv_dx2 = kc[6], inv12dx2 = kc[7];
    const R* Kin = STAGE == 1 ? a.K[0][0] : (STAGE == 2 ? a.K[1][0] : nullptr);
    const R* Kin2 = STAGE == 1 ? a.K[0][1] : (STAGE == 2 ? a.K[1][1] : nullptr);

    /* plane element q of this thread: ring position and periodic source */
    int ppos[NPL], pgx[NPL], pgy[NPL];
#pragma unroll
    for (int q = 0; q < NPL; ++q) {
        const int p = tid + q * NT;
        ppos[q] = p < W * HH ? p : -1;
        const int px = p % W, py = p / W;
        pgx[q] = wrap(tl.x0 - H + px, N);
        pgy[q] = wrap(tl.y0 - H + py, N);
    }
    R raw[NPL][6]; /* y0 (2), y0' (2), K (2) of the next plane */
    auto fetch = [&](int z) {
        const int zw = wrap(z, N);
#pragma unroll
        for (int q = 0; q < NPL; ++q) {
            if (ppos[q] < 0) continue;
            const long long e = off + ((long long)zw * N + pgy[q]) * N + pgx[q];
            raw[q][0] = a.y0[0][e];
            raw[q][1] = a.y0[1][e];
            if (STAGE > 0) {
                raw[q][2] = a.m0[0][e];
                raw[q][3] = a.m0[1][e];
                raw[q][4] = Kin[e];
                raw[q][5] = Kin2[e];
            }
        }
    };
    auto commit = [&](int slot) {
#pragma unroll
        for (int q = 0; q < NPL; ++q) {
            if (ppos[q] < 0) continue;
            R v0 = raw[q][0], v1 = raw[q][1];
            if (STAGE > 0) {
                if constexpr (sizeof(R) == 4) {
                    v0 = f32::stage_pos(v0, raw[q][2], raw[q][4], cm, ck);
                    v1 = f32::stage_pos(v1, raw[q][3], raw[q][5], cm, ck);
                } else {
                    v0 += cm * raw[q][2] + ck * raw[q][4];
                    v1 += cm * raw[q][3] + ck * raw[q][5];
                }
            }
            const int px = ppos[q] % W, py = ppos[q] / W;
            ring[slot][0][py][px] = v0;
            ring[slot][1][py][px] = v1;
        }
    };

    const int zb = tl.z0 - H, ze = tl.z0 + tl.nz + H; /* planes [zb, ze) */
    fetch(zb);
    for (int z = zb; z < ze; ++z) {
        const int zc = z - H;
        const bool out = zc >= tl.z0 && active;
        const long long e = off + ((long long)zc * N + y) * N + x;
        /* centre values of the plane computed below */
        R q0 = 0, q1 = 0, ka0 = 0, ka1 = 0, kb0 = 0, kb1 = 0, y0c = 0, y1c = 0;
        R c0 = 0, c1 = 0, c2 = 0, c3 = 0;
        if (out) {
            q0 = a.m0[0][e];
            q1 = a.m0[1][e];
            if (STAGE == 2) {
                ka0 = a.K[0][0][e];
                ka1 = a.K[0][1][e];
                kb0 = a.K[1][0][e];
                kb1 = a.K[1][1][e];
                y0c = a.y0[0][e];
                y1c = a.y0[1][e];
                if (KAHAN) {
                    c0 = a.cy[0][e];
                    c1 = a.cy[1][e];
                    c2 = a.cm[0][e];
                    c3 = a.cm[1][e];
                }
            }
        }
        commit((z - zb) % RING);
        if (z + 1 < ze) fetch(z + 1);
        __syncthreads();
        if (out) {
            const int sc = (zc - zb) % RING;
            R lap[2];
#pragma unroll
            for (int c = 0; c < 2; ++c) {
                const R u0 = ring[sc][c][ty + H][tx + H];
                if constexpr (sizeof(R) == 8) {
                    /* FP64 members: the ring sums exactly in 64-bit integers
                     * (sh_fixed_stencil.h), as the drop-in path's stencils */
                    namespace fx = sledgehamr::utils::fixed;
                    const double r1[7] = {
                        u0, ring[sc][c][ty + H][tx + H + 1], ring[sc][c][ty + H][tx + H - 1],
                        ring[sc][c][ty + H + 1][tx + H], ring[sc][c][ty + H - 1][tx + H],
                        ring[(sc + 1) % RING][c][ty + H][tx + H],
                        ring[(sc + RING - 1) % RING][c][ty + H][tx + H]};
                    if (ORDER == 1) {
                        const int n[2] = {1, 6};
                        const long long w[2] = {-6, 1};
                        lap[c] = fx::weighted_sum<7, 2, -6>(r1, n, w, inv_dx2);
                    } else {
                        const double r2[13] = {
                            r1[0], r1[1], r1[2], r1[3], r1[4], r1[5], r1[6],
                            ring[sc][c][ty + H][tx + H + 2], ring[sc][c][ty + H][tx + H - 2],
                            ring[sc][c][ty + H + 2][tx + H], ring[sc][c][ty + H - 2][tx + H],
                            ring[(sc + 2) % RING][c][ty + H][tx + H],
                            ring[(sc + RING - 2) % RING][c][ty + H][tx + H]};
                        const int n[3] = {1, 6, 6};
                        const long long w[3] = {-90, 16, -1};
                        lap[c] = fx::weighted_sum<13, 3, -2>(r2, n, w, inv12dx2);
                    }
                } else if (ORDER == 1) {
                    lap[c] = f32::lap7(
                        u0, ring[sc][c][ty + H][tx + H + 1], ring[sc][c][ty + H][tx + H - 1],
                        ring[sc][c][ty + H + 1][tx + H], ring[sc][c][ty + H - 1][tx + H],
                        ring[(sc + 1) % RING][c][ty + H][tx + H],
                        ring[(sc + RING - 1) % RING][c][ty + H][tx + H], inv_dx2);
                } else {
                    const R s1 = f32::ring(
                        ring[sc][c][ty + H][tx + H + 1], ring[sc][c][ty + H][tx + H - 1],
                        ring[sc][c][ty + H + 1][tx + H], ring[sc][c][ty + H - 1][tx + H],
                        ring[(sc + 1) % RING][c][ty + H][tx + H],
                        ring[(sc + RING - 1) % RING][c][ty + H][tx + H]);
                    const R s2 = f32::ring(
                        ring[sc][c][ty + H][tx + H + 2], ring[sc][c][ty + H][tx + H - 2],
                        ring[sc][c][ty + H + 2][tx + H], ring[sc][c][ty + H - 2][tx + H],
                        ring[(sc + 2) % RING][c][ty + H][tx + H],
                        ring[(sc + RING - 2) % RING][c][ty + H][tx + H]);
                    lap[c] = f32::lap13(u0, s1, s2, inv12dx2);
                }
            }
            const R p0 = ring[sc][0][ty + H][tx + H], p1 = ring[sc][1][ty + H][tx + H];
            R k0, k1;
            if constexpr (sizeof(R) == 4) {
                const float v = f32::potential(p0, p1, lam, eta2, cst);
                k0 = f32::accel(q0, lap[0], p0, v, friction);
                k1 = f32::accel(q1, lap[1], p1, v, friction);
            } else {
                const R v = lam * (eta2 * (p0 * p0 + p1 * p1 - (R)1) + cst);
                k0 = friction * q0 + lap[0] - p0 * v;
                k1 = friction * q1 + lap[1] - p1 * v;
            }
            if (STAGE < 2) {
                a.K[STAGE][0][e] = k0;
                a.K[STAGE][1][e] = k1;
            } else {
                const R h = kc[8], h2 = kc[9];
                /* y1 = y0 + h y0' + h^2 (K0/6 + K1/3); y1' = y0' + h (K0/6 + 2K1/3 + K2/6) */
                R dy0, dy1, dm0, dm1;
                if constexpr (sizeof(R) == 4) {
                    dy0 = f32::dpos(q0, ka0, kb0, h, h2);
                    dy1 = f32::dpos(q1, ka1, kb1, h, h2);
                    dm0 = f32::dmom(ka0, kb0, k0, h);
                    dm1 = f32::dmom(ka1, kb1, k1, h);
                } else {
                    dy0 = h * q0 + h2 * (ka0 * (R)(1. / 6.) + kb0 * (R)(1. / 3.));
                    dy1 = h * q1 + h2 * (ka1 * (R)(1. / 6.) + kb1 * (R)(1. / 3.));
                    dm0 = h * ((ka0 + k0) * (R)(1. / 6.) + kb0 * (R)(2. / 3.));
                    dm1 = h * ((ka1 + k1) * (R)(1. / 6.) + kb1 * (R)(2. / 3.));
                }
                R y0v = y0c, y1v = y1c, m0v = q0, m1v = q1;
                if (KAHAN) {
                    kahan_add(y0v, dy0, c0);
                    kahan_add(y1v, dy1, c1);
                    kahan_add(m0v, dm0, c2);
                    kahan_add(m1v, dm1, c3);
                    a.cy[0][e] = c0;
                    a.cy[1][e] = c1;
                    a.cm[0][e] = c2;
                    a.cm[1][e] = c3;
                } else {
                    y0v += dy0;
                    y1v += dy1;
                    m0v += dm0;
                    m1v += dm1;
                }
                a.y1[0][e] = y0v;
                a.y1[1][e] = y1v;
                a.m1[0][e] = m0v;
                a.m1[1][e] = m1v;
            }
        }
    }
}

template <class R>
struct FoptArgs {
    const RealDesc *desc;
    const FastTile *tiles;
    const R *x[7];   /* positions read by the stencil (Phi, u_xx..u_yz) */
    const R *v[7];   /* momenta in (S0: v0, S1: vh) */
    R *xo[7];        /* S0: x1 */
    R *vo[7];        /* S0: vh, S1: v1 */
    R *cx[7], *cv[7];
    double *time; /* two slots, as for AxionArgs; STAGE 1 writes slot 1 - slot */
    int slot;
    double dt;
};

/* Leapfrog kick-drift-kick stage kernel for Phi + GW tensor (7 position and
 * 7 momentum components; 4th-order Laplacian and gradient, halo 2).
 * STAGE 0: a = f(x0); vh = v0 + dt/2 a; x1 = x0 + dt vh.
 * STAGE 1: a = f(x1); v1 = vh + dt/2 a.
 * Potential: dPhi' = lap Phi + q2 Phi + q3 Phi^2 + q4 Phi^3 (p[0..2]). */
template <class R, int STAGE, bool KAHAN>
__global__ void __launch_bounds__(TX *TY, sizeof(R) == 4 ? 3 : 1) fopt_leapfrog_kernel(const __grid_constant__ FoptArgs<R> a) {
    constexpr int H = 2, RING = 5, W = TX + 2 * H, HH = TY + 2 * H, NC = 7;
    extern __shared__ unsigned char smem_raw[];
    R(*ring)[NC][HH][W] = reinterpret_cast<R(*)[NC][HH][W]>(smem_raw);

    const FastTile tl = a.tiles[blockIdx.x];
    const RealDesc d = a.desc[tl.r];
    const int N = d.N;
    const long long off = d.off;
    const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * TX + tx;
    const int x = tl.x0 + tx, y = tl.y0 + ty;
    const bool active = x < N && y < N;
    __shared__ R kc[7];
    if (tid == 0) {
        const double sdt = a.dt > 0. ? a.dt : d.dt; /* pools: every member its own step */
        kc[0] = (R)d.p[0];
        kc[1] = (R)d.p[1];
        kc[2] = (R)d.p[2];
        kc[3] = (R)(1. / (12. * d.dx * d.dx));
        kc[4] = (R)(1. / (12. * d.dx));
        kc[5] = (R)(0.5 * sdt);
        kc[6] = (R)sdt;
        if (STAGE == 1 && blockIdx.x == 0) a.time[1 - a.slot] = a.time[a.slot] + a.dt;
    }
    __syncthreads();
    const R q2 = kc[0], q3 = kc[1], q4 = kc[2], inv12dx2 = kc[3], inv12dx = kc[4];
    const R hdt = kc[5], dt = kc[6];

    /* software pipeline: the next plane's loads are issued into registers
     * before the current plane is computed */
    constexpr int NT = TX * TY;
    constexpr int NPL = (W * HH + NT - 1) / NT;
    int ppos[NPL];
    long long pxy[NPL]; /* in-plane offset of the periodic source cell */
#pragma unroll
    for (int q = 0; q < NPL; ++q) {
        const int p = tid + q * NT;
        ppos[q] = p < W * HH ? p : -1;
        const int gx = wrap(tl.x0 - H + p % W, N), gy = wrap(tl.y0 - H + p / W, N);
        pxy[q] = (long long)gy * N + gx;
    }
    R raw[NPL][NC];
    auto fetch = [&](int z) {
        const long long pz = off + (long long)wrap(z, N) * N * N;
#pragma unroll
        for (int q = 0; q < NPL; ++q) {
            if (ppos[q] < 0) continue;
#pragma unroll
            for (int c = 0; c < NC; ++c) raw[q][c] = a.x[c][pz + pxy[q]];
        }
    };
    auto commit = [&](int slot) {
#pragma unroll
        for (int q = 0; q < NPL; ++q) {
            if (ppos[q] < 0) continue;
            const int px = ppos[q] % W, py = ppos[q] / W;
#pragma unroll
            for (int c = 0; c < NC; ++c) ring[slot][c][py][px] = raw[q][c];
        }
    };
    const int zb = tl.z0 - H, ze = tl.z0 + tl.nz + H;
    fetch(zb);
    for (int z = zb; z < ze; ++z) {
        const int zc = z - H;
        const bool outp = zc >= tl.z0 && active;
        const long long e = off + ((long long)zc * N + y) * N + x;
        /* centre values of the plane computed below */
        R cv_[NC], cc_[NC], cx_c[NC];
#pragma unroll
        for (int c = 0; c < NC; ++c) {
            cv_[c] = outp ? a.v[c][e] : (R)0;
            cc_[c] = (outp && KAHAN) ? a.cv[c][e] : (R)0;
            cx_c[c] = (outp && KAHAN && STAGE == 0) ? a.cx[c][e] : (R)0;
        }
        __syncthreads(); /* the slot about to be written is no longer read */
        commit((z - zb) % RING);
        if (z + 1 < ze) fetch(z + 1);
        __syncthreads();
        if (outp) {
            const int s0 = (zc - zb) % RING;
            const int sp1 = (s0 + 1) % RING, sp2 = (s0 + 2) % RING;
            const int sm1 = (s0 + RING - 1) % RING, sm2 = (s0 + RING - 2) % RING;
            const int cx_ = tx + H, cy_ = ty + H;
            R acc[NC];
#pragma unroll
            for (int c = 0; c < NC; ++c) {
                const R u0 = ring[s0][c][cy_][cx_];
                if constexpr (sizeof(R) == 8) {
                    /* FP64 members: exact integer ring sums (sh_fixed_stencil.h) */
                    const double v[13] = {
                        u0, ring[s0][c][cy_][cx_ + 1], ring[s0][c][cy_][cx_ - 1],
                        ring[s0][c][cy_ + 1][cx_], ring[s0][c][cy_ - 1][cx_],
                        ring[sp1][c][cy_][cx_], ring[sm1][c][cy_][cx_],
                        ring[s0][c][cy_][cx_ + 2], ring[s0][c][cy_][cx_ - 2],
                        ring[s0][c][cy_ + 2][cx_], ring[s0][c][cy_ - 2][cx_],
                        ring[sp2][c][cy_][cx_], ring[sm2][c][cy_][cx_]};
                    const int n[3] = {1, 6, 6};
                    const long long w[3] = {-90, 16, -1};
                    acc[c] = sledgehamr::utils::fixed::weighted_sum<13, 3, -2>(v, n, w, inv12dx2);
                    continue;
                }
                R s1 = ring[s0][c][cy_][cx_ + 1] + ring[s0][c][cy_][cx_ - 1];
                s1 += ring[s0][c][cy_ + 1][cx_] + ring[s0][c][cy_ - 1][cx_];
                s1 += ring[sp1][c][cy_][cx_] + ring[sm1][c][cy_][cx_];
                R s2 = ring[s0][c][cy_][cx_ + 2] + ring[s0][c][cy_][cx_ - 2];
                s2 += ring[s0][c][cy_ + 2][cx_] + ring[s0][c][cy_ - 2][cx_];
                s2 += ring[sp2][c][cy_][cx_] + ring[sm2][c][cy_][cx_];
                acc[c] = ((R)16 * s1 - s2 - (R)90 * u0) * inv12dx2;
            }
            /* 4th-order gradient of Phi */
            R g[3];
            if constexpr (sizeof(R) == 8) {
                /* FP64 members: exact integer sums (sh_fixed_stencil.h) */
                const int n[4] = {1, 1, 1, 1};
                const long long w[4] = {8, -8, -1, 1};
                const double gx[4] = {ring[s0][0][cy_][cx_ + 1], ring[s0][0][cy_][cx_ - 1],
                                      ring[s0][0][cy_][cx_ + 2], ring[s0][0][cy_][cx_ - 2]};
                const double gy[4] = {ring[s0][0][cy_ + 1][cx_], ring[s0][0][cy_ - 1][cx_],
                                      ring[s0][0][cy_ + 2][cx_], ring[s0][0][cy_ - 2][cx_]};
                const double gz[4] = {ring[sp1][0][cy_][cx_], ring[sm1][0][cy_][cx_],
                                      ring[sp2][0][cy_][cx_], ring[sm2][0][cy_][cx_]};
                namespace fx = sledgehamr::utils::fixed;
                g[0] = fx::weighted_sum<4, 4, -5>(gx, n, w, inv12dx);
                g[1] = fx::weighted_sum<4, 4, -5>(gy, n, w, inv12dx);
                g[2] = fx::weighted_sum<4, 4, -5>(gz, n, w, inv12dx);
            } else {
            g[0] = ((R)8 * (ring[s0][0][cy_][cx_ + 1] - ring[s0][0][cy_][cx_ - 1]) -
                    (ring[s0][0][cy_][cx_ + 2] - ring[s0][0][cy_][cx_ - 2])) * inv12dx;
            g[1] = ((R)8 * (ring[s0][0][cy_ + 1][cx_] - ring[s0][0][cy_ - 1][cx_]) -
                    (ring[s0][0][cy_ + 2][cx_] - ring[s0][0][cy_ - 2][cx_])) * inv12dx;
            g[2] = ((R)8 * (ring[sp1][0][cy_][cx_] - ring[sm1][0][cy_][cx_]) -
                    (ring[sp2][0][cy_][cx_] - ring[sm2][0][cy_][cx_])) * inv12dx;
            }
            const R phi = ring[s0][0][cy_][cx_];
            acc[0] += phi * (q2 + phi * (q3 + phi * q4));
            acc[1] += g[0] * g[0];
            acc[2] += g[1] * g[1];
            acc[3] += g[2] * g[2];
            acc[4] += g[0] * g[1];
            acc[5] += g[0] * g[2];
            acc[6] += g[1] * g[2];
#pragma unroll
            for (int c = 0; c < NC; ++c) {
                R vv = cv_[c];
                if (KAHAN) {
                    R cvv = cc_[c];
                    kahan_add(vv, hdt * acc[c], cvv);
                    a.cv[c][e] = cvv;
                } else {
                    vv += hdt * acc[c];
                }
                a.vo[c][e] = vv;
                if (STAGE == 0) {
                    R xx = ring[s0][c][cy_][cx_];
                    if (KAHAN) {
                        R cxx = cx_c[c];
                        kahan_add(xx, dt * vv, cxx);
                        a.cx[c][e] = cxx;
                    } else {
                        xx += dt * vv;
                    }
                    a.xo[c][e] = xx;
                }
            }
        }
    }
}

} // namespace fast
} // namespace sh

#include "sh_fast_tma.cuh"

/* ======================================================================= */
/* Diagnostics: FP64 energy per realisation and string (winding) counts.   */
namespace sh {
namespace fast {

/* Energy density summed per block in FP64; one partial per block, reduced
 * per realisation on the host in block order (deterministic).
 * axion: 1/2 (Pi1^2 + Pi2^2) + 1/2 |grad Psi|^2 + lambda/4 eta^2 (|Psi|^2-1)^2
 *        + lambda c/2 |Psi|^2
 * FOPT : 1/2 dPhi^2 + 1/2 |grad Phi|^2 + V(Phi),
 *        V = -(q2/2 Phi^2 + q3/3 Phi^3 + q4/4 Phi^4);
 * gradients are 2nd-order central differences. */
template <class R>
__global__ void energy_kernel(const RealDesc *desc, const FastTile *tiles, const R *f0,
                              const R *f1, const R *m0, const R *m1, const R *cf0, const R *cf1,
                              const R *cm0, const R *cm1, int family, double eta,
                              double *partial) {
    const FastTile tl = tiles[blockIdx.x];
    const RealDesc d = desc[tl.r];
    const int N = d.N;
    const double dx = d.dx;
    const int x = tl.x0 + threadIdx.x, y = tl.y0 + threadIdx.y;
    double acc = 0.;
    /* the compensation holds minus the lost low part */
    auto val = [&](const R *f, const R *c, long long e) {
        return (double)f[e] - (c ? (double)c[e] : 0.);
    };
    if (x < N && y < N) {
        for (int z = tl.z0; z < tl.z0 + tl.nz; ++z) {
            const long long e = d.off + ((long long)z * N + y) * N + x;
            auto at = [&](const R *f, const R *c, int dx_, int dy_, int dz_) {
                return val(f, c, d.off + ((long long)wrap(z + dz_, N) * N + wrap(y + dy_, N)) * N +
                                     wrap(x + dx_, N));
            };
            double gsum = 0.;
            const int ncf = family == 3 ? 1 : 2;
            for (int q = 0; q < ncf; ++q) {
                const R *f = q == 0 ? f0 : f1;
                const R *c = q == 0 ? cf0 : cf1;
                const double gx = (at(f, c, 1, 0, 0) - at(f, c, -1, 0, 0)) / (2. * dx);
                const double gy = (at(f, c, 0, 1, 0) - at(f, c, 0, -1, 0)) / (2. * dx);
                const double gz = (at(f, c, 0, 0, 1) - at(f, c, 0, 0, -1)) / (2. * dx);
                gsum += gx * gx + gy * gy + gz * gz;
            }
            if (family == 3) {
                const double phi = val(f0, cf0, e), dp = val(m0, cm0, e);
                const double V =
                    -(d.p[0] / 2. * phi * phi + d.p[1] / 3. * phi * phi * phi +
                      d.p[2] / 4. * phi * phi * phi * phi);
                acc += 0.5 * dp * dp + 0.5 * gsum + V;
            } else {
                const double p0 = val(f0, cf0, e), p1 = val(f1, cf1, e);
                const double q0 = val(m0, cm0, e), q1 = val(m1, cm1, e);
                const double r2m1 = p0 * p0 + p1 * p1 - 1.;
                acc += 0.5 * (q0 * q0 + q1 * q1) + 0.5 * gsum +
                       d.p[0] / 4. * eta * eta * r2m1 * r2m1 +
                       d.p[0] * d.p[1] / 2. * (p0 * p0 + p1 * p1);
            }
        }
    }
    acc *= dx * dx * dx;
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    __shared__ double ws[TX * TY / 32];
    if ((threadIdx.x & 31) == 0) ws[(threadIdx.y * TX + threadIdx.x) >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0 && threadIdx.y == 0) {
        double s = 0.;
        for (int w = 0; w < TX * TY / 32; ++w) s += ws[w];
        partial[blockIdx.x] = s;
    }
}

/* Cells pierced by a string (AxionStrings TagCellForRefinement, the count of
 * Cosmology::GetStringTags, projects/AxionStrings/cosmology.cpp:114-142). */
__device__ __forceinline__ int edge_xing(double a1, double a2, double b1, double b2) {
    if (__dmul_rn(a2, b2) >= 0) return 0;
    return (__dmul_rn(a2, b1) - __dmul_rn(a1, b2)) > 0 ? 1 : -1;
}

template <class R>
__global__ void string_count_kernel(const RealDesc *desc, const FastTile *tiles, const R *f0,
                                    const R *f1, const R *c0, const R *c1,
                                    unsigned long long *counts) {
    const FastTile tl = tiles[blockIdx.x];
    const RealDesc d = desc[tl.r];
    const int N = d.N;
    const int x = tl.x0 + threadIdx.x, y = tl.y0 + threadIdx.y;
    unsigned long long n = 0;
    if (x < N && y < N) {
        for (int z = tl.z0; z < tl.z0 + tl.nz; ++z) {
            auto v = [&](const R *f, int dx_, int dy_, int dz_) {
                const long long e =
                    d.off + ((long long)wrap(z + dz_, N) * N + wrap(y + dy_, N)) * N + wrap(x + dx_, N);
                const R *c = f == f0 ? c0 : c1;
                return (double)f[e] - (c ? (double)c[e] : 0.);
            };
            const int P[3][2][3] = {{{1, 0, 0}, {0, 1, 0}}, {{1, 0, 0}, {0, 0, 1}},
                                    {{0, 1, 0}, {0, 0, 1}}};
            bool hit = false;
            for (int pl = 0; pl < 3 && !hit; ++pl) {
                const int *p = P[pl][0], *q = P[pl][1];
                const int cx[4] = {0, p[0], p[0] + q[0], q[0]};
                const int cy[4] = {0, p[1], p[1] + q[1], q[1]};
                const int cz[4] = {0, p[2], p[2] + q[2], q[2]};
                int w = 0;
                for (int e = 0; e < 4; ++e) {
                    const int f = (e + 1) & 3;
                    w += edge_xing(v(f0, cx[e], cy[e], cz[e]), v(f1, cx[e], cy[e], cz[e]),
                                   v(f0, cx[f], cy[f], cz[f]), v(f1, cx[f], cy[f], cz[f]));
                }
                hit = w != 0;
            }
            n += hit;
        }
    }
    for (int o = 16; o > 0; o >>= 1) n += __shfl_down_sync(0xffffffffu, n, o);
    if ((threadIdx.x & 31) == 0 && n) atomicAdd(&counts[tl.r], n);
}

/* Conversion between host FP64 and device storage (value + compensation). */
template <class R>
__global__ void store_kernel(const double *src, R *dst, R *comp, long long n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const double v = src[i];
        const R r = (R)v;
        dst[i] = r;
        if (comp) comp[i] = (R)0;
    }
}
template <class R>
__global__ void load_kernel(const R *src, const R *comp, double *dst, long long n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        /* the compensation holds minus the lost low part */
        dst[i] = (double)src[i] - (comp ? (double)comp[i] : 0.);
    }
}

/* Pack two GW components of realisation r (compensations included) into
 * the real and imaginary parts of a zero-padded complex (pN)^3 FP64 array
 * for the spectrum. */
template <class R>
__global__ void gw_pack_fast_kernel(const R *sa, const R *ca, const R *sb, const R *cb,
                                    long long off, int N, int P, double2 *dst) {
    const long long n = (long long)N * N * N;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const int x = (int)(i % N), y = (int)((i / N) % N), z = (int)(i / ((long long)N * N));
        dst[((long long)z * P + y) * P + x] =
            make_double2((double)sa[off + i] - (ca ? (double)ca[off + i] : 0.),
                         (double)sb[off + i] - (cb ? (double)cb[off + i] : 0.));
    }
}

/* The same into complex FP32 arrays (FP32 transforms); v - c in the
 * storage type, rounded to FP32. */
template <class R>
__global__ void gw_pack_fast32_kernel(const R *sa, const R *ca, const R *sb, const R *cb,
                                      long long off, int N, int P, float2 *dst) {
    const long long n = (long long)N * N * N;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const int x = (int)(i % N), y = (int)((i / N) % N), z = (int)(i / ((long long)N * N));
        const R a = ca ? sa[off + i] - ca[off + i] : sa[off + i];
        const R b = cb ? sb[off + i] - cb[off + i] : sb[off + i];
        dst[((long long)z * P + y) * P + x] = make_float2((float)a, (float)b);
    }
}

/* Bubbles added to Phi (array phi) and dPhi (array dphi) of realisation r;
 * with compensations the sum is formed from the compensated values and the
 * new compensation holds the rounding of the stored result. */
template <class R>
__global__ void add_bubbles_kernel(const RealDesc *desc, int r, R *phi, R *dphi, R *cphi,
                                   R *cdphi, BubbleList bl) {
    const RealDesc d = desc[r];
    const int N = d.N;
    const long long n = (long long)N * N * N;
    const double L = N * d.dx;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
         q += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(q % N), j = (int)((q / N) % N), k = (int)(q / ((long long)N * N));
        const long long e = d.off + q;
        double a = (double)phi[e] - (cphi ? (double)cphi[e] : 0.);
        double b = (double)dphi[e] - (cdphi ? (double)cdphi[e] : 0.);
        add_bubbles_at(bl, i, j, k, d.dx, L, a, b);
        const R ra = (R)a, rb = (R)b;
        phi[e] = ra;
        dphi[e] = rb;
        if (cphi) cphi[e] = (R)((double)ra - a);
        if (cdphi) cdphi[e] = (R)((double)rb - b);
    }
}

} // namespace fast
} // namespace sh

/* ======================================================================= */
/* Host side: ensembles (sh_ensemble_* of include/sledgehamr_gb300.h).      */
#include <functional>
#include <map>
#include <memory>
#include <stdexcept>

#include "sh_gw.h"

namespace {
using namespace sh::fast;

struct FastErr : std::runtime_error {
    int code;
    FastErr(int c, const std::string &m) : std::runtime_error(m), code(c) {}
};
inline void fck(cudaError_t e, const char *what) {
    if (e != cudaSuccess) {
        cudaGetLastError();
        throw FastErr(e == cudaErrorMemoryAllocation ? SH_ERR_NOMEM : SH_ERR_CUDA,
                      std::string(what) + ": " + cudaGetErrorString(e));
    }
}
inline void freq(bool c, const std::string &m) {
    if (!c) throw FastErr(SH_ERR_ARG, m);
}
int fgrid(long long n) {
    return (int)std::max<long long>(1, std::min<long long>((n + 255) / 256, 152LL * 32));
}
constexpr int kTuneCandidates[5] = {4, 8, 16, 32, 64};
} // namespace

struct sh_ensemble {
    sh_ctx *ctx = nullptr;
    int family = 0, precision = 0, nreal = 0, ncomp = 0;
    size_t esize = 4;
    std::vector<RealDesc> desc;
    long long total = 0; /* cells of all realisations */
    RealDesc *d_desc = nullptr;
    std::vector<FastTile> tiles;
    FastTile *d_tiles = nullptr;
    size_t tiles_cap = 0, desc_cap = 0;
    int tile_nz = 16;
    /* pools: capacity in cells of every array and the free extents
     * (offset -> length) */
    bool pool = false;
    long long capacity = 0;
    std::map<long long, long long> free_ext;
    /* component arrays of `total` elements: state A (current) and B, the
     * Kahan compensations C (FP32_KAHAN only) and stage scratch K */
    std::vector<void *> A, B, C, K;
    void *A0 = nullptr; /* A[0] at creation: parity of the A/B buffers */
    double *d_time = nullptr; /* two slots */
    int slot = 0;
    double *d_partial = nullptr;
    size_t partial_cap = 0;
    unsigned long long *d_counts = nullptr;
    size_t counts_cap = 0;
    double *staging = nullptr; /* host transfers and bubble lists; only grows */
    size_t staging_cap = 0;
    sh::GwCache gw;
    void *gw_scratch = nullptr;
    size_t gw_scratch_cap = 0;
    int spectrum_precision = SH_PREC_FP64; /* of the GW transforms and projection */
    std::string err;
    long long launches = 0;
    /* one CUDA graph of a whole step per buffer parity, for step size graph_dt */
    bool use_graph = false;
    cudaGraphExec_t graph[2] = {nullptr, nullptr};
    double graph_dt[2] = {0., 0.};
    /* stencil-plane staging of the axion stage kernels in FP32: 0 planes
     * loaded through registers (axion_rkn4_kernel), 1 tensor copies into
     * shared memory (axion_rkn4_tma_kernel) with their tiles and maps */
    int plane_staging = 0;
    std::vector<sh::fast::tma::TmaTile> ttiles;
    sh::fast::tma::TmaTile *d_ttiles = nullptr;
    size_t ttiles_cap = 0;
    CUtensorMap *d_maps = nullptr;
    size_t maps_cap = 0;
    int tma_slab = 0; /* largest shared-memory slab of the tiles (floats) */
    int *d_err = nullptr; /* SH_ERR_TIMEOUT from a kernel whose wait ran out */
};

namespace {

cudaStream_t est(const sh_ensemble *E) { return (cudaStream_t)sh_ctx_stream(E->ctx); }

void drop_graphs(sh_ensemble *E) {
    for (int p = 0; p < 2; ++p)
        if (E->graph[p]) {
            cudaGraphExecDestroy(E->graph[p]);
            E->graph[p] = nullptr;
        }
}

/* Device copy of a host table in a buffer that only grows, written in
 * stream order (kernels queued earlier still read the old contents). */
template <class T>
void upload_table(const std::vector<T> &h, T *&d, size_t &cap, cudaStream_t s, const char *what) {
    if (h.size() > cap) {
        if (d) {
            fck(cudaStreamSynchronize(s), what);
            cudaFree(d);
            d = nullptr;
            cap = 0;
        }
        const size_t n = std::max<size_t>(h.size(), 2 * cap + 64);
        fck(cudaMalloc(&d, n * sizeof(T)), what);
        cap = n;
    }
    if (!h.empty())
        fck(cudaMemcpyAsync(d, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice, s), what);
}

/* Rows per tile of the tensor-copy kernels for a realisation of N cells
 * per side and stencil reach H: the largest of 16, 8, 4, 2 that divides N,
 * covers the reach, keeps a plane of the tile at most kMaxCells cells and
 * its shared-memory slab (rows with halo times the padded pitch) at most
 * 1024 floats; 0 when none does (or N is not a multiple of 4, which the
 * 16-byte row strides of a tensor map need, or wider than a copy box). */
int tma_rows(int N, int H) {
    namespace T = sh::fast::tma;
    if (N % 4 != 0 || N > 256 || N < 2 * H + 1) return 0;
    for (int t : {16, 8, 4, 2})
        if (N % t == 0 && t >= H && N * t <= T::kMaxCells && (t + 2 * H) * T::pitch_of(N) <= 1024)
            return t;
    return 0;
}

int family_reach(const sh_ensemble *E) { return E->family == SH_FAMILY_AXION_LAP2 ? 2 : 1; }

/* Whether the tensor-copy kernels can run this ensemble: axion family in
 * FP32 storage, every member of a size tma_rows accepts, every member's
 * arrays 16-byte aligned. */
bool tma_possible(const sh_ensemble *E) {
    if (E->family == SH_FAMILY_FOPT_GW || E->esize != 4) return false;
    for (const RealDesc &d : E->desc)
        if (d.active && (tma_rows(d.N, family_reach(E)) == 0 || d.off % 4 != 0)) return false;
    return true;
}

typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *,
                                  const cuuint64_t *, const cuuint64_t *, const cuuint32_t *,
                                  const cuuint32_t *, CUtensorMapInterleave, CUtensorMapSwizzle,
                                  CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

/* cuTensorMapEncodeTiled through the runtime's driver entry point (no link
 * against the driver library); null when unavailable. */
EncodeTiledFn encode_tiled() {
    static EncodeTiledFn fn = [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000,
                                             cudaEnableDefault, &q) != cudaSuccess ||
            q != cudaDriverEntryPointSuccess) {
            cudaGetLastError();
            return (EncodeTiledFn) nullptr;
        }
        return (EncodeTiledFn)p;
    }();
    return fn;
}

/* Tiles and tensor maps of the tensor-copy kernels (tiles of nz planes). */
void build_tma(sh_ensemble *E, int nz) {
    namespace T = sh::fast::tma;
    const int H = family_reach(E);
    EncodeTiledFn enc = encode_tiled();
    if (!enc) throw FastErr(SH_ERR_UNSUPPORTED, "tensor map encoding unavailable");
    std::vector<T::TmaTile> tiles;
    std::vector<CUtensorMap> maps((size_t)E->nreal * T::kMapsPerReal);
    std::memset(maps.data(), 0, maps.size() * sizeof(CUtensorMap));
    int slab = 0;
    for (int r = 0; r < E->nreal; ++r) {
        const RealDesc &d = E->desc[r];
        if (!d.active) continue;
        const int N = d.N, t = tma_rows(N, H), P = T::pitch_of(N);
        if (t == 0) throw FastErr(SH_ERR_UNSUPPORTED, "realisation size unsuited to tensor copies");
        slab = std::max(slab, (t + 2 * H) * P);
        const int tz = std::min(nz, N);
        for (int z = 0; z < N; z += tz)
            for (int y = 0; y < N; y += t) tiles.push_back(T::TmaTile{r, y, z, std::min(tz, N - z), t});
        const cuuint64_t dims[3] = {(cuuint64_t)N, (cuuint64_t)N, (cuuint64_t)N};
        const cuuint64_t strides[2] = {(cuuint64_t)N * 4, (cuuint64_t)N * N * 4};
        const cuuint32_t estr[3] = {1, 1, 1};
        for (int a = 0; a < 12; ++a) {
            float *base = (float *)(a < 4 ? E->A0 == E->A[0] ? E->A[a] : E->B[a]
                                          : a < 8 ? (E->A0 == E->A[0] ? E->B[a - 4] : E->A[a - 4])
                                                  : E->K[a - 8]) +
                          d.off;
            for (int sh = 0; sh < 2; ++sh) {
                const cuuint32_t box[3] = {(cuuint32_t)P, (cuuint32_t)(sh == 0 ? t : H), 1};
                const CUresult rc =
                    enc(&maps[T::map_slot(r, a, sh)], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, base,
                        dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                        CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
                if (rc != CUDA_SUCCESS)
                    throw FastErr(SH_ERR_UNSUPPORTED,
                                  "cuTensorMapEncodeTiled failed (" + std::to_string((int)rc) + ")");
            }
        }
    }
    upload_table(tiles, E->d_ttiles, E->ttiles_cap, est(E), "tensor-copy tiles");
    upload_table(maps, E->d_maps, E->maps_cap, est(E), "tensor maps");
    E->ttiles.swap(tiles);
    E->tma_slab = slab;
}

void build_tiles(sh_ensemble *E, int nz) {
    std::vector<FastTile> t;
    for (int r = 0; r < E->nreal; ++r) {
        if (!E->desc[r].active) continue;
        const int N = E->desc[r].N;
        const int tz = std::min(nz, N);
        for (int z = 0; z < N; z += tz)
            for (int y = 0; y < N; y += TY)
                for (int x = 0; x < N; x += TX) t.push_back(FastTile{r, x, y, z, std::min(tz, N - z)});
    }
    upload_table(t, E->d_tiles, E->tiles_cap, est(E), "tile table");
    E->tiles.swap(t);
    E->tile_nz = nz;
    if (E->plane_staging == 1) {
        if (tma_possible(E)) build_tma(E, nz);
        else E->plane_staging = 0;
    }
    drop_graphs(E);
}

void upload_desc(sh_ensemble *E) {
    upload_table(E->desc, E->d_desc, E->desc_cap, est(E), "descriptor table");
    drop_graphs(E);
}

template <class R>
R *arr(const std::vector<void *> &v, int i) {
    return (R *)v[i];
}

int launches_per_step(const sh_ensemble *E) { return E->family == 3 ? 2 : 3; }

/* One step from state `in` (time slot `slot`) to state `out`. */
template <class R, bool KAHAN>
void step_impl(sh_ensemble *E, const std::vector<void *> &in, const std::vector<void *> &out,
               int slot, double dt, cudaStream_t s) {
    const dim3 block(TX, TY);
    const int nt = (int)E->tiles.size();
    if (nt == 0) return; /* an empty pool */
    if (E->family != 3) {
        AxionArgs<R> a;
        std::memset(&a, 0, sizeof(a));
        a.desc = E->d_desc;
        a.tiles = E->d_tiles;
        for (int c = 0; c < 2; ++c) {
            a.y0[c] = arr<R>(in, c);
            a.m0[c] = arr<R>(in, 2 + c);
            a.y1[c] = arr<R>(out, c);
            a.m1[c] = arr<R>(out, 2 + c);
            a.cy[c] = KAHAN ? arr<R>(E->C, c) : nullptr;
            a.cm[c] = KAHAN ? arr<R>(E->C, 2 + c) : nullptr;
            a.K[0][c] = arr<R>(E->K, c);
            a.K[1][c] = arr<R>(E->K, 2 + c);
        }
        a.time = E->d_time;
        a.slot = slot;
        a.h = dt;
        if constexpr (sizeof(R) == 4) {
            if (E->plane_staging == 1) {
                namespace T = sh::fast::tma;
                T::AxionTmaArgs t;
                std::memset(&t, 0, sizeof(t));
                t.desc = E->d_desc;
                t.tiles = E->d_ttiles;
                t.maps = E->d_maps;
                for (int c = 0; c < 2; ++c) {
                    t.y0[c] = a.y0[c];
                    t.m0[c] = a.m0[c];
                    t.y1[c] = a.y1[c];
                    t.m1[c] = a.m1[c];
                    t.cy[c] = a.cy[c];
                    t.cm[c] = a.cm[c];
                    t.K[0][c] = a.K[0][c];
                    t.K[1][c] = a.K[1][c];
                }
                t.time = a.time;
                t.slot = slot;
                t.h = dt;
                /* maps 0-3 describe the buffer that was A at creation */
                t.in_base = in[0] == E->A0 ? 0 : 4;
                t.err = E->d_err;
                const int ntt = (int)E->ttiles.size();
                const size_t s0 = T::smem_bytes(family_reach(E), 2, E->tma_slab);
                const size_t s1 = T::smem_bytes(family_reach(E), 6, E->tma_slab);
                if (E->family == SH_FAMILY_AXION_LAP1) {
                    T::axion_rkn4_tma_kernel<1, 0, KAHAN><<<ntt, T::kThreads, s0, s>>>(t);
                    T::axion_rkn4_tma_kernel<1, 1, KAHAN><<<ntt, T::kThreads, s1, s>>>(t);
                    T::axion_rkn4_tma_kernel<1, 2, KAHAN><<<ntt, T::kThreads, s1, s>>>(t);
                } else {
                    T::axion_rkn4_tma_kernel<2, 0, KAHAN><<<ntt, T::kThreads, s0, s>>>(t);
                    T::axion_rkn4_tma_kernel<2, 1, KAHAN><<<ntt, T::kThreads, s1, s>>>(t);
                    T::axion_rkn4_tma_kernel<2, 2, KAHAN><<<ntt, T::kThreads, s1, s>>>(t);
                }
                return;
            }
        }
        if (E->family == SH_FAMILY_AXION_LAP1) {
            axion_rkn4_kernel<R, 1, 0, KAHAN><<<nt, block, 0, s>>>(a);
            axion_rkn4_kernel<R, 1, 1, KAHAN><<<nt, block, 0, s>>>(a);
            axion_rkn4_kernel<R, 1, 2, KAHAN><<<nt, block, 0, s>>>(a);
        } else {
            axion_rkn4_kernel<R, 2, 0, KAHAN><<<nt, block, 0, s>>>(a);
            axion_rkn4_kernel<R, 2, 1, KAHAN><<<nt, block, 0, s>>>(a);
            axion_rkn4_kernel<R, 2, 2, KAHAN><<<nt, block, 0, s>>>(a);
        }
    } else {
        FoptArgs<R> a;
        std::memset(&a, 0, sizeof(a));
        a.desc = E->d_desc;
        a.tiles = E->d_tiles;
        a.time = E->d_time;
        a.slot = slot;
        a.dt = dt;
        const size_t shm = (size_t)5 * 7 * (TY + 4) * (TX + 4) * sizeof(R);
        for (int c = 0; c < 7; ++c) {
            a.x[c] = arr<R>(in, c);
            a.v[c] = arr<R>(in, 7 + c);
            a.xo[c] = arr<R>(out, c);
            a.vo[c] = arr<R>(E->K, c); /* vh */
            a.cx[c] = KAHAN ? arr<R>(E->C, c) : nullptr;
            a.cv[c] = KAHAN ? arr<R>(E->C, 7 + c) : nullptr;
        }
        fopt_leapfrog_kernel<R, 0, KAHAN><<<nt, block, shm, s>>>(a);
        for (int c = 0; c < 7; ++c) {
            a.x[c] = arr<R>(out, c);
            a.v[c] = arr<R>(E->K, c);
            a.vo[c] = arr<R>(out, 7 + c);
        }
        fopt_leapfrog_kernel<R, 1, KAHAN><<<nt, block, shm, s>>>(a);
    }
}

void step_dispatch(sh_ensemble *E, const std::vector<void *> &in,
                   const std::vector<void *> &out, int slot, double dt, cudaStream_t s) {
    if (E->precision == SH_PREC_FP64) step_impl<double, false>(E, in, out, slot, dt, s);
    else if (E->precision == SH_PREC_FP32) step_impl<float, false>(E, in, out, slot, dt, s);
    else step_impl<float, true>(E, in, out, slot, dt, s);
    fck(cudaGetLastError(), "ensemble step launch");
}

/* One step A -> B, then swap, either by direct launches or by the graph of
 * the current parity (captured on first use for this step size). */
void step_once(sh_ensemble *E, double dt, cudaStream_t s) {
    const int par = E->A[0] == E->A0 ? 0 : 1;
    if (E->use_graph) {
        if (E->graph[par] && E->graph_dt[par] != dt) {
            cudaGraphExecDestroy(E->graph[par]);
            E->graph[par] = nullptr;
        }
        if (!E->graph[par]) {
            cudaStream_t cs = nullptr;
            fck(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking), "capture stream");
            cudaGraph_t g = nullptr;
            cudaError_t e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
            if (e == cudaSuccess) {
                step_dispatch(E, E->A, E->B, E->slot, dt, cs);
                e = cudaStreamEndCapture(cs, &g);
            }
            cudaStreamDestroy(cs);
            fck(e, "step capture");
            e = cudaGraphInstantiate(&E->graph[par], g, 0);
            cudaGraphDestroy(g);
            fck(e, "graph instantiate");
            E->graph_dt[par] = dt;
        }
        fck(cudaGraphLaunch(E->graph[par], s), "graph launch");
    } else {
        step_dispatch(E, E->A, E->B, E->slot, dt, s);
    }
    E->launches += launches_per_step(E);
    std::swap(E->A, E->B);
    E->slot = 1 - E->slot;
}

template <class F>
int fguard(sh_ensemble *E, F &&f) {
    try {
        f();
        return SH_OK;
    } catch (const FastErr &e) {
        if (E) E->err = e.what();
        return e.code;
    } catch (const std::bad_alloc &) {
        if (E) E->err = "host allocation failed";
        return SH_ERR_NOMEM;
    } catch (const std::exception &e) {
        if (E) E->err = e.what();
        return SH_ERR_ARG;
    }
}

void set_smem_limits() {
    namespace T = sh::fast::tma;
    const cudaFuncAttribute dyn = cudaFuncAttributeMaxDynamicSharedMemorySize;
    const int t1 = (int)T::smem_bytes(1, 6, 1024), t2 = (int)T::smem_bytes(2, 6, 1024);
    fck(cudaFuncSetAttribute(T::axion_rkn4_tma_kernel<1, 0, false>, dyn, t1), "smem limit");
    fck(cudaFuncSetAttribute(T::axion_rkn4_tma_kernel<1, 1, false>, dyn, t1), "smem limit");
    fck(cudaFuncSetAttribute(T::axion_rkn4_tma_kernel<1, 2, false>, dyn, t1), "smem limit");
    fck(cudaFuncSetAttribute(T::axion_rkn4_tma_kernel<1, 0, true>, dyn, t1), "smem limit");
    fck(cudaFuncSetAttribute(T::axion_rkn4_tma_kernel<1, 1, true>, dyn, t1), "smem limit");
    fck(cudaFuncSetAttribute(T::axion_rkn4_tma_kernel<1, 2, true>, dyn, t1), "smem limit");
    fck(cudaFuncSetAttribute(T::axion_rkn4_tma_kernel<2, 0, false>, dyn, t2), "smem limit");
    fck(cudaFuncSetAttribute(T::axion_rkn4_tma_kernel<2, 1, false>, dyn, t2), "smem limit");
    fck(cudaFuncSetAttribute(T::axion_rkn4_tma_kernel<2, 2, false>, dyn, t2), "smem limit");
    fck(cudaFuncSetAttribute(T::axion_rkn4_tma_kernel<2, 0, true>, dyn, t2), "smem limit");
    fck(cudaFuncSetAttribute(T::axion_rkn4_tma_kernel<2, 1, true>, dyn, t2), "smem limit");
    fck(cudaFuncSetAttribute(T::axion_rkn4_tma_kernel<2, 2, true>, dyn, t2), "smem limit");
    const int shf = 5 * 7 * (TY + 4) * (TX + 4) * (int)sizeof(float);
    const int shd = 5 * 7 * (TY + 4) * (TX + 4) * (int)sizeof(double);
    const cudaFuncAttribute at = cudaFuncAttributeMaxDynamicSharedMemorySize;
    fck(cudaFuncSetAttribute(fopt_leapfrog_kernel<float, 0, true>, at, shf), "smem limit");
    fck(cudaFuncSetAttribute(fopt_leapfrog_kernel<float, 1, true>, at, shf), "smem limit");
    fck(cudaFuncSetAttribute(fopt_leapfrog_kernel<float, 0, false>, at, shf), "smem limit");
    fck(cudaFuncSetAttribute(fopt_leapfrog_kernel<float, 1, false>, at, shf), "smem limit");
    fck(cudaFuncSetAttribute(fopt_leapfrog_kernel<double, 0, false>, at, shd), "smem limit");
    fck(cudaFuncSetAttribute(fopt_leapfrog_kernel<double, 1, false>, at, shd), "smem limit");
}

/* Host component c (level order: fields, scalar momenta, u_ij, du_ij) to the
 * internal array (positions, then momenta). */
int internal_comp(const sh_ensemble *E, int c) {
    if (E->family != SH_FAMILY_FOPT_GW) return c;
    return c == 0 ? 0 : (c == 1 ? 7 : (c < 8 ? c - 1 : c));
}

double *staging(sh_ensemble *E, size_t elems) {
    if (elems > E->staging_cap) {
        if (E->staging) {
            fck(cudaStreamSynchronize(est(E)), "staging");
            cudaFree(E->staging);
            E->staging = nullptr;
            E->staging_cap = 0;
        }
        fck(cudaMalloc(&E->staging, elems * sizeof(double)), "staging");
        E->staging_cap = elems;
    }
    return E->staging;
}

long long cells_of(const sh_ensemble *E, int r) {
    return (long long)E->desc[r].N * E->desc[r].N * E->desc[r].N;
}

/* A wait of a stage kernel that ran out (SH_ERR_TIMEOUT recorded on the
 * device) is reported by the next call that synchronises; the flag is
 * cleared then. */
void check_device_error(sh_ensemble *E) {
    int e = 0;
    fck(cudaMemcpyAsync(&e, E->d_err, sizeof(int), cudaMemcpyDeviceToHost, est(E)),
        "error flag download");
    fck(cudaStreamSynchronize(est(E)), "error flag");
    if (e != 0) {
        fck(cudaMemsetAsync(E->d_err, 0, sizeof(int), est(E)), "error flag clear");
        throw FastErr(e, "a stage kernel's wait for its tensor copies ran out; the state of "
                         "the steps since the last check is not valid");
    }
}

double read_time(sh_ensemble *E) {
    double t = 0.;
    fck(cudaMemcpyAsync(&t, E->d_time + E->slot, sizeof(double), cudaMemcpyDeviceToHost, est(E)),
        "time download");
    fck(cudaStreamSynchronize(est(E)), "time");
    check_device_error(E);
    return t;
}

void alloc_error_flag(sh_ensemble *E) {
    fck(cudaMalloc(&E->d_err, sizeof(int)), "error flag");
    fck(cudaMemset(E->d_err, 0, sizeof(int)), "error flag clear");
}

} // namespace

extern "C" {

int sh_ensemble_create(sh_ctx *ctx, int family, int precision, int nreal, const int *N,
                       const double *dx, const double *params, sh_ensemble **out) {
    if (!ctx || !out || !N || !dx || nreal <= 0) return SH_ERR_ARG;
    *out = nullptr;
    if (family != SH_FAMILY_AXION_LAP1 && family != SH_FAMILY_AXION_LAP2 &&
        family != SH_FAMILY_FOPT_GW)
        return SH_ERR_ARG;
    if (precision != SH_PREC_FP64 && precision != SH_PREC_FP32_KAHAN && precision != SH_PREC_FP32)
        return SH_ERR_ARG;
    sh_ensemble *E = new (std::nothrow) sh_ensemble();
    if (!E) return SH_ERR_NOMEM;
    E->ctx = ctx;
    int rc = fguard(E, [&] {
        set_smem_limits();
        E->family = family;
        E->precision = precision;
        E->nreal = nreal;
        E->ncomp = family == SH_FAMILY_FOPT_GW ? 14 : 4;
        E->esize = precision == SH_PREC_FP64 ? 8 : 4;
        long long off = 0;
        for (int r = 0; r < nreal; ++r) {
            freq(N[r] >= 8 && N[r] <= 4096, "realisations need 8 <= N <= 4096");
            freq(dx[r] > 0, "dx must be positive");
            RealDesc d;
            d.off = off;
            d.N = N[r];
            d.active = 1;
            d.dx = dx[r];
            d.dt = 0.;
            for (int q = 0; q < 4; ++q) d.p[q] = params ? params[4 * r + q] : 0.;
            off += (long long)N[r] * N[r] * N[r];
            E->desc.push_back(d);
        }
        E->total = off;
        upload_desc(E);
        const size_t bytes = (size_t)E->total * E->esize;
        auto alloc = [&](std::vector<void *> &v, int n) {
            for (int q = 0; q < n; ++q) {
                void *p = nullptr;
                fck(cudaMalloc(&p, bytes), "ensemble allocation");
                v.push_back(p);
                fck(cudaMemset(p, 0, bytes), "ensemble clear");
            }
        };
        alloc(E->A, E->ncomp);
        alloc(E->B, E->ncomp);
        if (precision == SH_PREC_FP32_KAHAN) alloc(E->C, E->ncomp);
        alloc(E->K, family == SH_FAMILY_FOPT_GW ? 7 : 4);
        E->A0 = E->A[0];
        fck(cudaMalloc(&E->d_time, 2 * sizeof(double)), "time");
        fck(cudaMemset(E->d_time, 0, 2 * sizeof(double)), "time clear");
        fck(cudaMalloc(&E->d_counts, nreal * sizeof(unsigned long long)), "counts");
        E->counts_cap = nreal;
        alloc_error_flag(E);
        build_tiles(E, 16);
    });
    if (rc != SH_OK) {
        std::string m = E->err;
        sh_ensemble_destroy(E);
        return rc;
    }
    *out = E;
    return SH_OK;
}

int sh_ensemble_destroy(sh_ensemble *E) {
    if (!E) return SH_ERR_ARG;
    cudaStreamSynchronize(est(E));
    drop_graphs(E);
    for (auto *v : {&E->A, &E->B, &E->C, &E->K})
        for (void *p : *v) cudaFree(p);
    cudaFree(E->d_desc);
    cudaFree(E->d_tiles);
    cudaFree(E->d_ttiles);
    cudaFree(E->d_maps);
    cudaFree(E->d_err);
    cudaFree(E->d_time);
    cudaFree(E->d_partial);
    cudaFree(E->d_counts);
    cudaFree(E->gw_scratch);
    cudaFree(E->staging);
    E->gw.release();
    delete E;
    return SH_OK;
}

const char *sh_ensemble_last_error(const sh_ensemble *E) { return E ? E->err.c_str() : ""; }

int sh_ensemble_info(const sh_ensemble *E, int *family, int *precision, int *nreal, int *ncomp,
                     long long *cells, long long *device_bytes, int *tile_nz) {
    if (!E) return SH_ERR_ARG;
    if (family) *family = E->family;
    if (precision) *precision = E->precision;
    if (nreal) *nreal = E->nreal;
    if (ncomp) *ncomp = E->ncomp;
    if (cells) *cells = E->total;
    if (device_bytes)
        *device_bytes =
            (long long)(E->A.size() + E->B.size() + E->C.size() + E->K.size()) * E->total *
            (long long)E->esize;
    if (tile_nz) *tile_nz = E->tile_nz;
    return SH_OK;
}

long long sh_ensemble_kernel_launches(const sh_ensemble *E) { return E ? E->launches : 0; }

int sh_ensemble_set_time(sh_ensemble *E, double t) {
    if (!E) return SH_ERR_ARG;
    return fguard(E, [&] {
        const double tt[2] = {t, t};
        fck(cudaMemcpyAsync(E->d_time, tt, sizeof(tt), cudaMemcpyHostToDevice, est(E)),
            "time upload");
        fck(cudaStreamSynchronize(est(E)), "time");
    });
}

int sh_ensemble_time(sh_ensemble *E, double *t) {
    if (!E || !t) return SH_ERR_ARG;
    return fguard(E, [&] { *t = read_time(E); });
}

int sh_ensemble_write(sh_ensemble *E, int r, const double *host) {
    if (!E || !host || r < 0 || r >= E->nreal || !E->desc[r].active) return SH_ERR_ARG;
    return fguard(E, [&] {
        const long long n = cells_of(E, r), o = E->desc[r].off;
        cudaStream_t s = est(E);
        double *d = staging(E, (size_t)n);
        for (int hc = 0; hc < E->ncomp; ++hc) {
            const int c = internal_comp(E, hc);
            fck(cudaMemcpyAsync(d, host + (size_t)hc * n, n * sizeof(double),
                                cudaMemcpyHostToDevice, s),
                "upload");
            if (E->esize == 8)
                store_kernel<double><<<fgrid(n), 256, 0, s>>>(d, (double *)E->A[c] + o, nullptr, n);
            else
                store_kernel<float><<<fgrid(n), 256, 0, s>>>(
                    d, (float *)E->A[c] + o, E->C.empty() ? nullptr : (float *)E->C[c] + o, n);
            E->launches++;
        }
        fck(cudaStreamSynchronize(s), "write");
    });
}

int sh_ensemble_read(sh_ensemble *E, int r, double *host) {
    if (!E || !host || r < 0 || r >= E->nreal || !E->desc[r].active) return SH_ERR_ARG;
    return fguard(E, [&] {
        const long long n = cells_of(E, r), o = E->desc[r].off;
        cudaStream_t s = est(E);
        double *d = staging(E, (size_t)n);
        for (int hc = 0; hc < E->ncomp; ++hc) {
            const int c = internal_comp(E, hc);
            if (E->esize == 8)
                load_kernel<double><<<fgrid(n), 256, 0, s>>>((double *)E->A[c] + o, nullptr, d, n);
            else
                load_kernel<float><<<fgrid(n), 256, 0, s>>>(
                    (float *)E->A[c] + o, E->C.empty() ? nullptr : (float *)E->C[c] + o, d, n);
            E->launches++;
            fck(cudaMemcpyAsync(host + (size_t)hc * n, d, n * sizeof(double),
                                cudaMemcpyDeviceToHost, s),
                "download");
        }
        fck(cudaStreamSynchronize(s), "read");
        check_device_error(E);
    });
}

int sh_ensemble_set_graph(sh_ensemble *E, int on) {
    if (!E) return SH_ERR_ARG;
    E->use_graph = on != 0;
    if (!E->use_graph) drop_graphs(E);
    return SH_OK;
}

int sh_ensemble_step(sh_ensemble *E, double dt, int nsteps) {
    if (!E || nsteps < 0 || !(dt >= 0)) return SH_ERR_ARG;
    if (dt == 0 && !(E->pool && E->family == SH_FAMILY_FOPT_GW)) return SH_ERR_ARG;
    return fguard(E, [&] {
        cudaStream_t s = est(E);
        for (int q = 0; q < nsteps; ++q) step_once(E, dt, s);
    });
}

int sh_ensemble_set_staging(sh_ensemble *E, int staging) {
    if (!E || (staging != 0 && staging != 1)) return SH_ERR_ARG;
    return fguard(E, [&] {
        if (staging == 1 && !(tma_possible(E) && encode_tiled()))
            throw FastErr(SH_ERR_UNSUPPORTED,
                          "tensor-copy staging needs the axion family in FP32 storage with "
                          "every realisation's N a multiple of 4 and at most 256");
        E->plane_staging = staging;
        build_tiles(E, E->tile_nz);
    });
}

int sh_ensemble_staging(const sh_ensemble *E, int *staging) {
    if (!E || !staging) return SH_ERR_ARG;
    *staging = E->plane_staging;
    return SH_OK;
}

int sh_probe_wait_timeout(int device, int *status) {
    if (!status) return SH_ERR_ARG;
    *status = SH_OK;
    if (cudaSetDevice(device) != cudaSuccess) return SH_ERR_CUDA;
    int *d = nullptr;
    if (cudaMalloc(&d, sizeof(int)) != cudaSuccess) return SH_ERR_NOMEM;
    int h = -1;
    cudaError_t e = cudaMemset(d, 0xFF, sizeof(int));
    if (e == cudaSuccess) {
        sh::fast::tma::wait_timeout_probe_kernel<<<1, 32>>>(d, 2000000ull); /* 2 ms */
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(&h, d, sizeof(int), cudaMemcpyDeviceToHost);
    cudaFree(d);
    if (e != cudaSuccess) return SH_ERR_CUDA;
    *status = h;
    return SH_OK;
}

int sh_ensemble_tune(sh_ensemble *E, int tile_nz, double dt, int *chosen) {
    if (!E || tile_nz < 0 || !(dt > 0)) return SH_ERR_ARG;
    return fguard(E, [&] {
        if (tile_nz > 0) {
            build_tiles(E, tile_nz);
        } else {
            cudaStream_t s = est(E);
            /* the trial steps write B, K, the compensations and the other
             * time slot: keep a copy of the compensations and the time */
            const size_t bytes = (size_t)E->total * E->esize;
            std::vector<void *> saved;
            auto release = [&] {
                for (void *p : saved) cudaFree(p);
            };
            try {
                for (void *c : E->C) {
                    void *p = nullptr;
                    fck(cudaMalloc(&p, bytes), "tune backup");
                    saved.push_back(p);
                    fck(cudaMemcpyAsync(p, c, bytes, cudaMemcpyDeviceToDevice, s), "tune backup");
                }
                double tsave[2];
                fck(cudaMemcpyAsync(tsave, E->d_time, sizeof(tsave), cudaMemcpyDeviceToHost, s),
                    "time");
                cudaEvent_t ev[2];
                fck(cudaEventCreate(&ev[0]), "event");
                fck(cudaEventCreate(&ev[1]), "event");
                float best = 1e30f;
                int bestnz = E->tile_nz, best_staging = E->plane_staging;
                /* two dimensions: the stencil-plane staging (registers, or
                 * tensor copies where the ensemble allows them) and the
                 * planes per tile */
                const int nstaging = tma_possible(E) && encode_tiled() ? 2 : 1;
                for (int stg = 0; stg < nstaging; ++stg)
                    for (int nz : kTuneCandidates) {
                        E->plane_staging = stg;
                        build_tiles(E, nz);
                        step_dispatch(E, E->A, E->B, E->slot, dt, s); /* warm-up */
                        fck(cudaEventRecord(ev[0], s), "record");
                        for (int rep = 0; rep < 3; ++rep)
                            step_dispatch(E, E->A, E->B, E->slot, dt, s);
                        fck(cudaEventRecord(ev[1], s), "record");
                        fck(cudaEventSynchronize(ev[1]), "tune");
                        E->launches += 4 * launches_per_step(E);
                        float ms = 0.f;
                        cudaEventElapsedTime(&ms, ev[0], ev[1]);
                        if (ms < best) {
                            best = ms;
                            bestnz = nz;
                            best_staging = stg;
                        }
                    }
                cudaEventDestroy(ev[0]);
                cudaEventDestroy(ev[1]);
                check_device_error(E);
                E->plane_staging = best_staging;
                build_tiles(E, bestnz);
                for (size_t q = 0; q < saved.size(); ++q)
                    fck(cudaMemcpyAsync(E->C[q], saved[q], bytes, cudaMemcpyDeviceToDevice, s),
                        "tune restore");
                fck(cudaMemcpyAsync(E->d_time, tsave, sizeof(tsave), cudaMemcpyHostToDevice, s),
                    "time");
                fck(cudaStreamSynchronize(s), "tune");
            } catch (...) {
                cudaStreamSynchronize(s);
                release();
                throw;
            }
            release();
        }
        if (chosen) *chosen = E->tile_nz;
    });
}

int sh_ensemble_energy(sh_ensemble *E, double *energy) {
    if (!E || !energy) return SH_ERR_ARG;
    return fguard(E, [&] {
        cudaStream_t s = est(E);
        const double eta = read_time(E);
        const int nt = (int)E->tiles.size();
        for (int r = 0; r < E->nreal; ++r) energy[r] = 0.;
        if (nt == 0) return;
        if (E->partial_cap < (size_t)nt) {
            cudaFree(E->d_partial);
            E->d_partial = nullptr;
            E->partial_cap = 0;
            fck(cudaMalloc(&E->d_partial, nt * sizeof(double)), "partials");
            E->partial_cap = nt;
        }
        const dim3 block(TX, TY);
        const bool fopt = E->family == SH_FAMILY_FOPT_GW;
        const int i0 = 0, i1 = fopt ? 0 : 1, i2 = fopt ? 7 : 2, i3 = fopt ? 7 : 3;
        auto C = [&](int c) { return E->C.empty() ? nullptr : (const float *)E->C[c]; };
        if (E->esize == 8)
            energy_kernel<double><<<nt, block, 0, s>>>(
                E->d_desc, E->d_tiles, (double *)E->A[i0], (double *)E->A[i1],
                (double *)E->A[i2], (double *)E->A[i3], nullptr, nullptr, nullptr, nullptr,
                E->family, eta, E->d_partial);
        else
            energy_kernel<float><<<nt, block, 0, s>>>(
                E->d_desc, E->d_tiles, (float *)E->A[i0], (float *)E->A[i1], (float *)E->A[i2],
                (float *)E->A[i3], C(i0), C(i1), C(i2), C(i3), E->family, eta, E->d_partial);
        E->launches++;
        fck(cudaGetLastError(), "energy launch");
        std::vector<double> part(nt);
        fck(cudaMemcpyAsync(part.data(), E->d_partial, nt * sizeof(double),
                            cudaMemcpyDeviceToHost, s),
            "partials download");
        fck(cudaStreamSynchronize(s), "energy");
        for (int r = 0; r < E->nreal; ++r) energy[r] = 0.;
        for (int q = 0; q < nt; ++q) energy[E->tiles[q].r] += part[q];
    });
}

int sh_ensemble_string_count(sh_ensemble *E, long long *counts) {
    if (!E || !counts || E->family == SH_FAMILY_FOPT_GW) return SH_ERR_ARG;
    return fguard(E, [&] {
        cudaStream_t s = est(E);
        const int nt = (int)E->tiles.size();
        for (int r = 0; r < E->nreal; ++r) counts[r] = 0;
        if (nt == 0) return;
        fck(cudaMemsetAsync(E->d_counts, 0, E->nreal * sizeof(unsigned long long), s), "clear");
        const dim3 block(TX, TY);
        auto C = [&](int c) { return E->C.empty() ? nullptr : (const float *)E->C[c]; };
        if (E->esize == 8)
            string_count_kernel<double><<<nt, block, 0, s>>>(E->d_desc, E->d_tiles,
                                                             (double *)E->A[0], (double *)E->A[1],
                                                             nullptr, nullptr, E->d_counts);
        else
            string_count_kernel<float><<<nt, block, 0, s>>>(E->d_desc, E->d_tiles,
                                                            (float *)E->A[0], (float *)E->A[1],
                                                            C(0), C(1), E->d_counts);
        E->launches++;
        fck(cudaGetLastError(), "string count launch");
        std::vector<unsigned long long> c(E->nreal);
        fck(cudaMemcpyAsync(c.data(), E->d_counts, E->nreal * sizeof(unsigned long long),
                            cudaMemcpyDeviceToHost, s),
            "counts download");
        fck(cudaStreamSynchronize(s), "string count");
        check_device_error(E);
        for (int r = 0; r < E->nreal; ++r) counts[r] = (long long)c[r];
    });
}

int sh_ensemble_gw_spectrum(sh_ensemble *E, int r, int zero_padding, int projection_type,
                            int unbinned, double *bins_out, long long *ks_out, int max_bins,
                            int *nbins) {
    if (!E || E->family != SH_FAMILY_FOPT_GW || r < 0 || r >= E->nreal ||
        !E->desc[r].active || !bins_out || !nbins)
        return SH_ERR_ARG;
    return fguard(E, [&] {
        freq(zero_padding >= 1, "zero_padding must be >= 1");
        freq(projection_type >= 1 && projection_type <= 3, "projection_type must be 1..3");
        cudaStream_t s = est(E);
        const int N = E->desc[r].N;
        const int P = N * zero_padding;
        freq(P % 2 == 0, "spectrum grid size must be even");
        const size_t sbytes = (sh::gw_scratch_bytes(N, zero_padding) + 255) & ~size_t(255);
        const size_t maxbins = (size_t)3 * (P / 2 + 1) * (P / 2 + 1) + 16;
        const size_t need = sbytes + maxbins * sizeof(double);
        if (need > E->gw_scratch_cap) {
            cudaFree(E->gw_scratch);
            E->gw_scratch = nullptr;
            E->gw_scratch_cap = 0;
            fck(cudaMalloc(&E->gw_scratch, need), "gw scratch");
            E->gw_scratch_cap = need;
        }
        double *scratch = (double *)E->gw_scratch;
        double *bins_dev = (double *)((char *)E->gw_scratch + sbytes);
        /* du_xx, du_xy, du_xz, du_yy, du_yz, du_zz among the momenta
         * (dPhi, du_xx, du_yy, du_zz, du_xy, du_xz, du_yz) */
        const int sel[6] = {8, 11, 12, 9, 13, 10};
        const long long n = cells_of(E, r), o = E->desc[r].off;
        int nb = 0;
        std::string err;
        const bool k = !E->C.empty();
        cudaError_t e;
        if (E->spectrum_precision == SH_PREC_FP64)
            e = sh::gw_spectrum_packed(
                E->gw, s, P, N, projection_type, unbinned, scratch, bins_dev, &nb, &E->launches,
                err, [&](int p, double2 *dst) {
                    const int a = sel[2 * p], b = sel[2 * p + 1];
                    if (E->esize == 8)
                        gw_pack_fast_kernel<double><<<fgrid(n), 256, 0, s>>>(
                            (double *)E->A[a], nullptr, (double *)E->A[b], nullptr, o, N, P,
                            dst);
                    else
                        gw_pack_fast_kernel<float><<<fgrid(n), 256, 0, s>>>(
                            (float *)E->A[a], k ? (float *)E->C[a] : nullptr, (float *)E->A[b],
                            k ? (float *)E->C[b] : nullptr, o, N, P, dst);
                });
        else
            e = sh::gw_spectrum_packed32(
                E->gw, s, P, N, projection_type, unbinned, scratch, bins_dev, &nb, &E->launches,
                err, [&](int p, float2 *dst) {
                    const int a = sel[2 * p], b = sel[2 * p + 1];
                    if (E->esize == 8)
                        gw_pack_fast32_kernel<double><<<fgrid(n), 256, 0, s>>>(
                            (double *)E->A[a], nullptr, (double *)E->A[b], nullptr, o, N, P,
                            dst);
                    else
                        gw_pack_fast32_kernel<float><<<fgrid(n), 256, 0, s>>>(
                            (float *)E->A[a], k ? (float *)E->C[a] : nullptr, (float *)E->A[b],
                            k ? (float *)E->C[b] : nullptr, o, N, P, dst);
                });
        if (!err.empty()) throw FastErr(SH_ERR_CUDA, err);
        fck(e, "gw spectrum");
        *nbins = nb;
        freq(nb <= max_bins, "bins_out too small");
        fck(cudaMemcpyAsync(bins_out, bins_dev, nb * sizeof(double), cudaMemcpyDeviceToHost, s),
            "bins download");
        fck(cudaStreamSynchronize(s), "gw spectrum");
        if (ks_out) std::copy(E->gw.ks().begin(), E->gw.ks().end(), ks_out);
    });
}

int sh_ensemble_set_spectrum_precision(sh_ensemble *E, int precision) {
    if (!E || (precision != SH_PREC_FP64 && precision != SH_PREC_FP32)) return SH_ERR_ARG;
    E->spectrum_precision = precision;
    return SH_OK;
}

int sh_ensemble_add_bubbles(sh_ensemble *E, int r, int nb, const double *xyz,
                            const double *profile, int nbins, double inv_dx, double Lcut) {
    if (!E || E->family != SH_FAMILY_FOPT_GW || r < 0 || r >= E->nreal ||
        !E->desc[r].active || nb < 0 ||
        (nb > 0 && (!xyz || !profile)) || nbins < 2 || !(inv_dx > 0) || !(Lcut > 0))
        return SH_ERR_ARG;
    if (nb == 0) return SH_OK;
    return fguard(E, [&] {
        freq((long long)(Lcut * inv_dx) + 2 <= nbins,
             "profile needs at least floor(Lcut * inv_dx) + 2 bins");
        cudaStream_t s = est(E);
        const size_t nx = 3 * (size_t)nb, np = 2 * (size_t)nbins;
        double *d = staging(E, nx + np);
        fck(cudaMemcpyAsync(d, xyz, nx * sizeof(double), cudaMemcpyHostToDevice, s), "upload");
        fck(cudaMemcpyAsync(d + nx, profile, np * sizeof(double), cudaMemcpyHostToDevice, s),
            "upload");
        sh::BubbleList bl{d, d + nx, nb, nbins, inv_dx, Lcut};
        const long long n = cells_of(E, r);
        /* internal arrays: Phi 0, dPhi 7 */
        if (E->esize == 8)
            add_bubbles_kernel<double><<<fgrid(n), 256, 0, s>>>(
                E->d_desc, r, (double *)E->A[0], (double *)E->A[7], nullptr, nullptr, bl);
        else
            add_bubbles_kernel<float><<<fgrid(n), 256, 0, s>>>(
                E->d_desc, r, (float *)E->A[0], (float *)E->A[7],
                E->C.empty() ? nullptr : (float *)E->C[0],
                E->C.empty() ? nullptr : (float *)E->C[7], bl);
        E->launches++;
        fck(cudaGetLastError(), "bubble launch");
        fck(cudaStreamSynchronize(s), "bubbles");
    });
}

/* ---- pools: ensembles whose members come and go ---- */

int sh_ensemble_create_pool(sh_ctx *ctx, int family, int precision, long long capacity_cells,
                            sh_ensemble **out) {
    if (!ctx || !out || capacity_cells < 0) return SH_ERR_ARG;
    *out = nullptr;
    if (family != SH_FAMILY_AXION_LAP1 && family != SH_FAMILY_AXION_LAP2 &&
        family != SH_FAMILY_FOPT_GW)
        return SH_ERR_ARG;
    if (precision != SH_PREC_FP64 && precision != SH_PREC_FP32_KAHAN && precision != SH_PREC_FP32)
        return SH_ERR_ARG;
    sh_ensemble *E = new (std::nothrow) sh_ensemble();
    if (!E) return SH_ERR_NOMEM;
    E->ctx = ctx;
    int rc = fguard(E, [&] {
        set_smem_limits();
        E->family = family;
        E->precision = precision;
        E->pool = true;
        E->ncomp = family == SH_FAMILY_FOPT_GW ? 14 : 4;
        E->esize = precision == SH_PREC_FP64 ? 8 : 4;
        const int narrays = 2 * E->ncomp + (precision == SH_PREC_FP32_KAHAN ? E->ncomp : 0) +
                            (family == SH_FAMILY_FOPT_GW ? 7 : 4);
        if (capacity_cells == 0) {
            /* 80% of the free device memory */
            size_t fr = 0, tot = 0;
            fck(cudaMemGetInfo(&fr, &tot), "cudaMemGetInfo");
            capacity_cells = (long long)(0.8 * (double)fr / ((double)narrays * E->esize));
        }
        freq(capacity_cells >= 512, "pool capacity too small");
        E->capacity = capacity_cells;
        E->total = capacity_cells;
        const size_t bytes = (size_t)capacity_cells * E->esize;
        auto alloc = [&](std::vector<void *> &v, int n) {
            for (int q = 0; q < n; ++q) {
                void *p = nullptr;
                fck(cudaMalloc(&p, bytes), "pool allocation");
                v.push_back(p);
            }
        };
        alloc(E->A, E->ncomp);
        alloc(E->B, E->ncomp);
        if (precision == SH_PREC_FP32_KAHAN) alloc(E->C, E->ncomp);
        alloc(E->K, family == SH_FAMILY_FOPT_GW ? 7 : 4);
        E->A0 = E->A[0];
        E->free_ext[0] = capacity_cells;
        fck(cudaMalloc(&E->d_time, 2 * sizeof(double)), "time");
        fck(cudaMemset(E->d_time, 0, 2 * sizeof(double)), "time clear");
        alloc_error_flag(E);
    });
    if (rc != SH_OK) {
        sh_ensemble_destroy(E);
        return rc;
    }
    *out = E;
    return SH_OK;
}

/* A new member of N^3 cells (state zero) in the first free extent that
 * holds it; SH_ERR_NOMEM when none does (the pool is full for now). */
int sh_ensemble_admit(sh_ensemble *E, int N, double dx, const double *params, double dt,
                      int *slot) {
    if (!E || !E->pool || !slot || N < 8 || N > 4096 || !(dx > 0) || dt < 0) return SH_ERR_ARG;
    return fguard(E, [&] {
        const long long n = (long long)N * N * N;
        auto it = E->free_ext.begin();
        while (it != E->free_ext.end() && it->second < n) ++it;
        if (it == E->free_ext.end()) throw FastErr(SH_ERR_NOMEM, "pool full");
        const long long off = it->first, len = it->second;
        E->free_ext.erase(it);
        if (len > n) E->free_ext[off + n] = len - n;
        RealDesc d;
        d.off = off;
        d.N = N;
        d.active = 1;
        d.dx = dx;
        d.dt = dt;
        for (int q = 0; q < 4; ++q) d.p[q] = params ? params[q] : 0.;
        int r = -1;
        for (int q = 0; q < E->nreal; ++q)
            if (!E->desc[q].active) {
                r = q;
                break;
            }
        if (r < 0) {
            r = E->nreal++;
            E->desc.push_back(d);
        } else {
            E->desc[r] = d;
        }
        if ((size_t)E->nreal > E->counts_cap) {
            cudaStream_t s = est(E);
            fck(cudaStreamSynchronize(s), "counts");
            cudaFree(E->d_counts);
            E->d_counts = nullptr;
            E->counts_cap = 0;
            const size_t c = 2 * (size_t)E->nreal + 16;
            fck(cudaMalloc(&E->d_counts, c * sizeof(unsigned long long)), "counts");
            E->counts_cap = c;
        }
        cudaStream_t s = est(E);
        for (auto *v : {&E->A, &E->B, &E->C, &E->K})
            for (void *p : *v)
                fck(cudaMemsetAsync((char *)p + off * E->esize, 0, n * E->esize, s), "clear");
        upload_desc(E);
        build_tiles(E, E->tile_nz);
        *slot = r;
    });
}

int sh_ensemble_release(sh_ensemble *E, int r) {
    if (!E || !E->pool || r < 0 || r >= E->nreal || !E->desc[r].active) return SH_ERR_ARG;
    return fguard(E, [&] {
        RealDesc &d = E->desc[r];
        long long off = d.off, len = (long long)d.N * d.N * d.N;
        d.active = 0;
        /* merge with the free neighbours */
        auto nx = E->free_ext.lower_bound(off);
        if (nx != E->free_ext.end() && nx->first == off + len) {
            len += nx->second;
            E->free_ext.erase(nx);
        }
        auto pv = E->free_ext.lower_bound(off);
        if (pv != E->free_ext.begin()) {
            --pv;
            if (pv->first + pv->second == off) {
                off = pv->first;
                len += pv->second;
                E->free_ext.erase(pv);
            }
        }
        E->free_ext[off] = len;
        upload_desc(E);
        build_tiles(E, E->tile_nz);
    });
}

int sh_ensemble_pool_info(const sh_ensemble *E, long long *capacity, long long *free_cells,
                          long long *largest_free, int *members) {
    if (!E || !E->pool) return SH_ERR_ARG;
    long long fr = 0, big = 0;
    for (const auto &kv : E->free_ext) {
        fr += kv.second;
        big = std::max(big, kv.second);
    }
    int m = 0;
    for (const RealDesc &d : E->desc) m += d.active;
    if (capacity) *capacity = E->capacity;
    if (free_cells) *free_cells = fr;
    if (largest_free) *largest_free = big;
    if (members) *members = m;
    return SH_OK;
}

} /* extern "C" */
