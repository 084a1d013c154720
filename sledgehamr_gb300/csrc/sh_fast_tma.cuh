/* RKN4 stage kernel of the axion family (FP32 storage) with its stencil
 * planes staged in shared memory by the Tensor Memory Accelerator.
 *
 * Same update as axion_rkn4_kernel (sh_fast.cu): stage 0 and 1 write
 * K_STAGE = accel(Y_STAGE, y0'), stage 2 writes the new state with
 * (optionally Kahan-compensated) increments, every stage reading y0, y0'
 * and the earlier K at the stencil points and rebuilding
 * Y = y0 + c h y0' + h^2 a K there (source/integrators/rkn.cpp:55-117,
 * tableau :130-139).
 *
 * Tile: all N cells of TYT rows of one realisation (TYT per realisation,
 * N * TYT <= 768 cells, TYT >= the stencil reach H), marching in z over nz
 * planes.  Taking whole rows makes the periodic wrap in x an index
 * operation in shared memory, so every copy stays inside the realisation:
 * per array and plane, three tiled tensor copies (cp.async.bulk.tensor,
 * 3-D tensor maps over the realisation's N^3 cube) bring the TYT tile rows
 * and the H wrapped rows below and above, each to its own rows of a
 * shared-memory slab whose row pitch is N rounded up to 32 floats (so that
 * every destination is 128-byte aligned; the copy box is that wide and the
 * cells past N arrive as the copy's zero fill, never read).  Two planes are
 * in flight (one mbarrier each, transaction-counted); one thread issues
 * the copies.  A plane, once landed, is turned into the stage positions Y
 * in a ring of 2H+2 planes (one barrier per plane suffices, as in the
 * register-pipelined kernel), and the cells of plane z - H are computed.
 * Values needed only at the cell itself (y0' for the friction, the earlier
 * K and y0 of the final update, the compensations) are read from global
 * memory directly.
 *
 * Every wait on an mbarrier is bounded (kWaitNs of the global timer); when
 * it runs out the block records SH_ERR_TIMEOUT in *err and returns without
 * touching the outputs of the planes it did not finish.
 */
#ifndef SH_FAST_TMA_CUH_
#define SH_FAST_TMA_CUH_

#include <cuda.h> /* CUtensorMap (type only; encoding goes through the runtime's driver entry point) */

namespace sh {
namespace fast {
namespace tma {

constexpr int kThreads = 256;
constexpr int kInFlight = 2;                 /* planes whose copies are in flight */
constexpr int kMaxCells = 768;               /* N * TYT per plane */
constexpr int kCellsPerThread = kMaxCells / kThreads;
constexpr int kMapsPerReal = 24;             /* 12 arrays x 2 box shapes */
constexpr unsigned long long kWaitNs = 1000000000ull; /* 1 s */

/* Tensor-map slots of a realisation: array a (0-3: state buffer A y, y, m,
 * m; 4-7: the same of buffer B; 8-11: K0 (two components), K1), box s (0:
 * TYT rows, 1: H rows). */
__host__ __device__ constexpr int map_slot(int r, int a, int s) {
    return (r * 12 + a) * 2 + s;
}

/* Row pitch (floats) of a shared-memory slab for a realisation of N. */
__host__ __device__ constexpr int pitch_of(int N) { return (N + 31) / 32 * 32; }

struct TmaTile {
    int r;   /* realisation */
    int y0;  /* first row */
    int z0;  /* first plane */
    int nz;  /* planes */
    int tyt; /* rows */
};

struct AxionTmaArgs {
    const RealDesc *desc;
    const TmaTile *tiles;
    const CUtensorMap *maps; /* kMapsPerReal per realisation */
    const float *y0[2], *m0[2];
    float *y1[2], *m1[2];
    float *cy[2], *cm[2];
    float *K[2][2];
    double *time;
    int slot;
    double h;
    int in_base; /* first map array of the input state: 0 (A) or 4 (B) */
    int *err;    /* SH_ERR_TIMEOUT when a wait ran out */
};

__device__ __forceinline__ unsigned smem_addr(const void *p) {
    return (unsigned)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(unsigned long long *bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count)
                 : "memory");
}
__device__ __forceinline__ void fence_mbar_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(unsigned long long *bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)),
                 "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned long long *bar, unsigned parity) {
    unsigned ok;
    asm volatile("{\n\t.reg .pred p;\n\t"
                 "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                 "selp.u32 %0, 1, 0, p;\n\t}"
                 : "=r"(ok)
                 : "r"(smem_addr(bar)), "r"(parity)
                 : "memory");
    return ok != 0;
}
__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
    return t;
}
/* Waits for phase `parity` of bar to complete, at most kWaitNs (then
 * false). */
__device__ __forceinline__ bool mbar_wait(unsigned long long *bar, unsigned parity) {
    if (mbar_try_wait(bar, parity)) return true;
    const unsigned long long t0 = global_ns();
    while (!mbar_try_wait(bar, parity))
        if (global_ns() - t0 > kWaitNs) return false;
    return true;
}
__device__ __forceinline__ void tma_load_3d(void *dst, const CUtensorMap *map, int x, int y,
                                            int z, unsigned long long *bar) {
    asm volatile("cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
                 " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(smem_addr(dst)),
                 "l"(map), "r"(x), "r"(y), "r"(z), "r"(smem_addr(bar))
                 : "memory");
}
__device__ __forceinline__ void tensormap_acquire(const CUtensorMap *map) {
    asm volatile("fence.proxy.tensormap::generic.acquire.gpu [%0], 128;" ::"l"(map) : "memory");
}

/* Dynamic shared memory of a launch whose largest slab (rows * pitch) is
 * `slab` floats. */
__host__ __device__ constexpr size_t smem_bytes(int H, int NA, int slab) {
    return 128 + (size_t)(kInFlight * NA + (2 * H + 2) * 2) * slab * sizeof(float) +
           kInFlight * sizeof(unsigned long long);
}

template <int H, int STAGE, bool KAHAN>
__global__ void __launch_bounds__(kThreads)
    axion_rkn4_tma_kernel(const __grid_constant__ AxionTmaArgs a) {
    constexpr int NA = STAGE == 0 ? 2 : 6; /* arrays at the stencil points */
    constexpr int RING = 2 * H + 2;
    extern __shared__ __align__(128) unsigned char smem_dyn[];
    __shared__ float kc[8];
    __shared__ int timed_out;
    /* every copy destination must be 128-byte aligned: the slabs start at
     * the first such address of the dynamic allocation (128 bytes extra) */
    unsigned char *smem = smem_dyn + ((128u - (smem_addr(smem_dyn) & 127u)) & 127u);

    const TmaTile tl = a.tiles[blockIdx.x];
    const RealDesc d = a.desc[tl.r];
    const int N = d.N, P = pitch_of(N), TYT = tl.tyt, ROWS = TYT + 2 * H;
    const int slab = ROWS * P; /* floats per array and plane: a multiple of 32 */
    const long long off = d.off;
    float *raw = reinterpret_cast<float *>(smem);         /* [kInFlight][NA][slab] */
    float *Yr = raw + kInFlight * NA * slab;             /* [RING][2][slab] */
    unsigned long long *bar = reinterpret_cast<unsigned long long *>(Yr + RING * 2 * slab);
    const int tid = threadIdx.x;

    /* maps of the arrays read at the stencil points, in raw order */
    const CUtensorMap *mp[NA][2];
    {
        const int ids[6] = {a.in_base, a.in_base + 1, a.in_base + 2, a.in_base + 3,
                            STAGE == 2 ? 10 : 8, STAGE == 2 ? 11 : 9};
#pragma unroll
        for (int q = 0; q < NA; ++q) {
            mp[q][0] = a.maps + map_slot(tl.r, ids[q], 0);
            mp[q][1] = a.maps + map_slot(tl.r, ids[q], 1);
        }
    }
    const int zb = tl.z0 - H;
    const int nplanes = tl.nz + 2 * H;
    const unsigned bytes = (unsigned)(NA * slab * sizeof(float));
    auto issue = [&](int p) { /* plane zb + p into raw slot p % kInFlight */
        const int s = p % kInFlight;
        const int zw = wrap(zb + p, N);
        unsigned long long *b = bar + s;
        mbar_expect_tx(b, bytes);
        const int ylo = tl.y0 >= H ? tl.y0 - H : tl.y0 - H + N;
        const int yhi = tl.y0 + TYT < N ? tl.y0 + TYT : tl.y0 + TYT - N;
#pragma unroll
        for (int q = 0; q < NA; ++q) {
            float *dst = raw + (s * NA + q) * slab;
            tma_load_3d(dst, mp[q][1], 0, ylo, zw, b);                 /* rows y0-H .. y0-1 */
            tma_load_3d(dst + H * P, mp[q][0], 0, tl.y0, zw, b);       /* rows y0 .. y0+TYT-1 */
            tma_load_3d(dst + (H + TYT) * P, mp[q][1], 0, yhi, zw, b); /* rows above */
        }
    };

    /* RKN4 tableau (rkn.cpp:130-139): c = {0, 1/2, 1}; a21 = 1/8; a32 = 1/2;
     * bbar = {1/6, 1/3, 0}; b = {1/6, 2/3, 1/6}. */
    if (tid == 0) {
        timed_out = 0;
        const double hh = a.h * a.h;
        const double t0 = a.time[a.slot];
        const double ts = t0 + a.h * (STAGE == 0 ? 0. : (STAGE == 1 ? 0.5 : 1.));
        if (STAGE == 2 && blockIdx.x == 0) a.time[1 - a.slot] = t0 + a.h;
        kc[0] = (float)(STAGE == 0 ? 0. : (STAGE == 1 ? 0.5 * a.h : a.h));   /* cm */
        kc[1] = (float)(STAGE == 1 ? hh / 8. : (STAGE == 2 ? hh / 2. : 0.)); /* ck */
        kc[2] = (float)(-2. / ts);                                           /* friction */
        kc[3] = (float)d.p[0];                                               /* lambda */
        kc[4] = (float)d.p[1];                                               /* c */
        kc[5] = (float)(ts * ts);                                            /* eta^2 */
        kc[6] = (float)(1. / (d.dx * d.dx));
        kc[7] = kc[6] / 12.f; /* as the register-pipelined kernel forms it */
#pragma unroll
        for (int q = 0; q < NA; ++q) {
            tensormap_acquire(mp[q][0]);
            tensormap_acquire(mp[q][1]);
        }
        for (int s = 0; s < kInFlight; ++s) mbar_init(bar + s, 1);
        fence_mbar_init();
    }
    __syncthreads();
    if (tid == 0)
        for (int p = 0; p < kInFlight && p < nplanes; ++p) issue(p);
    const float cm = kc[0], ck = kc[1], friction = kc[2], lam = kc[3], cst = kc[4],
                eta2 = kc[5], inv_dx2 = kc[6], inv12dx2 = kc[7];
    const float h = (float)a.h, h2 = (float)(a.h * a.h);
    const int ncell = N * TYT;

    for (int p = 0; p < nplanes; ++p) {
        const int zc = zb + p - H; /* plane computed in this iteration */
        const bool compute = p >= 2 * H;
        /* centre values of the cells of plane zc */
        float q0[kCellsPerThread], q1[kCellsPerThread], ka0[kCellsPerThread],
            ka1[kCellsPerThread], kb0[kCellsPerThread], kb1[kCellsPerThread],
            yc0[kCellsPerThread], yc1[kCellsPerThread];
        float c0[kCellsPerThread], c1[kCellsPerThread], c2[kCellsPerThread], c3[kCellsPerThread];
#pragma unroll
        for (int k = 0; k < kCellsPerThread; ++k) {
            const int qc = tid + k * kThreads;
            q0[k] = q1[k] = ka0[k] = ka1[k] = kb0[k] = kb1[k] = yc0[k] = yc1[k] = 0.f;
            c0[k] = c1[k] = c2[k] = c3[k] = 0.f;
            if (!compute || qc >= ncell) continue;
            const long long e = off + ((long long)zc * N + tl.y0 + qc / N) * N + qc % N;
            q0[k] = a.m0[0][e];
            q1[k] = a.m0[1][e];
            if (STAGE == 2) {
                ka0[k] = a.K[0][0][e];
                ka1[k] = a.K[0][1][e];
                kb0[k] = a.K[1][0][e];
                kb1[k] = a.K[1][1][e];
                yc0[k] = a.y0[0][e];
                yc1[k] = a.y0[1][e];
                if (KAHAN) {
                    c0[k] = a.cy[0][e];
                    c1[k] = a.cy[1][e];
                    c2[k] = a.cm[0][e];
                    c3[k] = a.cm[1][e];
                }
            }
        }
        /* the copies of plane zb + p */
        const int s = p % kInFlight;
        if (!mbar_wait(bar + s, (unsigned)((p / kInFlight) & 1))) timed_out = 1;
        __syncthreads();
        if (timed_out) {
            /* record the error, give the copies still in flight into this
             * block's shared memory (planes p .. p + kInFlight - 1) their
             * own bounded wait, and leave */
            if (tid == 0) {
                atomicExch(a.err, SH_ERR_TIMEOUT);
                for (int q = p + 1; q < p + kInFlight && q < nplanes; ++q)
                    mbar_wait(bar + q % kInFlight, (unsigned)((q / kInFlight) & 1));
            }
            __syncthreads();
            return;
        }
        /* stage positions of plane zb + p into ring slot p % RING */
        {
            const float *rs = raw + s * NA * slab;
            float *ys = Yr + (p % RING) * 2 * slab;
            for (int t = tid; t < ROWS * N; t += kThreads) {
                const int row = t / N, x = t - row * N;
                const int o = row * P + x;
#pragma unroll
                for (int c = 0; c < 2; ++c) {
                    float v = rs[c * slab + o];
                    if (STAGE > 0)
                        v = f32::stage_pos(v, rs[(2 + c) * slab + o], rs[(4 + c) * slab + o], cm,
                                           ck);
                    ys[c * slab + o] = v;
                }
            }
        }
        __syncthreads(); /* Y of plane zb + p visible; raw slot s consumed */
        if (tid == 0 && p + kInFlight < nplanes) issue(p + kInFlight);
        if (!compute) continue;
#pragma unroll
        for (int k = 0; k < kCellsPerThread; ++k) {
            const int qc = tid + k * kThreads;
            if (qc >= ncell) continue;
            const int row = qc / N, x = qc - row * N;
            const int xp = x + 1 < N ? x + 1 : x + 1 - N, xm = x > 0 ? x - 1 : x - 1 + N;
            const int o = (H + row) * P;
            float lap[2], pc[2];
#pragma unroll
            for (int c = 0; c < 2; ++c) {
                const float *y0p = Yr + ((p - H) % RING) * 2 * slab + c * slab; /* plane zc */
                const float *yp1 = Yr + ((p - H + 1) % RING) * 2 * slab + c * slab;
                const float *ym1 = Yr + ((p - H - 1 + RING) % RING) * 2 * slab + c * slab;
                const float u0 = y0p[o + x];
                pc[c] = u0;
                if (H == 1) {
                    lap[c] = f32::lap7(u0, y0p[o + xp], y0p[o + xm], y0p[o + P + x],
                                       y0p[o - P + x], yp1[o + x], ym1[o + x], inv_dx2);
                } else {
                    const float *yp2 = Yr + ((p - H + 2) % RING) * 2 * slab + c * slab;
                    const float *ym2 = Yr + ((p - H - 2 + RING) % RING) * 2 * slab + c * slab;
                    const int xpp = xp + 1 < N ? xp + 1 : xp + 1 - N;
                    const int xmm = xm > 0 ? xm - 1 : xm - 1 + N;
                    const float s1 = f32::ring(y0p[o + xp], y0p[o + xm], y0p[o + P + x],
                                               y0p[o - P + x], yp1[o + x], ym1[o + x]);
                    const float s2 = f32::ring(y0p[o + xpp], y0p[o + xmm], y0p[o + 2 * P + x],
                                               y0p[o - 2 * P + x], yp2[o + x], ym2[o + x]);
                    lap[c] = f32::lap13(u0, s1, s2, inv12dx2);
                }
            }
            const float v = f32::potential(pc[0], pc[1], lam, eta2, cst);
            const float k0 = f32::accel(q0[k], lap[0], pc[0], v, friction);
            const float k1 = f32::accel(q1[k], lap[1], pc[1], v, friction);
            const long long e = off + ((long long)zc * N + tl.y0 + row) * N + x;
            if (STAGE < 2) {
                a.K[STAGE][0][e] = k0;
                a.K[STAGE][1][e] = k1;
            } else {
                /* y1 = y0 + h y0' + h^2 (K0/6 + K1/3); y1' = y0' + h (K0/6 + 2K1/3 + K2/6) */
                const float dy0 = f32::dpos(q0[k], ka0[k], kb0[k], h, h2);
                const float dy1 = f32::dpos(q1[k], ka1[k], kb1[k], h, h2);
                const float dm0 = f32::dmom(ka0[k], kb0[k], k0, h);
                const float dm1 = f32::dmom(ka1[k], kb1[k], k1, h);
                float y0v = yc0[k], y1v = yc1[k], m0v = q0[k], m1v = q1[k];
                if (KAHAN) {
                    kahan_add(y0v, dy0, c0[k]);
                    kahan_add(y1v, dy1, c1[k]);
                    kahan_add(m0v, dm0, c2[k]);
                    kahan_add(m1v, dm1, c3[k]);
                    a.cy[0][e] = c0[k];
                    a.cy[1][e] = c1[k];
                    a.cm[0][e] = c2[k];
                    a.cm[1][e] = c3[k];
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

/* A bounded wait on an mbarrier that nothing completes: the timeout path of
 * the kernels above, on its own (sh_probe_wait_timeout). */
__global__ void wait_timeout_probe_kernel(int *err, unsigned long long limit_ns) {
    __shared__ unsigned long long b;
    if (threadIdx.x == 0) {
        mbar_init(&b, 1);
        fence_mbar_init();
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        const unsigned long long t0 = global_ns();
        bool done = mbar_try_wait(&b, 0);
        while (!done && global_ns() - t0 <= limit_ns) done = mbar_try_wait(&b, 0);
        atomicExch(err, done ? 0 : SH_ERR_TIMEOUT);
    }
}

} // namespace tma
} // namespace fast
} // namespace sh

#endif // SH_FAST_TMA_CUH_
