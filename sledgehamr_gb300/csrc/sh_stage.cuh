/* Stage kernels instantiated once per project (included by proj_*.cu after
 * the project's hook headers and SLEDGEHAMR_FINISH_SETUP).
 *
 * One launch evaluates the project's per-cell Rhs (plus the GW source,
 * backreaction and Kreiss-Oliger terms when enabled) on every valid cell of
 * a level and fuses the linear combination that the reference performs
 * afterwards as separate MultiFab passes:
 *
 *   RKN stage i    K_i = accel(Y_i); Y_{i+1} = y0 + c h y0' + h^2 sum a K_j
 *                  (source/integrators/rkn.cpp:57-95)
 *   RKN final      y1 = y0 + h y0' + h^2 sum bbar K; y1' = y0' + h sum b K
 *                  (rkn.cpp:97-117)
 *   SSPRK3 stages  K = f(u) + w K; u' = y0 + c K   (lsssprk3.cpp:14-31,
 *                  FillAddRhs macros.h:392-485)
 *   leapfrog       vh = v0 + dt/2 a, x1 = x0 + dt vh; v1 = vh + dt/2 a
 *                  (leapfrog.cpp:13-57)
 *
 * Thread mapping: a block of kThreads = 128 threads owns a tile of one box,
 * nx <= 32 cells wide in x (the box width when the box is narrower, so that
 * the small boxes of refined levels keep every thread busy), kThreads / nx
 * rows in y and t.nz planes in z; each thread walks its z-column, so that
 * per-thread set-up (the reciprocals of dx^2 and of the time in the hooks)
 * is paid once per column.  Hooks read the stage state
 * straight from HBM through an Array4 view of the ghost-grown box; the
 * reuse of neighbour values comes from L1.  The per-cell Rhs output is an
 * Array4 over a register array (all strides zero), which the compiler keeps
 * in registers because every component index is a compile-time constant.
 */
#ifndef SH_STAGE_CUH_
#define SH_STAGE_CUH_

#include <sledgehamr.h>

#include "sh_internal.h"

namespace sh {


/* Position/momentum pairing of the reference (rkn.cpp:32-44): user fields
 * [0, uN) pair with [uN, 2uN); with GW the tensor block [Nf, Nf+6) pairs
 * with [Nf+6, Nf+12). */
template <int NSCAL, bool GW>
struct Pairs {
    static constexpr int kUN = NSCAL / 2;
    static constexpr int kNP = kUN + (GW ? 6 : 0);
    static constexpr int kNC = NSCAL + (GW ? 12 : 0);
    __host__ __device__ static constexpr int pos(int q) {
        return q < kUN ? q : NSCAL + (q - kUN);
    }
    __host__ __device__ static constexpr int mom(int q) {
        return q < kUN ? kUN + q : NSCAL + 6 + (q - kUN);
    }
};

/* Seven resident blocks per SM (at most 72 registers) for the plain
 * stages, whose instruction mix leaves memory latency to hide (measured on
 * the AMR workload: 5 blocks 5.04 s, 6 blocks 4.67 s, 7 blocks 4.44 s, 8
 * blocks 4.39 s of stage kernels, the last with 140-224 byte spills in the
 * 13- and 19-point variants); the GW and Kreiss-Oliger variants keep every
 * register they need. */
template <bool GW, int KO>
constexpr int stage_min_blocks() {
    return (GW || KO != 0) ? 1 : 7;
}

template <class H, bool GW, int KO, bool SP = false>
__global__ void __launch_bounds__(kTileX *kTileY, (stage_min_blocks<GW, KO>()))
    stage_kernel(const __grid_constant__ StageArgs a) {
    using PR = Pairs<H::kNScalars, GW>;
    constexpr int NC = PR::kNC;
    constexpr int NP = PR::kNP;

    const TileDev t = a.tiles[blockIdx.x];
    const BoxDev b = a.boxes[t.box];
    const int tid = threadIdx.x + kTileX * threadIdx.y;
    const int ty = tid / t.nx;
    const int i = t.x0 + (tid - ty * t.nx);
    const int j = t.y0 + ty;
    if (ty >= kThreads / t.nx || i > b.hi[0] || j > b.hi[1]) return;
    const int kend = min(t.z0 + t.nz - 1, b.hi[2]);

    const long long gx = b.gdim[0];
    const long long gxy = gx * b.gdim[1];
    const long long gvol = b.gvol;
    const amrex::Dim3 glo{b.glo[0], b.glo[1], b.glo[2]};
    const amrex::Dim3 ghi{b.glo[0] + b.gdim[0], b.glo[1] + b.gdim[1], b.glo[2] + b.gdim[2]};
    const amrex::Array4<const double> st(a.state + b.off * NC, gx, gxy, gvol, glo, ghi, NC);
    /* periodic images of a cell in the ghost cells of a self-periodic box:
     * along each axis within ng of a face, the element offset of its image
     * across the domain (0 elsewhere); the cell's images are the non-empty
     * combinations of the non-zero offsets (x and y fixed per thread, z per
     * cell).  SP: the instantiation for such boxes (a.self_periodic set). */
    long long ox = 0, oy = 0;
    if constexpr (SP) {
        if (i < b.lo[0] + a.ng) ox = a.per[0];
        else if (i > b.hi[0] - a.ng) ox = -a.per[0];
        if (j < b.lo[1] + a.ng) oy = a.per[1] * gx;
        else if (j > b.hi[1] - a.ng) oy = -a.per[1] * gx;
    }

    for (int k = t.z0; k <= kend; ++k) {
        /* the epilogue's inputs of the next cell (y0 and the earlier K) asked
         * into L1 while this cell's stencil runs; the stencil's own loads
         * are left to the cache (prefetching them too measured no better) */
        if (k < kend) {
            const long long next = (i - glo.x) + (j - glo.y) * gx + (k + 1 - glo.z) * gxy;
            if (a.y0) {
#pragma unroll
                for (int n = 0; n < NC; ++n)
                    asm volatile("prefetch.global.L1 [%0];" ::"l"(a.y0 + b.off * NC + next +
                                                                 n * gvol));
            }
            /* the K buffers hold every component in the SSPRK3 stages and
             * the momenta of the pairs otherwise */
            if (a.epi == kEpiSsp0 || a.epi == kEpiSspAdd) {
                for (int s = 0; s < a.nkin; ++s)
#pragma unroll
                    for (int n = 0; n < NC; ++n)
                        asm volatile("prefetch.global.L1 [%0];" ::"l"(
                            a.kin[s] + b.off * NC + next + n * gvol));
            } else {
                for (int s = 0; s < a.nkin; ++s)
#pragma unroll
                    for (int q = 0; q < NP; ++q)
                        asm volatile("prefetch.global.L1 [%0];" ::"l"(
                            a.kin[s] + b.off * NP + next + q * gvol));
            }
        }
        double r[NC];
#pragma unroll
        for (int n = 0; n < NC; ++n) r[n] = 0.;
        const amrex::Array4<double> rhs(r, 0, 0, 1, amrex::Dim3{i, j, k},
                                        amrex::Dim3{i + 1, j + 1, k + 1}, NC);
        H::rhs(rhs, st, i, j, k, a.lev, a.time, a.dt, a.dx, a.params);
        if constexpr (GW) {
            H::gw_rhs(rhs, st, i, j, k, a.lev, a.time, a.dt, a.dx, a.gw_params);
            H::gw_backreaction(rhs, st, i, j, k, a.lev, a.time, a.dt, a.dx, a.params,
                               a.gw_params);
        }
        if constexpr (KO == 2 || KO == 3) {
            sledgehamr::utils::constexpr_for<0, NC, 1>([&](auto n) {
                r[n] += sledgehamr::kernels::KreissOligerDissipation<KO>(
                    st, i, j, k, n, a.dx, a.ko_strength[n]);
            });
        }

        const long long lc = (i - glo.x) + (j - glo.y) * gx + (k - glo.z) * gxy;
        const long long sbase = b.off * NC + lc; /* state-layout element of comp 0 */
        long long oz = 0;
        if constexpr (SP) {
            if (k < b.lo[2] + a.ng) oz = a.per[2] * gxy;
            else if (k > b.hi[2] - a.ng) oz = -a.per[2] * gxy;
        }
        switch (a.epi) {
        case kEpiPlainRhs: {
#pragma unroll
            for (int n = 0; n < NC; ++n) a.out[sbase + n * gvol] = r[n];
            break;
        }
        case kEpiRknStage: {
            const long long kb = b.off * NP + lc;
#pragma unroll
            for (int q = 0; q < NP; ++q) {
                const double kq = r[PR::mom(q)];
                a.kout[kb + q * gvol] = kq;
                double y = a.y0[sbase + PR::pos(q) * gvol];
                const double m = a.y0[sbase + PR::mom(q) * gvol];
                y += a.c_mom * m;
                for (int s = 0; s < a.nkin; ++s) y += a.c_k[s] * a.kin[s][kb + q * gvol];
                y += a.c_k[a.nkin] * kq;
                a.out[sbase + PR::pos(q) * gvol] = y;
                a.out[sbase + PR::mom(q) * gvol] = m;
            }
            break;
        }
        case kEpiRknFinal:
        case kEpiRknFinalNoKqPos: {
            /* kEpiRknFinalNoKqPos: the tableau's last bbar is zero (RKN4), so
             * the current stage's K adds nothing to the positions */
            auto final_update = [&](auto kq_pos) {
                const long long kb = b.off * NP + lc;
#pragma unroll
                for (int q = 0; q < NP; ++q) {
                    double y = a.y0[sbase + PR::pos(q) * gvol];
                    double m = a.y0[sbase + PR::mom(q) * gvol];
                    y += a.c_mom * m;
                    for (int s = 0; s < a.nkin; ++s) {
                        const double ks = a.kin[s][kb + q * gvol];
                        y += a.c_k[s] * ks;
                        m += a.c_k2[s] * ks;
                    }
                    const double kq = r[PR::mom(q)];
                    if constexpr (decltype(kq_pos)::value) y += a.c_k[a.nkin] * kq;
                    m += a.c_k2[a.nkin] * kq;
                    a.out[sbase + PR::pos(q) * gvol] = y;
                    a.out[sbase + PR::mom(q) * gvol] = m;
                }
            };
            if (a.epi == kEpiRknFinal)
                final_update(std::true_type{});
            else
                final_update(std::false_type{});
            break;
        }
        case kEpiSsp0:
        case kEpiSspAdd: {
            const long long kb = b.off * NC + lc;
#pragma unroll
            for (int n = 0; n < NC; ++n) {
                double kn = r[n];
                if (a.epi == kEpiSspAdd) kn += a.weight * a.kin[0][kb + n * gvol];
                if (a.kout) a.kout[kb + n * gvol] = kn;
                a.out[sbase + n * gvol] = 1. * a.y0[sbase + n * gvol] + a.c_out * kn;
            }
            break;
        }
        case kEpiLf0: {
            const long long kb = b.off * NP + lc;
#pragma unroll
            for (int q = 0; q < NP; ++q) {
                const double vh =
                    1. * a.y0[sbase + PR::mom(q) * gvol] + (a.dt / 2.) * r[PR::mom(q)];
                a.kout[kb + q * gvol] = vh;
                a.out[sbase + PR::pos(q) * gvol] = 1. * a.y0[sbase + PR::pos(q) * gvol] + a.dt * vh;
            }
            break;
        }
        case kEpiLf1: {
            const long long kb = b.off * NP + lc;
#pragma unroll
            for (int q = 0; q < NP; ++q) {
                a.out[sbase + PR::mom(q) * gvol] =
                    1. * a.kin[0][kb + q * gvol] + (a.dt / 2.) * r[PR::mom(q)];
                a.out[sbase + PR::pos(q) * gvol] = a.state[sbase + PR::pos(q) * gvol];
            }
            break;
        }
        default:
            break;
        }
        /* a cell within ng of a face of a self-periodic box: its stored
         * values (every component, as a fill copies them) read back and
         * written to its periodic images, out of the epilogue so that no
         * value stays live across the image stores */
        if constexpr (SP) {
            if (((ox | oy | oz) != 0) && a.epi != kEpiPlainRhs) {
#pragma unroll
                for (int n = 0; n < NC; ++n) {
                    const long long e = sbase + n * gvol;
                    const double v = a.out[e];
                    if (ox != 0) a.out[e + ox] = v;
                    if (oy != 0) {
                        a.out[e + oy] = v;
                        if (ox != 0) a.out[e + ox + oy] = v;
                    }
                    if (oz != 0) {
                        a.out[e + oz] = v;
                        if (ox != 0) a.out[e + ox + oz] = v;
                        if (oy != 0) {
                            a.out[e + oy + oz] = v;
                            if (ox != 0) a.out[e + ox + oy + oz] = v;
                        }
                    }
                }
            }
        }
    }
}

/* Tagging with the CPU semantics of SLEDGEHAMR_PRJ_TAG_WITH_TRUNCATION_CPU
 * (macros.h:489-566): mask(c) = user(c) OR (c has all-even indices AND some
 * component's TruncationModifier<n>(te) >= te_crit[n]).  The sequential
 * reference loop sets the 2x2x2 block of such an even cell and then clears
 * the seven odd cells again when it reaches them, so only the even cell
 * keeps the truncation-error tag; this kernel computes that end state
 * directly, without the racy block writes of the reference's GPU variant.
 * The counters follow the CPU statistics: total += user, and for every
 * even truncation-error cell total += 8 - user; trunc[n] += 8. */
template <class H, int NC>
__global__ void __launch_bounds__(kTileX *kTileY) tag_kernel(const __grid_constant__ TagArgs a) {
    const TileDev t = a.tiles[blockIdx.x];
    const BoxDev b = a.boxes[t.box];
    const int tid = threadIdx.x + kTileX * threadIdx.y;
    const int ty = tid / t.nx;
    const int i = t.x0 + (tid - ty * t.nx);
    const int j = t.y0 + ty;
    const bool inside = (ty < kThreads / t.nx && i <= b.hi[0] && j <= b.hi[1]);
    const int kend = min(t.z0 + t.nz - 1, b.hi[2]);
    const long long gx = b.gdim[0], gxy = gx * b.gdim[1];
    const amrex::Dim3 glo{b.glo[0], b.glo[1], b.glo[2]};
    const amrex::Dim3 ghi{b.glo[0] + b.gdim[0], b.glo[1] + b.gdim[1], b.glo[2] + b.gdim[2]};
    const amrex::Array4<const double> st(a.state + b.off * a.ncomp, gx, gxy, b.gvol, glo, ghi,
                                         a.ncomp);
    const amrex::Array4<const double> te(a.te ? a.te + b.off * a.ncomp : nullptr, gx, gxy,
                                         b.gvol, glo, ghi, a.ncomp);
    const int vx = b.hi[0] - b.lo[0] + 1, vy = b.hi[1] - b.lo[1] + 1;
    unsigned long long n_user = 0, n_total = 0;
    unsigned long long n_trunc[NC];
#pragma unroll
    for (int n = 0; n < NC; ++n) n_trunc[n] = 0;
    if (inside) {
        for (int k = t.z0; k <= kend; ++k) {
            const bool user = H::tag(st, i, j, k, a.lev, a.time, a.dt, a.dx, a.params_tag);
            bool te_res = false;
            if (a.te && (i % 2 == 0) && (j % 2 == 0) && (k % 2 == 0)) {
                sledgehamr::utils::constexpr_for<0, NC, 1>([&](auto n) {
                    const double mte = H::template te_modifier<n>(
                        st, i, j, k, a.lev, a.time, a.dt, a.dx, te(i, j, k, n), a.params_mod);
                    if (mte >= a.te_crit[n]) {
                        te_res = true;
                        n_trunc[n] += 8;
                    }
                });
            }
            n_user += user;
            n_total += user;
            if (te_res) n_total += 8 - (int)user;
            const long long m = a.mask_off[t.box] + (i - b.lo[0]) +
                                (long long)vx * ((j - b.lo[1]) + (long long)vy * (k - b.lo[2]));
            a.mask[m] = (user || te_res) ? 1 : 0;
        }
    }
    /* warp sums, one atomic per warp and counter */
    const unsigned full = 0xffffffffu;
    for (int o = 16; o > 0; o >>= 1) {
        n_user += __shfl_down_sync(full, n_user, o);
        n_total += __shfl_down_sync(full, n_total, o);
#pragma unroll
        for (int n = 0; n < NC; ++n) n_trunc[n] += __shfl_down_sync(full, n_trunc[n], o);
    }
    if ((threadIdx.x & 31) == 0) {
        if (n_total) atomicAdd(&a.counts[0], n_total);
        if (n_user) atomicAdd(&a.counts[1], n_user);
#pragma unroll
        for (int n = 0; n < NC; ++n)
            if (n_trunc[n]) atomicAdd(&a.counts[2 + n], n_trunc[n]);
    }
}

template <class H>
cudaError_t launch_stage_impl(const StageLaunch &L, cudaStream_t s) {
    if (L.ntiles <= 0) return cudaSuccess;
    dim3 block(kTileX, kTileY, 1);
    dim3 grid(L.ntiles, 1, 1);
    if (L.with_gw) {
        if constexpr (H::kHasGw) {
            switch (L.ko_order) {
            case 2: stage_kernel<H, true, 2><<<grid, block, 0, s>>>(L.args); break;
            case 3: stage_kernel<H, true, 3><<<grid, block, 0, s>>>(L.args); break;
            default:
                if (L.args.self_periodic)
                    stage_kernel<H, true, 0, true><<<grid, block, 0, s>>>(L.args);
                else
                    stage_kernel<H, true, 0><<<grid, block, 0, s>>>(L.args);
                break;
            }
        } else {
            return cudaErrorNotSupported;
        }
    } else {
        switch (L.ko_order) {
        case 2: stage_kernel<H, false, 2><<<grid, block, 0, s>>>(L.args); break;
        case 3: stage_kernel<H, false, 3><<<grid, block, 0, s>>>(L.args); break;
        default:
            if (L.args.self_periodic)
                stage_kernel<H, false, 0, true><<<grid, block, 0, s>>>(L.args);
            else
                stage_kernel<H, false, 0><<<grid, block, 0, s>>>(L.args);
            break;
        }
    }
    return cudaGetLastError();
}

template <class H>
cudaError_t launch_tag_impl(const TagArgs &a, int ntiles, cudaStream_t s) {
    if (ntiles <= 0) return cudaSuccess;
    dim3 block(kTileX, kTileY, 1);
    if (a.ncomp == H::kNScalars) {
        tag_kernel<H, H::kNScalars><<<ntiles, block, 0, s>>>(a);
    } else if (a.ncomp == H::kNScalars + 12) {
        tag_kernel<H, H::kNScalars + 12><<<ntiles, block, 0, s>>>(a);
    } else {
        return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

} // namespace sh

/* Defines the ProjectOps table `sh::project_<NAME>` for the project namespace
 * NS (after its hooks and SLEDGEHAMR_FINISH_SETUP) and registers it with the
 * library when it loads.  HAS_GW: the project
 * specialises GravitationalWavesRhs<true>; REACH: the largest neighbour
 * offset its hooks read (levels need at least that many ghost cells). */
#define SH_DEFINE_PROJECT(NAME, NS, HAS_GW, REACH)                                    \
    namespace sh {                                                             \
    struct Hooks_##NAME : NS::ShHooks {                                        \
        static constexpr bool kHasGw = HAS_GW;                                 \
    };                                                                         \
    static const char *field_name_##NAME(int c) {                              \
        const auto &f = NS::ShHooks::fields();                                 \
        return c >= 0 && c < (int)f.size() ? f[c]->name.c_str() : nullptr;    \
    }                                                                          \
    extern const ProjectOps project_##NAME;                                    \
    const ProjectOps project_##NAME = {                                        \
        #NAME,                                                                 \
        NS::ShHooks::kNScalars,                                                \
        NS::ShHooks::kNFields,                                                 \
        HAS_GW,                                                                \
        REACH,                                                                 \
        &field_name_##NAME,                                                    \
        &launch_stage_impl<Hooks_##NAME>,                                      \
        &launch_tag_impl<Hooks_##NAME>};                                       \
    static const ProjectRegistrar registrar_##NAME(&project_##NAME);          \
    }

#endif // SH_STAGE_CUH_
