/* C ABI of libsledgehamr_gb300.so (declared in include/sledgehamr_gb300.h):
 * contexts, levels, host/device data movement, periodic ghost fill, the
 * integrator drivers that sequence the fused stage kernels of
 * sh_stage.cuh, average-down (with and without truncation errors) and
 * tagging with deterministic tag-list compaction.
 */
#include "sledgehamr_gb300.h"

#include <algorithm>
#include <atomic>
#include <cstdio>
#include <mutex>
#include <cstring>
#include <new>
#include <stdexcept>
#include <string>
#include <tuple>
#include <vector>

#include "sh_bubbles.cuh"
#include "sh_out.cuh"
#include "sh_fill_plan.h"
#include "sh_fixed_stencil.h"
#include "sh_gw.h"
#include "sh_internal.h"
#include "sh_stage32.cuh"

/* ---- project registry --------------------------------------------------- */
namespace sh {
namespace registry {
std::vector<const ProjectOps *> &registered() {
    static std::vector<const ProjectOps *> v; /* filled by static initialisers */
    return v;
}
/* Ids: the built-in projects first, in the oracle's numbering; every other
 * registered project after them in name order (so that ids do not depend
 * on the order in which the linker runs the initialisers). */
const std::vector<const ProjectOps *> &table() {
    static const std::vector<const ProjectOps *> t = [] {
        static const char *const kBuiltin[] = {
            "AxionStrings",     "MinimalExample",   "NextToMinimalExample",
            "FirstOrderPhaseTransition", "AxionStringsLap1", "AxionStringsLap2",
            "AxionStringsLap3"};
        std::vector<const ProjectOps *> reg = registered(), out;
        for (const char *name : kBuiltin)
            for (const ProjectOps *p : reg)
                if (std::strcmp(p->name, name) == 0) out.push_back(p);
        std::vector<const ProjectOps *> rest;
        for (const ProjectOps *p : reg)
            if (std::find(out.begin(), out.end(), p) == out.end()) rest.push_back(p);
        std::sort(rest.begin(), rest.end(), [](const ProjectOps *a, const ProjectOps *b) {
            return std::strcmp(a->name, b->name) < 0;
        });
        out.insert(out.end(), rest.begin(), rest.end());
        return out;
    }();
    return t;
}
} // namespace registry

void register_project(const ProjectOps *p) { registry::registered().push_back(p); }
int project_count() { return (int)registry::table().size(); }
const ProjectOps *project_by_id(int id) {
    return (id >= 0 && id < project_count()) ? registry::table()[id] : nullptr;
}
} // namespace sh

using namespace sh;

/* ---- context / level structures ------------------------------------------- */
struct ProfRecord {
    int category;
    cudaEvent_t start, stop;
};
static const char *const kProfCategories[] = {"rhs",     "fill_patch",  "average_down",
                                              "tagging", "gw_spectrum", "data_move",
                                              "coarse_fine"};
enum ProfCat {
    kProfRhs = 0,
    kProfFill,
    kProfAvg,
    kProfTag,
    kProfGw,
    kProfMove,
    kProfCf,
    kProfCount
};

/* Work items of the fill kernels (one thread block each): a rectangle of
 * cells of one destination box, at most kItemCells cells, with the flat
 * offsets of its first cell (component 0) and its row / plane strides. */
constexpr int kItemCells = 512;
struct CopyItem {
    long long dst, src;     /* first cell in the dst / src buffers */
    long long dgvol, sgvol; /* component strides */
    int nx, ny, nz;
    int dsy, dsz, ssy, ssz;
};
struct CfItem {
    long long dst, dgvol;
    long long first; /* running coarse-fine cell count of the first cell */
    int dsy, dsz;
    int lo[3]; /* fine index of the first cell */
    int nx, ny, nz;
    int pad;
};

struct sh_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    cudaStream_t own_stream = nullptr;
    std::string err;
    long long launches = 0;
    /* growing device scratch for host transfers and reductions */
    void *scratch = nullptr;
    size_t scratch_bytes = 0;
    GwCache gw;
    bool profiling = false;
    std::vector<ProfRecord> prof;
    std::vector<cudaEvent_t> event_pool;
    double prof_ms[kProfCount] = {};
    long long prof_n[kProfCount] = {};
};

struct sh_level {
    long long uid = 0;     /* unique per level object of the process */
    long long version = 0; /* bumped by every call that may write the buffers */
    /* coarse-fine ghost values interpolated in space from the coarse level's
     * old and new data (cf_cells x ncomp each), valid for the coarse level
     * with uid cf_uid at version cf_ver */
    double *cf_old = nullptr, *cf_new = nullptr;
    long long cf_uid = -1, cf_ver = -1;
    /* the last ghost fill of each buffer: the level's version and the
     * coarse level's uid and version then, and the time filled for */
    struct FillSig {
        const double *buf = nullptr;
        long long ver = -1, cuid = -1, cver = -1;
        double t = 0.;
    } fill_sig[3];
    int fill_sig_next = 0;
    /* average-down plan onto the level with uid avg_for (a cache) */
    mutable long long avg_for = -1;
    mutable void *d_avg = nullptr; /* AvgRect list */
    mutable int navg = 0;
    mutable long long avg_cells = 0;
    int project = -1;
    const ProjectOps *ops = nullptr;
    bool with_gw = false;
    int ncomp = 0, npairs = 0, nghost = 0;
    int dlo[3] = {0, 0, 0}, dhi[3] = {0, 0, 0};
    std::vector<sh_box> boxes;
    std::vector<BoxDev> hboxes;
    std::vector<long long> vbase; /* prefix sums of valid cells per box */
    long long total_gvol = 0, nvalid = 0;
    BoxDev *d_boxes = nullptr;
    TileDev *d_tiles = nullptr;
    int ntiles = 0;
    CopyItem *d_ghost = nullptr; /* periodic / same-level ghost copies */
    int nghost_items = 0;
    long long nghost_cells = 0;
    long long *d_vbase = nullptr; /* nbox + 1 */
    /* SH_NEW, SH_OLD, alt.  FP32 levels (esize 4) keep FP32 values here,
     * read through f32buf(); the pointer type stays double * so that the
     * FP64 path is untouched */
    double *buf[3] = {nullptr, nullptr, nullptr};
    int esize = 8; /* 8: FP64 storage; 4: FP32 values with FP32 Kahan compensations */
    /* one box covering the periodic domain (FP64): the stage kernels without
     * Kreiss-Oliger dissipation write the periodic images of their outputs
     * into the ghost cells themselves */
    bool self_periodic = false;
    /* FP32 levels: compensations of SH_NEW / SH_OLD (the value v and its
     * compensation c stand for v - c), the truncation errors in FP64 for the
     * tag comparison (an FP64 level keeps them in its SH_OLD buffer, as the
     * reference does; an FP32 level writes them there too, for the data
     * flow of the next shadow level, and reads them from here),
     * and an FP64 copy of one buffer for the read-only operations that go
     * through the FP64 hooks and kernels (tagging, reductions, outputs) */
    float *cmp[2] = {nullptr, nullptr};
    double *te64 = nullptr;
    double *view64 = nullptr;
    double *kbuf = nullptr;  /* K buffers, kbuf_elems each */
    size_t kbuf_elems = 0;
    int kbuf_count = 0;
    double t[2] = {-1.7976931348623157e308, -1.7976931348623157e308};
    int istep[2] = {0, 0};
    /* coarse level for two-level ghost fills (nullptr: periodic single level) */
    sh_level *coarse = nullptr;
    CfItem *d_cf = nullptr; /* ghost cells interpolated from the coarse level */
    int ncf_items = 0;
    long long ncf = 0;      /* cells of those items */
    std::vector<int> owner; /* owner box of each block of owner_res cells */
    int owner_res = 1;
    int owner_nb[3] = {1, 1, 1};
    int *d_owner = nullptr;
    int lev_index = 0;    /* `lev` handed to the project hooks */
};

namespace {

struct ShError : std::runtime_error {
    int code;
    ShError(int c, const std::string &m) : std::runtime_error(m), code(c) {}
};

inline void ck(cudaError_t e, const char *what) {
    if (e != cudaSuccess)
        throw ShError(SH_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

template <class F>
int guarded(sh_ctx *ctx, F &&f) {
    try {
        f();
        return SH_OK;
    } catch (const ShError &e) {
        if (ctx) ctx->err = e.what();
        return e.code;
    } catch (const std::bad_alloc &) {
        if (ctx) ctx->err = "host allocation failed";
        return SH_ERR_NOMEM;
    } catch (const std::exception &e) {
        if (ctx) ctx->err = e.what();
        return SH_ERR_ARG;
    }
}

inline void require(bool c, const std::string &msg) {
    if (!c) throw ShError(SH_ERR_ARG, msg);
}

void *dmalloc(size_t bytes, const char *what) {
    void *p = nullptr;
    if (bytes == 0) return nullptr;
    cudaError_t e = cudaMalloc(&p, bytes);
    if (e == cudaErrorMemoryAllocation) {
        cudaGetLastError();
        throw ShError(SH_ERR_NOMEM, std::string("device allocation failed: ") + what);
    }
    ck(e, what);
    return p;
}

/* Stream-ordered allocations from the device's memory pool, for level data
 * that regrids create and destroy often: the pool keeps freed memory for
 * reuse (release threshold set at context creation), and neither the
 * allocation nor the free waits for the device. */
void *dmalloc_async(sh_ctx *ctx, size_t bytes, const char *what) {
    void *p = nullptr;
    if (bytes == 0) return nullptr;
    cudaError_t e = cudaMallocAsync(&p, bytes, ctx->stream);
    if (e == cudaErrorMemoryAllocation) {
        cudaGetLastError();
        throw ShError(SH_ERR_NOMEM, std::string("device allocation failed: ") + what);
    }
    ck(e, what);
    return p;
}

inline void dfree_async(sh_ctx *ctx, void *p) {
    if (p) cudaFreeAsync(p, ctx->stream);
}

template <class T>
T *upload_async(sh_ctx *ctx, const T *h, size_t n, const char *what) {
    if (n == 0) return nullptr;
    T *d = (T *)dmalloc_async(ctx, n * sizeof(T), what);
    ck(cudaMemcpyAsync(d, h, n * sizeof(T), cudaMemcpyHostToDevice, ctx->stream), what);
    return d;
}

void *ctx_scratch(sh_ctx *ctx, size_t bytes) {
    if (bytes > ctx->scratch_bytes) {
        if (ctx->scratch) {
            ck(cudaStreamSynchronize(ctx->stream), "sync before scratch resize");
            cudaFree(ctx->scratch);
        }
        ctx->scratch = dmalloc(bytes, "context scratch");
        ctx->scratch_bytes = bytes;
    }
    return ctx->scratch;
}

inline void set_device(sh_ctx *ctx) { ck(cudaSetDevice(ctx->device), "cudaSetDevice"); }

cudaEvent_t pooled_event(sh_ctx *ctx) {
    if (!ctx->event_pool.empty()) {
        cudaEvent_t e = ctx->event_pool.back();
        ctx->event_pool.pop_back();
        return e;
    }
    cudaEvent_t e;
    ck(cudaEventCreate(&e), "event create");
    return e;
}

/* Records CUDA events around the launches of one category while profiling. */
struct ProfScope {
    sh_ctx *ctx;
    int cat;
    cudaEvent_t a = nullptr;
    ProfScope(sh_ctx *c, int category) : ctx(c), cat(category) {
        if (ctx->profiling) {
            a = pooled_event(ctx);
            cudaEventRecord(a, ctx->stream);
        }
    }
    ~ProfScope() {
        if (a) {
            cudaEvent_t b = pooled_event(ctx);
            cudaEventRecord(b, ctx->stream);
            ctx->prof.push_back(ProfRecord{cat, a, b});
        }
    }
};

void profile_resolve(sh_ctx *ctx) {
    if (ctx->prof.empty()) return;
    ck(cudaStreamSynchronize(ctx->stream), "profile sync");
    for (const ProfRecord &r : ctx->prof) {
        float ms = 0.f;
        if (cudaEventElapsedTime(&ms, r.start, r.stop) == cudaSuccess) {
            ctx->prof_ms[r.category] += ms;
            ctx->prof_n[r.category] += 1;
        }
        ctx->event_pool.push_back(r.start);
        ctx->event_pool.push_back(r.stop);
    }
    ctx->prof.clear();
}

/* ---- data movement kernels ------------------------------------------------ */

/* Locate the box of valid cell number v (prefix sums vbase[0..nbox]). */
__device__ __forceinline__ int find_box(const long long *vbase, int nbox, long long v) {
    int lo = 0, hi = nbox - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (vbase[mid] <= v) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

/* layout 0: canonical domain array; layout 1: boxes (packed valid cells).
 * dir 0: host-side array -> level buffer; dir 1: level buffer -> array. */
template <class T>
__global__ void move_kernel(const BoxDev *boxes, const long long *vbase, int nbox, int ncomp,
                            long long nvalid, T *buf, float *cmp, double *arr, int layout,
                            int dir, int N0, int N1, int N2, int dlo0, int dlo1, int dlo2) {
    const long long total = nvalid * ncomp;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
         e += (long long)gridDim.x * blockDim.x) {
        const long long v = e % nvalid;
        const int n = (int)(e / nvalid);
        const int bx = find_box(vbase, nbox, v);
        const BoxDev &b = boxes[bx];
        const long long lv = v - vbase[bx];
        const int vx = b.hi[0] - b.lo[0] + 1, vy = b.hi[1] - b.lo[1] + 1;
        const int i = b.lo[0] + (int)(lv % vx);
        const int j = b.lo[1] + (int)((lv / vx) % vy);
        const int k = b.lo[2] + (int)(lv / ((long long)vx * vy));
        const long long bi = b.off * ncomp + (long long)n * b.gvol + (i - b.glo[0]) +
                             (long long)(j - b.glo[1]) * b.gdim[0] +
                             (long long)(k - b.glo[2]) * b.gdim[0] * b.gdim[1];
        long long ai;
        if (layout == 0)
            ai = (((long long)n * N2 + (k - dlo2)) * N1 + (j - dlo1)) * N0 + (i - dlo0);
        else
            ai = vbase[bx] * ncomp + (long long)n * (vbase[bx + 1] - vbase[bx]) + lv;
        if constexpr (sizeof(T) == 8) {
            if (dir == 0) buf[bi] = arr[ai];
            else arr[ai] = buf[bi];
        } else {
            /* FP32 value and compensation of an FP64 value x: v = fl32(x),
             * c = fl32(v - x), so that v - c is x to about 2^-48 */
            if (dir == 0) {
                const double x = arr[ai];
                const float v = (float)x;
                buf[bi] = v;
                cmp[bi] = (float)((double)v - x);
            } else {
                arr[ai] = (double)buf[bi] - (double)cmp[bi];
            }
        }
    }
}

/* FP64 copy v - c of a whole FP32 buffer (ghost cells included). */
__global__ void widen_kernel(const float *v, const float *c, double *out, long long n) {
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n;
         e += (long long)gridDim.x * blockDim.x)
        out[e] = (double)v[e] - (c ? (double)c[e] : 0.);
}

/* Copies of rectangles of cells (ghost fill from the same level, periodic
 * images, or level-to-level copies): one thread block per item (at most
 * kItemCells = 512 cells), threads over its cells (x fastest), all
 * components.  Cell t is split into (i, j, k) with FP32 reciprocals of nx
 * and nx*ny taken once per item instead of integer divisions per cell: for
 * t < 512 the product (t + 1/2) * (1/m) is within 512 * 2^-23 of
 * (t + 1/2) / m, whose distance to the nearest integer is at least
 * 1/(2m) >= 2^-10, so the truncation is exact (checked for every item
 * shape).  dst and src may be the same buffer (ghost fill): the cells
 * written (ghost cells) are never read by the same launch, so the
 * pointers are restrict-qualified and each thread loads two cells' four
 * components before it stores any (measured against one cell, and against
 * four cells at 128 registers, which lost occupancy). */
constexpr int kItemThreads = 128; /* threads per item of the copy and combine kernels */
template <class T>
__global__ void copy_items_kernel(const CopyItem *__restrict__ items, T *__restrict__ dst,
                                  const T *__restrict__ src, int ncomp) {
    const CopyItem it = items[blockIdx.x];
    const int nxy = it.nx * it.ny;
    const int n = nxy * it.nz;
    const float inv_nx = 1.f / (float)it.nx, inv_nxy = 1.f / (float)nxy;
    auto offsets = [&](int t, long long &d, long long &s) {
        const int k = (int)(((float)t + 0.5f) * inv_nxy);
        const int r = t - k * nxy;
        const int j = (int)(((float)r + 0.5f) * inv_nx);
        const int i = r - j * it.nx;
        d = it.dst + i + (long long)j * it.dsy + (long long)k * it.dsz;
        s = it.src + i + (long long)j * it.ssy + (long long)k * it.ssz;
    };
    /* two cells of four components in flight: loaded before any is stored */
    for (int t0 = threadIdx.x; t0 < n; t0 += 2 * blockDim.x) {
        const int t1 = t0 + blockDim.x;
        const bool two = t1 < n;
        long long d0, s0, d1 = 0, s1 = 0;
        offsets(t0, d0, s0);
        if (two) offsets(t1, d1, s1);
        for (int c0 = 0; c0 < ncomp; c0 += 4) {
            T v0[4], v1[4];
#pragma unroll
            for (int c = 0; c < 4; ++c) {
                if (c0 + c >= ncomp) continue;
                v0[c] = __ldg(src + s0 + (c0 + c) * it.sgvol);
                if (two) v1[c] = __ldg(src + s1 + (c0 + c) * it.sgvol);
            }
#pragma unroll
            for (int c = 0; c < 4; ++c) {
                if (c0 + c >= ncomp) continue;
                dst[d0 + (c0 + c) * it.dgvol] = v0[c];
                if (two) dst[d1 + (c0 + c) * it.dgvol] = v1[c];
            }
        }
    }
}


/* Block map of a level: owner box of every aligned block of `res` cells
 * (-1 where no box). */
struct OwnerMapDev {
    const int *owner;
    int res;
    int nb[3];
    int dlo[3];
    int ext[3];
};

/* The children of one coarse parent from the 19 coarse values of src
 * around index `base` (x stride 1, y stride cx, z stride cxy), evaluated
 * exactly in 64-bit integers: every weight of the quadratic interpolation
 * below is a multiple of 1/64 (u000: 52, the face neighbours 2 +- 8 s_d,
 * the edge neighbours +-1 s_d s_e), so each child is an integer
 * combination of the values written as multiples of 2^(A-3-1075)
 * (sh_fixed_stencil.h, A their largest exponent), rounded once to FP64.
 * The partial sums stay below 124 * 2^56 < 2^63.  Returns false (and writes
 * nothing) when a value is not finite; the FP64 formula then runs. */
template <class T, class Put>
__device__ __forceinline__ bool cf_children_fixed(const T *src, long long base, long long cx,
                                                  long long cxy, const int P[3], const int c0[3],
                                                  const int c1[3], Put &put) {
    namespace fx = sledgehamr::utils::fixed;
    const long long off[19] = {0,
                               1, -1, cx, -cx, cxy, -cxy,
                               1 + cx, 1 - cx, -1 + cx, -1 - cx,
                               1 + cxy, 1 - cxy, -1 + cxy, -1 - cxy,
                               cx + cxy, cx - cxy, -cx + cxy, -cx - cxy};
    double v[19];
#pragma unroll
    for (int q = 0; q < 19; ++q) v[q] = (double)src[base + off[q]];
    int hi[19];
    const int A = fx::anchor(v, hi);
    if (A == 0x7FF) return false;
    long long t[19];
#pragma unroll
    for (int q = 0; q < 19; ++q) t[q] = fx::to_fixed<3>(hi[q], fx::lo_word(v[q]), A);
    const long long S = 52 * t[0] + 2 * (t[1] + t[2] + t[3] + t[4] + t[5] + t[6]);
    const long long Ex = 8 * (t[1] - t[2]), Ey = 8 * (t[3] - t[4]), Ez = 8 * (t[5] - t[6]);
    const long long Fxy = t[7] - t[8] - t[9] + t[10];
    const long long Fxz = t[11] - t[12] - t[13] + t[14];
    const long long Fyz = t[15] - t[16] - t[17] + t[18];
    const int pw = A - 3 - 1075 - 6;
    for (int fk = c0[2]; fk <= c1[2]; ++fk) {
        const bool zp = (fk - 2 * P[2]) != 0;
        for (int fj = c0[1]; fj <= c1[1]; ++fj) {
            const bool yp = (fj - 2 * P[1]) != 0;
            const long long yz = S + (yp ? Ey : -Ey) + (zp ? Ez : -Ez) + (yp == zp ? Fyz : -Fyz);
            const long long slope = Ex + (yp ? Fxy : -Fxy) + (zp ? Fxz : -Fxz);
            for (int fi = c0[0]; fi <= c1[0]; ++fi)
                put(fi, fj, fk, fx::to_double((fi - 2 * P[0]) ? yz + slope : yz - slope, pw));
        }
    }
    return true;
}

/* Quadratic (CellQuadratic) interpolation of fine cells from the 3x3x3
 * coarse cells around their parent, after linear interpolation in time
 * between the coarse old and new data (mode 0: old only, 1: new only,
 * 2: alpha old + beta new).  With u_abc the coarse values at offsets
 * a, b, c in {-1, 0, 1} and xi = -1/4 or +1/4 the fine-cell centre offset
 * in coarse units per axis:
 *   u = u000 + sum_d xi_d D_d + 1/2 sum_d xi_d^2 D_dd + sum_{d<e} xi_d xi_e D_de
 * with D_d = (u_+ - u_-)/2, D_dd = u_+ - 2 u_0 + u_-, and
 * D_de = (u_++ - u_+- - u_-+ + u_--)/4 in the plane of d and e.
 * One thread per coarse parent: the 19 coarse values and the differences
 * are formed once and evaluated for each of its children inside the item
 * (xi_d^2 = 1/16 for every child, so the second-order term is shared).
 * The parent (periodically wrapped) is found through the coarse level's
 * block map; its neighbours are read from the parent box's ghost cells. */
template <class T>
__global__ void cf_interp_kernel(const CfItem *items, const BoxDev *cboxes, T *fbuf,
                                 OwnerMapDev cmap, const T *c_old, const T *c_new, int mode,
                                 double alpha, double beta, int ncomp, T *store, long long ncf,
                                 float *fcmp) {
    const CfItem it = items[blockIdx.x];
    auto fl2 = [](int a) { return a >= 0 ? a / 2 : -((-a + 1) / 2); };
    const int lo[3] = {it.lo[0], it.lo[1], it.lo[2]};
    const int hi[3] = {it.lo[0] + it.nx - 1, it.lo[1] + it.ny - 1, it.lo[2] + it.nz - 1};
    int plo[3], pn[3];
    for (int d = 0; d < 3; ++d) {
        plo[d] = fl2(lo[d]);
        pn[d] = fl2(hi[d]) - plo[d] + 1;
    }
    const int np = pn[0] * pn[1] * pn[2];
    for (int q = threadIdx.x; q < np; q += blockDim.x) {
        const int P[3] = {plo[0] + q % pn[0], plo[1] + (q / pn[0]) % pn[1],
                          plo[2] + q / (pn[0] * pn[1])};
        int W[3], c0[3], c1[3];
        for (int d = 0; d < 3; ++d) {
            int w = (P[d] - cmap.dlo[d]) % cmap.ext[d];
            if (w < 0) w += cmap.ext[d];
            W[d] = cmap.dlo[d] + w;
            c0[d] = max(2 * P[d], lo[d]);
            c1[d] = min(2 * P[d] + 1, hi[d]);
        }
        const int cbox = cmap.owner[((long long)((W[2] - cmap.dlo[2]) / cmap.res) * cmap.nb[1] +
                                     (W[1] - cmap.dlo[1]) / cmap.res) *
                                        cmap.nb[0] +
                                    (W[0] - cmap.dlo[0]) / cmap.res];
        if (cbox < 0) continue; /* excluded by the host's coverage check */
        const BoxDev &cb = cboxes[cbox];
        const long long cx = cb.gdim[0], cxy = cx * cb.gdim[1];
        const long long cbase = cb.off * ncomp + (W[0] - cb.glo[0]) + (W[1] - cb.glo[1]) * cx +
                                (W[2] - cb.glo[2]) * cxy;
        for (int nn = 0; nn < ncomp; ++nn) {
            const long long base = cbase + nn * cb.gvol;
            /* FP32 levels interpolate in FP32 (no FP32/FP64 conversions,
             * which GB300 runs at the FP64 rate), FP64 levels in FP64 */
            using A = T;
            auto put = [&](int fi, int fj, int fk, A v) {
                if (store) {
                    store[it.first + (fi - lo[0]) +
                          (long long)it.nx * ((fj - lo[1]) + (long long)it.ny * (fk - lo[2])) +
                          nn * ncf] = (T)v;
                } else {
                    const long long d = it.dst + (fi - lo[0]) + (long long)(fj - lo[1]) * it.dsy +
                                        (long long)(fk - lo[2]) * it.dsz + nn * it.dgvol;
                    fbuf[d] = (T)v;
                    /* FP32 levels: a cell filled for good starts without compensation */
                    if (fcmp) fcmp[d] = 0.f;
                }
            };
            if constexpr (sizeof(T) == 8) {
                if (mode != 2 && cf_children_fixed(mode == 0 ? c_old : c_new, base, cx, cxy, P,
                                                   c0, c1, put))
                    continue;
            }
            const A al = (A)alpha, be = (A)beta;
            auto u = [&](int a, int b2, int d) -> A {
                const long long e = base + a + b2 * cx + d * cxy;
                if (mode == 0) return c_old[e];
                if (mode == 1) return c_new[e];
                return al * c_old[e] + be * c_new[e];
            };
            const A half = (A)0.5, quarter = (A)0.25, sixteenth = (A)0.0625, two = (A)2.;
            const A u0 = u(0, 0, 0);
            const A dxp = u(1, 0, 0), dxm = u(-1, 0, 0);
            const A dyp = u(0, 1, 0), dym = u(0, -1, 0);
            const A dzp = u(0, 0, 1), dzm = u(0, 0, -1);
            const A Dx = (dxp - dxm) * half, Dy = (dyp - dym) * half, Dz = (dzp - dzm) * half;
            const A Dxx = dxp - two * u0 + dxm;
            const A Dyy = dyp - two * u0 + dym;
            const A Dzz = dzp - two * u0 + dzm;
            const A Dxy = (u(1, 1, 0) - u(1, -1, 0) - u(-1, 1, 0) + u(-1, -1, 0)) * quarter;
            const A Dxz = (u(1, 0, 1) - u(1, 0, -1) - u(-1, 0, 1) + u(-1, 0, -1)) * quarter;
            const A Dyz = (u(0, 1, 1) - u(0, 1, -1) - u(0, -1, 1) + u(0, -1, -1)) * quarter;
            /* every child has xi_d^2 = 1/16: with s_d = +-1,
             * u = S + sum_d s_d E_d + sum_{d<e} s_d s_e F_de,
             * S = u000 + (Dxx + Dyy + Dzz)/32, E_d = D_d/4, F_de = D_de/16 */
            const A S = u0 + half * (sixteenth * Dxx + sixteenth * Dyy + sixteenth * Dzz);
            const A Ex = quarter * Dx, Ey = quarter * Dy, Ez = quarter * Dz;
            const A Fxy = sixteenth * Dxy, Fxz = sixteenth * Dxz, Fyz = sixteenth * Dyz;
            for (int fk = c0[2]; fk <= c1[2]; ++fk) {
                const bool zp = (fk - 2 * P[2]) != 0;
                for (int fj = c0[1]; fj <= c1[1]; ++fj) {
                    const bool yp = (fj - 2 * P[1]) != 0;
                    /* the part without x, and the coefficient of s_x */
                    const A fyz = (yp == zp) ? Fyz : -Fyz;
                    const A base = S + (yp ? Ey : -Ey) + (zp ? Ez : -Ez) + fyz;
                    const A slope = Ex + (yp ? Fxy : -Fxy) + (zp ? Fxz : -Fxz);
                    for (int fi = c0[0]; fi <= c1[0]; ++fi)
                        put(fi, fj, fk, (fi - 2 * P[0]) ? base + slope : base - slope);
                }
            }
        }
    }
}

/* Coarse-fine ghost cells from the stored spatial interpolations of the
 * coarse old and new data: the interpolation is linear in the coarse data,
 * so interpolating alpha old + beta new equals alpha I(old) + beta I(new). */
template <class T>
__global__ void cf_combine_kernel(const CfItem *__restrict__ items, T *__restrict__ fbuf,
                                  const T *__restrict__ i_old, const T *__restrict__ i_new,
                                  int mode, double alpha, double beta, int ncomp,
                                  long long ncf) {
    const CfItem it = items[blockIdx.x];
    const int nxy = it.nx * it.ny;
    const int n = nxy * it.nz;
    const float inv_nx = 1.f / (float)it.nx, inv_nxy = 1.f / (float)nxy;
    for (int q = threadIdx.x; q < n; q += blockDim.x) {
        /* exact for q < kItemCells (see copy_items_kernel) */
        const int k = (int)(((float)q + 0.5f) * inv_nxy);
        const int r = q - k * nxy;
        const int j = (int)(((float)r + 0.5f) * inv_nx);
        const int i = r - j * it.nx;
        const long long d = it.dst + i + (long long)j * it.dsy + (long long)k * it.dsz;
        const long long c = it.first + q;
        /* four components in flight: loaded before any is stored */
        for (int c0 = 0; c0 < ncomp; c0 += 4) {
            /* in the storage type: FP32 levels combine in FP32 */
            T v[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                if (c0 + u >= ncomp) continue;
                const long long e = c + (c0 + u) * ncf;
                if (mode == 0) v[u] = __ldg(i_old + e);
                else if (mode == 1) v[u] = __ldg(i_new + e);
                else v[u] = (T)alpha * __ldg(i_old + e) + (T)beta * __ldg(i_new + e);
            }
#pragma unroll
            for (int u = 0; u < 4; ++u)
                if (c0 + u < ncomp) fbuf[d + (c0 + u) * it.dgvol] = v[u];
        }
    }
}

/* The output function of every valid cell into a P^3 array (x fastest). */
__global__ void out_pack_kernel(const BoxDev *boxes, const long long *vbase, int nbox,
                                long long nvalid, int ncomp, int fn, int comp, const double *buf,
                                double *dst, int P, int dlo0, int dlo1, int dlo2) {
    for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < nvalid;
         v += (long long)gridDim.x * blockDim.x) {
        const int bx = find_box(vbase, nbox, v);
        const BoxDev &b = boxes[bx];
        const long long lv = v - vbase[bx];
        const int vx = b.hi[0] - b.lo[0] + 1, vy = b.hi[1] - b.lo[1] + 1;
        const int i = b.lo[0] + (int)(lv % vx);
        const int j = b.lo[1] + (int)((lv / vx) % vy);
        const int k = b.lo[2] + (int)(lv / ((long long)vx * vy));
        const long long c = b.off * ncomp + (i - b.glo[0]) +
                            (long long)(j - b.glo[1]) * b.gdim[0] +
                            (long long)(k - b.glo[2]) * b.gdim[0] * b.gdim[1];
        dst[((long long)(k - dlo2) * P + (j - dlo1)) * P + (i - dlo0)] =
            out_function(fn, comp, buf + c, b.gvol);
    }
}

/* One level of a projection. */
struct ProjLevel {
    OwnerMapDev map;
    const BoxDev *boxes;
    const double *buf;
    int ncomp, dimN;
};
constexpr int kMaxProjLevels = 8;
struct ProjArgs {
    ProjLevel lev[kMaxProjLevels];
    int nlev, fn, comp, mode, dimN;
};

__device__ __forceinline__ int owner_at(const OwnerMapDev &m, int i, int j, int k) {
    return m.owner[((long long)((k - m.dlo[2]) / m.res) * m.nb[1] + (j - m.dlo[1]) / m.res) *
                       m.nb[0] +
                   (i - m.dlo[0]) / m.res];
}

/* One thread per pixel (x, y) of the finest level: levels in order, along z
 * in increasing k, the cells of each level that exist there and are not
 * covered by the next level (the order in which the reference's loops over
 * z-sorted boxes reach the pixel). */
__global__ void projection_kernel(const __grid_constant__ ProjArgs a, double *data, int *nproj) {
    const long long npix = (long long)a.dimN * a.dimN;
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < npix;
         p += (long long)gridDim.x * blockDim.x) {
        const int X = (int)(p / a.dimN), Y = (int)(p % a.dimN);
        double acc = 0.;
        int cnt = 0;
        for (int l = 0; l < a.nlev; ++l) {
            const ProjLevel &L = a.lev[l];
            const int ratio = a.dimN / L.dimN;
            const int i = X / ratio, j = Y / ratio;
            for (int k = 0; k < L.dimN; ++k) {
                const int own = owner_at(L.map, i, j, k);
                if (own < 0) {
                    k += L.map.res - 1 - (k % L.map.res); /* skip the block */
                    continue;
                }
                if (l + 1 < a.nlev && owner_at(a.lev[l + 1].map, 2 * i, 2 * j, 2 * k) >= 0)
                    continue;
                const BoxDev &b = L.boxes[own];
                const long long c = b.off * L.ncomp + (i - b.glo[0]) +
                                    (long long)(j - b.glo[1]) * b.gdim[0] +
                                    (long long)(k - b.glo[2]) * b.gdim[0] * b.gdim[1];
                const double val = out_function(a.fn, a.comp, L.buf + c, b.gvol);
                if (a.mode == 0) acc = __dadd_rn(acc, __dmul_rn((double)ratio, val));
                else acc = fmax(acc, val);
                ++cnt;
            }
        }
        data[p] = acc;
        nproj[p] = cnt;
    }
}

/* Bubble injection on the valid cells of a level (sh_level_add_bubbles). */
/* FP32 levels (T = float): the bubbles are added to the FP64 values v - c
 * and the sums stored as value and compensation again. */
template <class T>
__global__ void level_bubbles_kernel(const BoxDev *boxes, const long long *vbase, int nbox,
                                     long long nvalid, int ncomp, int cphi, int cdphi,
                                     T *buf, float *cmp, BubbleList bl, double dx, double L) {
    for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < nvalid;
         v += (long long)gridDim.x * blockDim.x) {
        const int bx = find_box(vbase, nbox, v);
        const BoxDev &b = boxes[bx];
        const long long lv = v - vbase[bx];
        const int vx = b.hi[0] - b.lo[0] + 1, vy = b.hi[1] - b.lo[1] + 1;
        const int i = b.lo[0] + (int)(lv % vx);
        const int j = b.lo[1] + (int)((lv / vx) % vy);
        const int k = b.lo[2] + (int)(lv / ((long long)vx * vy));
        const long long c = b.off * ncomp + (i - b.glo[0]) +
                            (long long)(j - b.glo[1]) * b.gdim[0] +
                            (long long)(k - b.glo[2]) * b.gdim[0] * b.gdim[1];
        const long long ep = c + cphi * b.gvol, ed = c + cdphi * b.gvol;
        double phi = buf[ep], dphi = buf[ed];
        if constexpr (sizeof(T) == 4) {
            phi -= cmp[ep];
            dphi -= cmp[ed];
        }
        add_bubbles_at(bl, i, j, k, dx, L, phi, dphi);
        buf[ep] = (T)phi;
        buf[ed] = (T)dphi;
        if constexpr (sizeof(T) == 4) {
            cmp[ep] = (float)((double)buf[ep] - phi);
            cmp[ed] = (float)((double)buf[ed] - dphi);
        }
    }
}

/* One rectangle of coarse cells [lo, hi] lying in coarse box cbox and under
 * fine box fbox. */
struct AvgRect {
    int fbox, cbox;
    int lo[3], hi[3];
    long long first;
};

/* Plain average-down (k, j, i summation order) or, with te != nullptr, the
 * average-down with truncation error of kernels::AverageDownWithTruncationError
 * (summation order (0,0,0) (1,0,0) (0,1,0) (0,0,1) (1,1,0) (1,0,1) (0,1,1)
 * (1,1,1)). */
/* Reductions of one component over the valid cells of a level
 * (sh_level_reduce).  One block per box: thread t combines the box's cells
 * t, t + 256, ... in order, then a fixed tree over the block gives the
 * box's partial; a single block combines the partials in box order the same
 * way.  The order of every FP64 addition is fixed, so sums are
 * deterministic. */
constexpr int kReduceThreads = 256;

__device__ __forceinline__ double reduce_identity(int op) {
    if (op == SH_REDUCE_MIN) return __longlong_as_double(0x7FF0000000000000ll);  /* +inf */
    if (op == SH_REDUCE_MAX) return __longlong_as_double((long long)0xFFF0000000000000ull); /* -inf */
    return 0.;
}
/* v: the cell's value of comp; w: of comp + 1 (SH_REDUCE_SUM_MODULUS) */
__device__ __forceinline__ double reduce_value(int op, double v, double w) {
    if (op == SH_REDUCE_MAX_ABS) return fabs(v);
    if (op == SH_REDUCE_SUM_SQ) return v * v;
    if (op == SH_REDUCE_COUNT_NONFINITE) return isfinite(v) ? 0. : 1.;
    if (op == SH_REDUCE_SUM_MODULUS) return sqrt(v * v + w * w);
    return v;
}
__device__ __forceinline__ double reduce_combine(int op, double a, double b) {
    if (op == SH_REDUCE_MAX_ABS || op == SH_REDUCE_MAX) return b > a ? b : a;
    if (op == SH_REDUCE_MIN) return b < a ? b : a;
    return a + b;
}
__device__ double reduce_block(int op, double acc) {
    __shared__ double sm[kReduceThreads];
    sm[threadIdx.x] = acc;
    __syncthreads();
    for (int w = kReduceThreads / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) sm[threadIdx.x] = reduce_combine(op, sm[threadIdx.x], sm[threadIdx.x + w]);
        __syncthreads();
    }
    return sm[0];
}

__global__ void __launch_bounds__(kReduceThreads)
    reduce_boxes_kernel(const BoxDev *boxes, const double *buf, int ncomp, int comp, int op,
                        double *partial) {
    const BoxDev b = boxes[blockIdx.x];
    const int nx = b.hi[0] - b.lo[0] + 1, ny = b.hi[1] - b.lo[1] + 1;
    const int n = nx * ny * (b.hi[2] - b.lo[2] + 1);
    const long long gx = b.gdim[0], gxy = gx * b.gdim[1];
    const double *base = buf + b.off * ncomp + (long long)comp * b.gvol +
                         (b.lo[0] - b.glo[0]) + (b.lo[1] - b.glo[1]) * gx +
                         (b.lo[2] - b.glo[2]) * gxy;
    const double *base2 = op == SH_REDUCE_SUM_MODULUS ? base + b.gvol : base;
    double acc = reduce_identity(op);
    for (int t = threadIdx.x; t < n; t += kReduceThreads) {
        const int i = t % nx, r = t / nx;
        const int j = r % ny, k = r / ny;
        const long long e = i + j * gx + k * gxy;
        acc = reduce_combine(op, acc, reduce_value(op, base[e], base2[e]));
    }
    const double v = reduce_block(op, acc);
    if (threadIdx.x == 0) partial[blockIdx.x] = v;
}

__global__ void __launch_bounds__(kReduceThreads)
    reduce_final_kernel(const double *partial, int n, int op, double *out) {
    double acc = reduce_identity(op);
    for (int t = threadIdx.x; t < n; t += kReduceThreads)
        acc = reduce_combine(op, acc, partial[t]);
    const double v = reduce_block(op, acc);
    if (threadIdx.x == 0) out[0] = v;
}

/* FP32 levels (T = float): the fine values are read as v - c with their
 * compensations fc, the average is formed in FP64 and stored as a value and
 * compensation (cc), the truncation error goes to an FP64 array. */
template <class T>
__global__ void avgdown_kernel(const AvgRect *rects, int nrects, long long ncells,
                               const BoxDev *fboxes, const BoxDev *cboxes, int ncomp,
                               const T *fine, const float *fc, T *crse, float *cc, double *te,
                               T *te_old, float *te_old_c) {
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < ncells;
         c += (long long)gridDim.x * blockDim.x) {
        int lo = 0, hi = nrects - 1;
        while (lo < hi) {
            int mid = (lo + hi + 1) >> 1;
            if (rects[mid].first <= c) lo = mid;
            else hi = mid - 1;
        }
        const AvgRect &r = rects[lo];
        const long long lc = c - r.first;
        const int nx = r.hi[0] - r.lo[0] + 1, ny = r.hi[1] - r.lo[1] + 1;
        const int i = r.lo[0] + (int)(lc % nx);
        const int j = r.lo[1] + (int)((lc / nx) % ny);
        const int k = r.lo[2] + (int)(lc / ((long long)nx * ny));
        const BoxDev &fb = fboxes[r.fbox];
        const BoxDev &cb = cboxes[r.cbox];
        const long long fx = fb.gdim[0], fxy = fx * fb.gdim[1];
        const long long f0 = fb.off * ncomp + (2 * i - fb.glo[0]) + (2 * j - fb.glo[1]) * fx +
                             (2 * k - fb.glo[2]) * fxy;
        const long long c0 = cb.off * ncomp + (i - cb.glo[0]) +
                             (long long)(j - cb.glo[1]) * cb.gdim[0] +
                             (long long)(k - cb.glo[2]) * cb.gdim[0] * cb.gdim[1];
        if constexpr (sizeof(T) == 4) {
            /* The sum of the eight children's v - c in FP32 pairs (hi, lo)
             * with error-free TwoSum steps, about 48 bits, without the
             * FP32/FP64 conversions that GB300 runs at the FP64 rate; the
             * average is (hi, lo) / 8 (exact), stored as value hi and
             * compensation -lo.  The truncation error is formed the same
             * way and widened to FP64 once. */
            auto two_sum = [](float a, float b, float &err) {
                const float s = __fadd_rn(a, b);
                const float bb = __fsub_rn(s, a);
                err = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
                return s;
            };
            for (int n = 0; n < ncomp; ++n) {
                const long long fo = f0 + n * fb.gvol;
                float hi = 0.f, lo = 0.f, e;
                for (int dk = 0; dk < 2; ++dk)
                    for (int dj = 0; dj < 2; ++dj)
                        for (int di = 0; di < 2; ++di) {
                            const long long q = fo + di + dj * fx + dk * fxy;
                            hi = two_sum(hi, fine[q], e);
                            lo = __fadd_rn(lo, e);
                            hi = two_sum(hi, -fc[q], e);
                            lo = __fadd_rn(lo, e);
                        }
                hi = two_sum(hi, lo, lo);
                hi = __fmul_rn(hi, 0.125f);
                lo = __fmul_rn(lo, 0.125f);
                const long long co = c0 + n * cb.gvol;
                if (te) {
                    /* (v_c - c_c) - (hi + lo) */
                    const float d = two_sum(crse[co], -hi, e);
                    const float r = __fadd_rn(e, __fsub_rn(-cc[co], lo));
                    const double tev = fabs((double)d + (double)r);
                    te[fo] = tev;
                    /* and into the fine level's old buffer, where the
                     * reference keeps it (the next shadow level averages
                     * that buffer down) */
                    const float tv = (float)tev;
                    te_old[fo] = tv;
                    te_old_c[fo] = (float)((double)tv - tev);
                }
                crse[co] = hi;
                cc[co] = -lo;
            }
            continue;
        } else
        for (int n = 0; n < ncomp; ++n) {
            const double *f = fine + f0 + n * fb.gvol;
            if (te) {
                double s = f[0];
                s += f[1];
                s += f[fx];
                s += f[fxy];
                s += f[1 + fx];
                s += f[1 + fxy];
                s += f[fx + fxy];
                s += f[1 + fx + fxy];
                const double avg = 0.125 * s;
                double *cc = crse + c0 + n * cb.gvol;
                te[f0 + n * fb.gvol] = fabs(*cc - avg);
                *cc = avg;
            } else {
                double s = 0.0;
                for (int dk = 0; dk < 2; ++dk)
                    for (int dj = 0; dj < 2; ++dj)
                        for (int di = 0; di < 2; ++di) s += f[di + dj * fx + dk * fxy];
                crse[c0 + n * cb.gvol] = s * 0.125;
            }
        }
    }
}

/* Tag-list compaction, pass 1: tagged cells per chunk of kChunk mask bytes. */
constexpr int kChunk = 4096;
__global__ void tag_count_kernel(const unsigned char *mask, long long n, int *chunk_counts) {
    const long long base = (long long)blockIdx.x * kChunk;
    int cnt = 0;
    for (int q = threadIdx.x; q < kChunk; q += blockDim.x) {
        long long e = base + q;
        if (e < n) cnt += mask[e] != 0;
    }
    for (int o = 16; o > 0; o >>= 1) cnt += __shfl_down_sync(0xffffffffu, cnt, o);
    __shared__ int ws[32];
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = cnt;
    __syncthreads();
    if (threadIdx.x == 0) {
        int s = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += ws[w];
        chunk_counts[blockIdx.x] = s;
    }
}
/* pass 2: exclusive scan of the chunk counts (one block). */
__global__ void tag_scan_kernel(int *chunk_counts, int nchunks, long long *chunk_base,
                                long long *total) {
    __shared__ long long carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int start = 0; start < nchunks; start += blockDim.x) {
        const int idx = start + threadIdx.x;
        long long v = idx < nchunks ? chunk_counts[idx] : 0;
        /* inclusive block scan via warp shuffles */
        const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
        long long x = v;
        for (int o = 1; o < 32; o <<= 1) {
            long long y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        __shared__ long long wsum[32];
        if (lane == 31) wsum[warp] = x;
        __syncthreads();
        if (warp == 0) {
            long long w = lane < (int)(blockDim.x >> 5) ? wsum[lane] : 0;
            for (int o = 1; o < 32; o <<= 1) {
                long long y = __shfl_up_sync(0xffffffffu, w, o);
                if (lane >= o) w += y;
            }
            wsum[lane] = w;
        }
        __syncthreads();
        const long long incl = x + (warp > 0 ? wsum[warp - 1] : 0);
        if (idx < nchunks) chunk_base[idx] = carry + incl - v;
        __syncthreads();
        if (threadIdx.x == blockDim.x - 1) carry += incl;
        __syncthreads();
    }
    if (threadIdx.x == 0) *total = carry;
}
/* pass 3: write the indices of tagged cells in ascending order; within a
 * chunk, warps take 32-byte slices in order and use ballots for their
 * offsets. */
__global__ void tag_write_kernel(const unsigned char *mask, long long n,
                                 const long long *chunk_base, int *list, long long capacity) {
    const long long base = (long long)blockIdx.x * kChunk;
    __shared__ int warp_tot[32];
    __shared__ long long running;
    if (threadIdx.x == 0) running = chunk_base[blockIdx.x];
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int slab = 0; slab < kChunk; slab += blockDim.x) {
        const long long e = base + slab + threadIdx.x;
        const bool t = (slab + threadIdx.x < kChunk) && e < n && mask[e] != 0;
        const unsigned bal = __ballot_sync(0xffffffffu, t);
        if (lane == 0) warp_tot[warp] = __popc(bal);
        __syncthreads();
        long long off = running;
        for (int w = 0; w < warp; ++w) off += warp_tot[w];
        if (t) {
            const long long pos = off + __popc(bal & ((1u << lane) - 1u));
            if (pos < capacity) list[pos] = (int)e;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            long long s = 0;
            for (int w = 0; w < nw; ++w) s += warp_tot[w];
            running += s;
        }
        __syncthreads();
    }
}

/* Buffered tags coarsened to blocks: every tagged valid cell marks the
 * blocks of `block` cells (periodically wrapped, nb per side) that its
 * neighbourhood [i - buffer, i + buffer]^3 touches.  Concurrent writes
 * store the same value. */
__global__ void tag_blocks_kernel(const BoxDev *boxes, const long long *vbase, int nbox,
                                  long long nvalid, const unsigned char *mask, int dlo0, int dlo1,
                                  int dlo2, int block, int buffer, int nb,
                                  unsigned char *blocks) {
    auto fdiv = [](int a, int b) { return a >= 0 ? a / b : -((-a + b - 1) / b); };
    auto pmod = [](int a, int n) {
        const int r = a % n;
        return r < 0 ? r + n : r;
    };
    for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < nvalid;
         v += (long long)gridDim.x * blockDim.x) {
        if (!mask[v]) continue;
        const int bx = find_box(vbase, nbox, v);
        const BoxDev &b = boxes[bx];
        const long long lv = v - vbase[bx];
        const int vx = b.hi[0] - b.lo[0] + 1, vy = b.hi[1] - b.lo[1] + 1;
        const int c[3] = {b.lo[0] + (int)(lv % vx) - dlo0,
                          b.lo[1] + (int)((lv / vx) % vy) - dlo1,
                          b.lo[2] + (int)(lv / ((long long)vx * vy)) - dlo2};
        int b0[3], b1[3];
        for (int d = 0; d < 3; ++d) {
            b0[d] = fdiv(c[d] - buffer, block);
            b1[d] = fdiv(c[d] + buffer, block);
        }
        for (int z = b0[2]; z <= b1[2]; ++z)
            for (int y = b0[1]; y <= b1[1]; ++y)
                for (int x = b0[0]; x <= b1[0]; ++x)
                    blocks[((long long)pmod(z, nb) * nb + pmod(y, nb)) * nb + pmod(x, nb)] = 1;
    }
}

int grid_for(long long work, int block = 256) {
    long long g = (work + block - 1) / block;
    if (g < 1) g = 1;
    if (g > 152LL * 32) g = 152LL * 32;
    return (int)g;
}

/* ---- level construction ------------------------------------------------- */

bool box_intersect(const int alo[3], const int ahi[3], const int blo[3], const int bhi[3],
                   int lo[3], int hi[3]) {
    for (int d = 0; d < 3; ++d) {
        lo[d] = std::max(alo[d], blo[d]);
        hi[d] = std::min(ahi[d], bhi[d]);
        if (lo[d] > hi[d]) return false;
    }
    return true;
}

/* Owner map of a level: blocks of `res` cells, res = the largest size that
 * divides the domain and every box bound (boxes are unions of blocks). */
void build_owner_map(sh_ctx *ctx, sh_level *L) {
    OwnerMap m;
    try {
        sh::build_owner_map(L->dlo, L->dhi, L->boxes.data(), (int)L->boxes.size(), m);
    } catch (const PlanError &e) {
        throw ShError(SH_ERR_ARG, e.what());
    }
    L->owner.swap(m.owner);
    L->owner_res = m.res;
    for (int d = 0; d < 3; ++d) L->owner_nb[d] = m.nb[d];
    L->d_owner = upload_async(ctx, L->owner.data(), L->owner.size(), "owner map");
}

OwnerMapDev owner_map_dev(const sh_level *L) {
    OwnerMapDev m;
    m.owner = L->d_owner;
    m.res = L->owner_res;
    for (int d = 0; d < 3; ++d) {
        m.nb[d] = L->owner_nb[d];
        m.dlo[d] = L->dlo[d];
        m.ext[d] = L->dhi[d] - L->dlo[d] + 1;
    }
    return m;
}

/* The fill planning of sh_fill_plan.h on the levels' host metadata; its
 * errors become SH_ERR_ARG. */
PlanLevel plan_level(const sh_level *L) {
    PlanLevel p;
    for (int d = 0; d < 3; ++d) {
        p.dlo[d] = L->dlo[d];
        p.dhi[d] = L->dhi[d];
        p.owner_nb[d] = L->owner_nb[d];
    }
    p.boxes = L->boxes.data();
    p.nbox = (int)L->boxes.size();
    p.nghost = L->nghost;
    p.ncomp = L->ncomp;
    p.owner = L->owner.data();
    p.owner_res = L->owner_res;
    return p;
}

FillPlan build_fill_plan(const sh_level *D, const sh_level *S, const sh_level *C,
                         bool ghosts_only, bool want_copies = true) {
    const PlanLevel d = plan_level(D);
    const PlanLevel s = S ? plan_level(S) : PlanLevel{};
    const PlanLevel c = C ? plan_level(C) : PlanLevel{};
    try {
        return sh::build_fill_plan(d, S == D ? &d : (S ? &s : nullptr), C ? &c : nullptr,
                                   ghosts_only, want_copies);
    } catch (const PlanError &e) {
        throw ShError(SH_ERR_ARG, e.what());
    }
}

/* Splits the rectangle [lo, hi] into pieces of at most kItemCells cells
 * (whole planes, else whole rows, else row segments). */
template <class F>
void split_rect(const int lo[3], const int hi[3], F &&emit) {
    const int nx = hi[0] - lo[0] + 1, ny = hi[1] - lo[1] + 1, nz = hi[2] - lo[2] + 1;
    if ((long long)nx * ny <= kItemCells) {
        const int pz = std::max(1, kItemCells / (nx * ny));
        for (int z = 0; z < nz; z += pz)
            emit(lo[0], lo[1], lo[2] + z, nx, ny, std::min(pz, nz - z));
    } else if (nx <= kItemCells) {
        const int py = std::max(1, kItemCells / nx);
        for (int z = 0; z < nz; ++z)
            for (int y = 0; y < ny; y += py)
                emit(lo[0], lo[1] + y, lo[2] + z, nx, std::min(py, ny - y), 1);
    } else {
        for (int z = 0; z < nz; ++z)
            for (int y = 0; y < ny; ++y)
                for (int x = 0; x < nx; x += kItemCells)
                    emit(lo[0] + x, lo[1] + y, lo[2] + z, std::min(kItemCells, nx - x), 1, 1);
    }
}

/* Number of pieces split_rect makes of [lo, hi]. */
inline long long split_count(const int lo[3], const int hi[3]) {
    const long long nx = hi[0] - lo[0] + 1, ny = hi[1] - lo[1] + 1, nz = hi[2] - lo[2] + 1;
    if (nx * ny <= kItemCells) {
        const long long pz = std::max<long long>(1, kItemCells / (nx * ny));
        return (nz + pz - 1) / pz;
    }
    if (nx <= kItemCells) {
        const long long py = std::max<long long>(1, kItemCells / nx);
        return nz * ((ny + py - 1) / py);
    }
    return nz * ny * ((nx + kItemCells - 1) / kItemCells);
}

/* Items of all rectangles, in rectangle order, made by host threads:
 * make(rect, x, y, z, nx, ny, nz, cells of the rectangle's earlier pieces). */
template <class Item, class Rect, class Make>
std::vector<Item> expand_items(const std::vector<Rect> &rects, Make make) {
    const long long n = (long long)rects.size();
    std::vector<long long> off(n + 1, 0);
    for (long long q = 0; q < n; ++q) off[q + 1] = off[q] + split_count(rects[q].lo, rects[q].hi);
    std::vector<Item> items((size_t)off[n]);
#pragma omp parallel for schedule(dynamic, 256)
    for (long long q = 0; q < n; ++q) {
        long long at = off[q], before = 0;
        split_rect(rects[q].lo, rects[q].hi, [&](int x, int y, int z, int nx, int ny, int nz) {
            items[at++] = make(rects[q], x, y, z, nx, ny, nz, before);
            before += (long long)nx * ny * nz;
        });
    }
    return items;
}

inline long long cell_offset(const BoxDev &b, int ncomp, int i, int j, int k) {
    return b.off * ncomp + (i - b.glo[0]) + (long long)(j - b.glo[1]) * b.gdim[0] +
           (long long)(k - b.glo[2]) * b.gdim[0] * b.gdim[1];
}

std::vector<CopyItem> copy_items(const std::vector<GhostCopyDev> &rects, const sh_level *D,
                                 const sh_level *S) {
    return expand_items<CopyItem>(
        rects, [&](const GhostCopyDev &r, int x, int y, int z, int nx, int ny, int nz, long long) {
            const BoxDev &db = D->hboxes[r.dbox];
            const BoxDev &sb = S->hboxes[r.sbox];
            CopyItem it;
            it.dst = cell_offset(db, D->ncomp, x, y, z);
            it.src = cell_offset(sb, S->ncomp, x - r.shift[0], y - r.shift[1], z - r.shift[2]);
            it.dgvol = db.gvol;
            it.sgvol = sb.gvol;
            it.nx = nx;
            it.ny = ny;
            it.nz = nz;
            it.dsy = db.gdim[0];
            it.dsz = db.gdim[0] * db.gdim[1];
            it.ssy = sb.gdim[0];
            it.ssz = sb.gdim[0] * sb.gdim[1];
            return it;
        });
}

std::vector<CfItem> cf_items(const std::vector<CfRect> &rects, const sh_level *D) {
    return expand_items<CfItem>(
        rects, [&](const CfRect &r, int x, int y, int z, int nx, int ny, int nz, long long before) {
            const BoxDev &db = D->hboxes[r.dbox];
            CfItem it;
            it.first = r.first + before;
            it.dst = cell_offset(db, D->ncomp, x, y, z);
            it.dgvol = db.gvol;
            it.dsy = db.gdim[0];
            it.dsz = db.gdim[0] * db.gdim[1];
            it.lo[0] = x;
            it.lo[1] = y;
            it.lo[2] = z;
            it.nx = nx;
            it.ny = ny;
            it.nz = nz;
            it.pad = 0;
            return it;
        });
}

template <class T>
T *upload_items(sh_ctx *ctx, const std::vector<T> &v, const char *what) {
    return upload_async(ctx, v.data(), v.size(), what);
}

void build_ghost_plan(sh_ctx *ctx, sh_level *L) {
    FillPlan P = build_fill_plan(L, L, nullptr, true);
    const std::vector<CopyItem> items = copy_items(P.rects, L, L);
    L->nghost_items = (int)items.size();
    L->nghost_cells = P.rect_cells;
    L->d_ghost = upload_items(ctx, items, "ghost plan");
}

/* GetLevelData time selection (level_synchronizer.cpp:613-632) for data of
 * level C at time t; mode 0 old, 1 new, 2 both with weights. */
void coarse_time_weights(const sh_level *C, double t, int &mode, double &alpha, double &beta) {
    const double tn = C->t[SH_NEW], to = C->t[SH_OLD];
    const double teps = std::fabs(tn - to) * 1.e-3;
    alpha = 0.;
    beta = 0.;
    if (t > tn - teps && t < tn + teps) {
        mode = 1;
    } else if (t > to - teps && t < to + teps) {
        mode = 0;
    } else {
        mode = 2;
        alpha = (tn - t) / (tn - to);
        beta = (t - to) / (tn - to);
    }
}

void level_free(sh_ctx *ctx, sh_level *L) {
    dfree_async(ctx, L->d_boxes);
    dfree_async(ctx, L->d_tiles);
    dfree_async(ctx, L->d_ghost);
    dfree_async(ctx, L->d_vbase);
    dfree_async(ctx, L->d_cf);
    dfree_async(ctx, L->d_owner);
    dfree_async(ctx, L->d_avg);
    dfree_async(ctx, L->cf_old);
    dfree_async(ctx, L->cf_new);
    for (int q = 0; q < 3; ++q) dfree_async(ctx, L->buf[q]);
    dfree_async(ctx, L->kbuf);
    dfree_async(ctx, L->cmp[0]);
    dfree_async(ctx, L->cmp[1]);
    dfree_async(ctx, L->te64);
    dfree_async(ctx, L->view64);
}

/* An FP64 view of buffer `which` of L for read-only work through the FP64
 * kernels and hooks: the buffer itself on an FP64 level; on an FP32 level
 * v - c of every element (ghost cells included) in the level's FP64 copy,
 * valid until the next call of this function on L. */
const double *state64(sh_ctx *ctx, const sh_level *L, int which) {
    if (L->esize == 8) return L->buf[which];
    sh_level *Lm = const_cast<sh_level *>(L);
    const long long n = L->total_gvol * L->ncomp;
    if (!Lm->view64) Lm->view64 = (double *)dmalloc_async(ctx, n * sizeof(double), "FP64 view");
    widen_kernel<<<grid_for(n), 256, 0, ctx->stream>>>(
        (const float *)L->buf[which], which == SH_NEW || which == SH_OLD ? L->cmp[which] : nullptr,
        Lm->view64, n);
    ctx->launches++;
    ck(cudaGetLastError(), "FP64 view launch");
    return Lm->view64;
}

/* The truncation errors of L (FP64 levels: its old buffer). */
const double *te_of(const sh_level *L) { return L->esize == 8 ? L->buf[SH_OLD] : L->te64; }

inline void require_fp64(const sh_level *L, const char *what) {
    if (L->esize != 8)
        throw ShError(SH_ERR_UNSUPPORTED, std::string(what) + " needs an FP64 level");
}

void ensure_kbuf(sh_ctx *ctx, sh_level *L, size_t elems, int count) {
    if (elems * count <= L->kbuf_elems * L->kbuf_count && elems <= L->kbuf_elems) return;
    dfree_async(ctx, L->kbuf);
    L->kbuf = nullptr;
    L->kbuf = (double *)dmalloc_async(ctx, elems * count * sizeof(double),
                                      "integrator K buffers");
    L->kbuf_elems = elems;
    L->kbuf_count = count;
}

/* FillPatch / FillIntermediatePatch of one buffer of L at time t: ghost
 * cells from the valid cells of the same level (periodic images), then, on a
 * fine level linked to its coarse level, the remaining ghost cells from the
 * coarse data at time t. */
/* Records that buf's ghost cells were filled for time t with the level at
 * its current version and the coarse level as it is now. */
void note_fill(sh_level *L, const double *buf, double t) {
    int q = 0;
    while (q < 3 && L->fill_sig[q].buf != buf) ++q;
    if (q == 3) {
        q = L->fill_sig_next;
        L->fill_sig_next = (q + 1) % 3;
    }
    L->fill_sig[q].buf = buf;
    L->fill_sig[q].ver = L->version;
    L->fill_sig[q].cuid = L->coarse ? L->coarse->uid : -1;
    L->fill_sig[q].cver = L->coarse ? L->coarse->version : -1;
    L->fill_sig[q].t = t;
}

/* Whether buf's ghost cells already hold what a fill for time t would
 * write: filled for t while the level was at version ver and the coarse
 * level (if any) at its present version. */
bool fill_current(const sh_level *L, const double *buf, double t, long long ver) {
    for (const auto &f : L->fill_sig)
        if (f.buf == buf)
            return f.ver == ver && f.t == t && f.cuid == (L->coarse ? L->coarse->uid : -1) &&
                   f.cver == (L->coarse ? L->coarse->version : -1);
    return false;
}

template <class T>
void fill_patch_t(sh_ctx *ctx, sh_level *L, T *buf, double t, int nfill) {
    if (L->nghost_items > 0) {
        ProfScope ps(ctx, kProfFill);
        copy_items_kernel<T><<<L->nghost_items, kItemThreads, 0, ctx->stream>>>(L->d_ghost, buf,
                                                                              buf, nfill);
        ctx->launches++;
        ck(cudaGetLastError(), "ghost fill launch");
    }
    if (L->coarse && L->ncf_items > 0) {
        ProfScope ps(ctx, kProfCf);
        const sh_level *C = L->coarse;
        if (L->cf_uid != C->uid || L->cf_ver != C->version) {
            /* spatial interpolation of the coarse old and new data, once per
             * coarse data version (every fine sub-step and stage between two
             * coarse steps reuses it) */
            if (!L->cf_old) {
                const size_t bytes = (size_t)L->ncf * L->ncomp * sizeof(T);
                L->cf_old = (double *)dmalloc_async(ctx, bytes, "coarse-fine values");
                L->cf_new = (double *)dmalloc_async(ctx, bytes, "coarse-fine values");
            }
            for (int m = 0; m < 2; ++m) {
                cf_interp_kernel<T><<<L->ncf_items, 128, 0, ctx->stream>>>(
                    L->d_cf, C->d_boxes, nullptr, owner_map_dev(C), (const T *)C->buf[SH_OLD],
                    (const T *)C->buf[SH_NEW], m, 0., 0., L->ncomp,
                    (T *)(m == 0 ? L->cf_old : L->cf_new), L->ncf, nullptr);
                ctx->launches++;
            }
            L->cf_uid = C->uid;
            L->cf_ver = C->version;
        }
        int mode;
        double alpha, beta;
        coarse_time_weights(C, t, mode, alpha, beta);
        cf_combine_kernel<T><<<L->ncf_items, kItemThreads, 0, ctx->stream>>>(
            L->d_cf, buf, (const T *)L->cf_old, (const T *)L->cf_new, mode, alpha, beta, nfill,
            L->ncf);
        ctx->launches++;
        ck(cudaGetLastError(), "coarse-fine fill launch");
    }
}

/* FP32 levels store floats behind the double pointers of their buffers
 * (and of the coarse-fine value caches): same layout, element size 4. */
void fill_patch(sh_ctx *ctx, sh_level *L, double *buf, double t) {
    if (L->esize == 4) fill_patch_t<float>(ctx, L, (float *)buf, t, L->ncomp);
    else fill_patch_t<double>(ctx, L, buf, t, L->ncomp);
    note_fill(L, buf, t);
}

/* The ghost cells of the first nfill components of an FP32 stage buffer,
 * not recorded as a fill of the buffer. */
void fill_patch_stage(sh_ctx *ctx, sh_level *L, double *buf, double t, int nfill) {
    fill_patch_t<float>(ctx, L, (float *)buf, t, nfill);
}

void launch_stage(sh_ctx *ctx, sh_level *L, StageArgs &a, int ko_order) {
    a.tiles = L->d_tiles;
    a.boxes = L->d_boxes;
    a.ncomp = L->ncomp;
    ProfScope ps(ctx, kProfRhs);
    StageLaunch sl;
    sl.args = a;
    sl.ntiles = L->ntiles;
    sl.with_gw = L->with_gw;
    sl.ko_order = ko_order;
    cudaError_t e = L->ops->launch_stage(sl, ctx->stream);
    if (e == cudaErrorNotSupported)
        throw ShError(SH_ERR_UNSUPPORTED, "project has no gravitational-wave hooks");
    ck(e, "stage kernel launch");
    ctx->launches++;
}

void fill_common(StageArgs &a, const sh_level *L, double dt, double dx, const double *params,
                 int nparams, const double *gw_params, int ngw, int ko_order,
                 const double *ko_strength) {
    require(nparams >= 0 && nparams <= kMaxParams, "at most 32 Rhs parameters");
    require(ngw >= 0 && ngw <= kMaxGwParams, "at most 16 GW parameters");
    require(ko_order == 0 || ko_order == 2 || ko_order == 3, "ko_order must be 0, 2 or 3");
    require(ko_order == 0 || ko_strength != nullptr, "ko_strength required");
    require(L->nghost >= ko_order, "nghost smaller than the dissipation stencil");
    std::memset(&a, 0, sizeof(a));
    a.dt = dt;
    a.dx = dx;
    a.self_periodic = (L->self_periodic && ko_order == 0) ? 1 : 0;
    a.ng = L->nghost;
    for (int d = 0; d < 3; ++d) a.per[d] = L->dhi[d] - L->dlo[d] + 1;
    for (int q = 0; q < nparams; ++q) a.params[q] = params[q];
    for (int q = 0; q < ngw; ++q) a.gw_params[q] = gw_params[q];
    if (ko_order)
        for (int n = 0; n < L->ncomp; ++n) a.ko_strength[n] = ko_strength[n];
}

struct Tableau {
    std::vector<double> nodes, bbar, b;
    std::vector<std::vector<double>> a;
};

/* source/integrators/rkn.cpp:130-152 */
Tableau rkn_tableau(int type, const double *flat, int s) {
    Tableau t;
    if (type == SH_INTEGRATOR_RKN4) {
        t.nodes = {0.0, 0.5, 1.0};
        t.a = {{0.0}, {1. / 8., 0.0}, {0.0, 0.5, 0.0}};
        t.bbar = {1. / 6., 1. / 3., 0.0};
        t.b = {1. / 6., 4. / 6., 1. / 6.};
    } else if (type == SH_INTEGRATOR_RKN5) {
        t.nodes = {0.0, 1. / 5., 2. / 3., 1.0};
        t.a = {{0.0}, {1. / 50., 0.0}, {-1. / 27., 7. / 27., 0.0},
               {3. / 10., -2. / 35., 9. / 35., 0.0}};
        t.bbar = {14. / 336., 100. / 336., 54. / 336., 0.0};
        t.b = {14. / 336., 125. / 336., 162. / 336., 35. / 336.};
    } else {
        require(flat != nullptr && s >= 1 && s <= kMaxStages, "user tableau: 1..8 stages");
        t.nodes.assign(flat, flat + s);
        t.bbar.assign(flat + s, flat + 2 * s);
        t.b.assign(flat + 2 * s, flat + 3 * s);
        const double *tri = flat + 3 * s;
        for (int i = 0; i < s; ++i) {
            t.a.emplace_back(tri, tri + i + 1);
            tri += i + 1;
            require(t.a.back().back() == 0.0, "RKN tableau must be explicit");
        }
    }
    return t;
}

/* Integrate old -> new with the fused stage kernels.  Buffers: 0 = new,
 * 1 = old, 2 = alt; stage states alternate between new and alt. */
/* The ghost cells of a stage's output buffer for time t: where the stage
 * kernel wrote them itself (periodic images, a.self_periodic), only the fill
 * is recorded; otherwise FillIntermediatePatch. */
void after_stage(sh_ctx *ctx, sh_level *L, const StageArgs &a, double *buf, double t) {
    if (a.self_periodic) note_fill(L, buf, t);
    else fill_patch(ctx, L, buf, t);
}

void integrate(sh_ctx *ctx, sh_level *L, int type, const double *tableau, int nstages,
               double dt, double dx, const double *params, int nparams, const double *gw_params,
               int ngw, int ko_order, const double *ko_strength) {
    const double t0 = L->t[SH_OLD];
    const size_t kelems = (size_t)L->total_gvol * L->ncomp;
    StageArgs a;
    fill_common(a, L, dt, dx, params, nparams, gw_params, ngw, ko_order, ko_strength);
    a.y0 = L->buf[SH_OLD];
    a.nk = L->npairs;
    a.lev = L->lev_index;

    if (type == SH_INTEGRATOR_RKN4 || type == SH_INTEGRATOR_RKN5 ||
        type == SH_INTEGRATOR_RKN_TABLEAU) {
        Tableau tb = rkn_tableau(type, tableau, nstages);
        const int S = (int)tb.b.size();
        ensure_kbuf(ctx, L, (size_t)L->total_gvol * L->npairs, S);
        double *kb[kMaxStages];
        for (int s = 0; s < S; ++s) kb[s] = L->kbuf + (size_t)s * L->total_gvol * L->npairs;
        int cur = SH_OLD; /* buffer holding Y_i */
        for (int i = 0; i < S; ++i) {
            StageArgs s = a;
            s.state = L->buf[cur];
            s.time = t0 + dt * tb.nodes[i];
            const int next = (cur == SH_NEW) ? 2 : SH_NEW;
            s.out = L->buf[next];
            /* earlier K with a zero coefficient (RKN4: a_31) would add an
             * exact zero for finite data: they are left out of the stage's
             * list, so their buffers are not read */
            s.nkin = 0;
            if (i < S - 1) {
                s.epi = kEpiRknStage;
                s.kout = kb[i];
                s.c_mom = dt * tb.nodes[i + 1];
                for (int j = 0; j < i; ++j)
                    if (tb.a[i + 1][j] != 0.) {
                        s.kin[s.nkin] = kb[j];
                        s.c_k[s.nkin++] = dt * dt * tb.a[i + 1][j];
                    }
                s.c_k[s.nkin] = dt * dt * tb.a[i + 1][i];
            } else {
                s.epi = kEpiRknFinal;
                s.kout = nullptr;
                s.c_mom = dt;
                for (int j = 0; j < S - 1; ++j)
                    if (tb.bbar[j] != 0. || tb.b[j] != 0.) {
                        s.kin[s.nkin] = kb[j];
                        s.c_k[s.nkin] = dt * dt * tb.bbar[j];
                        s.c_k2[s.nkin++] = dt * tb.b[j];
                    }
                s.c_k[s.nkin] = dt * dt * tb.bbar[S - 1];
                s.c_k2[s.nkin] = dt * tb.b[S - 1];
                if (tb.bbar[S - 1] == 0.) s.epi = kEpiRknFinalNoKqPos;
            }
            launch_stage(ctx, L, s, ko_order);
            after_stage(ctx, L, a, L->buf[next], i < S - 1 ? t0 + dt * tb.nodes[i + 1] : t0 + dt);
            cur = next;
        }
        if (cur != SH_NEW) std::swap(L->buf[SH_NEW], L->buf[2]);
    } else if (type == SH_INTEGRATOR_LSSSPRK3) {
        ensure_kbuf(ctx, L, kelems, 1);
        StageArgs s = a;
        /* k1 = f(y0); u1 = y0 + dt k1 */
        s.state = L->buf[SH_OLD];
        s.time = t0;
        s.epi = kEpiSsp0;
        s.kout = L->kbuf;
        s.c_out = dt;
        s.out = L->buf[SH_NEW];
        launch_stage(ctx, L, s, ko_order);
        after_stage(ctx, L, a, L->buf[SH_NEW], t0 + dt);
        /* k1 = f(u1) + k1; u2 = y0 + dt/4 k1 */
        s.state = L->buf[SH_NEW];
        s.time = t0 + dt;
        s.epi = kEpiSspAdd;
        s.weight = 1.;
        s.kin[0] = L->kbuf;
        s.nkin = 1;
        s.kout = L->kbuf;
        s.c_out = dt / 4.;
        s.out = L->buf[2];
        launch_stage(ctx, L, s, ko_order);
        after_stage(ctx, L, a, L->buf[2], t0 + dt / 2.);
        /* k1 = f(u2) + k1/4; y1 = y0 + 2dt/3 k1 */
        s.state = L->buf[2];
        s.time = t0 + dt / 2.;
        s.weight = 0.25;
        s.kout = nullptr;
        s.c_out = dt * 2. / 3.;
        s.out = L->buf[SH_NEW];
        launch_stage(ctx, L, s, ko_order);
        after_stage(ctx, L, a, L->buf[SH_NEW], t0 + dt);
    } else if (type == SH_INTEGRATOR_LEAPFROG) {
        ensure_kbuf(ctx, L, (size_t)L->total_gvol * L->npairs, 1);
        StageArgs s = a;
        s.state = L->buf[SH_OLD];
        s.time = t0;
        s.epi = kEpiLf0;
        s.kout = L->kbuf;
        s.out = L->buf[SH_NEW];
        launch_stage(ctx, L, s, ko_order);
        after_stage(ctx, L, a, L->buf[SH_NEW], t0 + dt);
        s.state = L->buf[SH_NEW];
        s.time = t0 + dt;
        s.epi = kEpiLf1;
        s.kin[0] = L->kbuf;
        s.nkin = 1;
        s.kout = nullptr;
        s.out = L->buf[2];
        launch_stage(ctx, L, s, ko_order);
        after_stage(ctx, L, a, L->buf[2], t0 + dt);
        std::swap(L->buf[SH_NEW], L->buf[2]);
    } else if (type >= 0 && type <= 4) {
        throw ShError(SH_ERR_UNSUPPORTED, "AMReX integrators (types 0-4) are not supported");
    } else {
        throw ShError(SH_ERR_ARG, "unknown integrator type " + std::to_string(type));
    }
}

/* The projects whose FP32 levels have stage kernels (sh_stage32.cuh):
 * 1, 2 the axion strings with the 7- / 13-point Laplacian (RKN4), 3
 * FirstOrderPhaseTransition (leapfrog); else 0. */
constexpr int kFam32Fopt = 3;
int stage32_family(const ProjectOps *ops) {
    if (!ops || !ops->name) return 0;
    if (std::strcmp(ops->name, "AxionStringsLap1") == 0) return 1;
    if (std::strcmp(ops->name, "AxionStringsLap2") == 0) return 2;
    if (std::strcmp(ops->name, "FirstOrderPhaseTransition") == 0) return kFam32Fopt;
    return 0;
}

/* One leapfrog step of an FP32 FirstOrderPhaseTransition level (the old
 * buffer's ghost cells filled): the drift writes the new positions, whose
 * ghost cells are then filled at t + dt, and the second kick the new
 * momenta in place beside them. */
void integrate32_fopt(sh_ctx *ctx, sh_level *L, int type, double dt, double dx,
                      const double *params, int nparams) {
    require(type == SH_INTEGRATOR_LEAPFROG,
            "FP32 FirstOrderPhaseTransition levels integrate with the leapfrog (type 11)");
    require(params && nparams >= 4 && params[0] == 0.,
            "FP32 FirstOrderPhaseTransition levels take the pure potential (params[0] = 0, "
            "params[1..3] = q2, q3, q4)");
    const int np = L->npairs;
    ensure_kbuf(ctx, L, (size_t)L->total_gvol * np, 1); /* vh and its compensation, FP32 */
    Stage32FoptArgs a;
    std::memset(&a, 0, sizeof(a));
    a.tiles = L->d_tiles;
    a.boxes = L->d_boxes;
    a.y0 = (const float *)L->buf[SH_OLD];
    a.c_old = L->cmp[SH_OLD];
    a.out = (float *)L->buf[SH_NEW];
    a.c_new = L->cmp[SH_NEW];
    a.kv = (float *)L->kbuf;
    a.kc = a.kv + (size_t)L->total_gvol * np;
    a.inv12dx2 = (float)(1. / (12. * dx * dx));
    a.inv12dx = (float)(1. / (12. * dx));
    a.hdt = (float)(0.5 * dt);
    a.dt = (float)dt;
    a.q2 = (float)params[1];
    a.q3 = (float)params[2];
    a.q4 = (float)params[3];
    const double t0 = L->t[SH_OLD];
    dim3 block(kTileX, kTileY, 1);
    for (int st = 0; st < 2; ++st) {
        a.state = (const float *)(st == 0 ? L->buf[SH_OLD] : L->buf[SH_NEW]);
        if (L->ntiles > 0) {
            ProfScope ps(ctx, kProfRhs);
            if (L->with_gw) {
                if (st == 0) stage32_fopt_kernel<0, true><<<L->ntiles, block, 0, ctx->stream>>>(a);
                else stage32_fopt_kernel<1, true><<<L->ntiles, block, 0, ctx->stream>>>(a);
            } else {
                if (st == 0) stage32_fopt_kernel<0, false><<<L->ntiles, block, 0, ctx->stream>>>(a);
                else stage32_fopt_kernel<1, false><<<L->ntiles, block, 0, ctx->stream>>>(a);
            }
            ctx->launches++;
            ck(cudaGetLastError(), "FP32 stage kernel launch");
        }
        if (st == 0) fill_patch_stage(ctx, L, L->buf[SH_NEW], t0 + dt, L->ncomp);
        else fill_patch(ctx, L, L->buf[SH_NEW], t0 + dt);
    }
}

/* One RKN4 step of an FP32 level (the old buffer's ghost cells filled):
 * the stage schedule of integrate() with the FP32 axion kernels; the stage
 * buffers' ghost cells are filled at the stage times between launches.
 * Stage 0 writes Y1 into SH_NEW, stage 1 Y2 into the third buffer (the
 * positions only, whose ghost cells are filled), the last stage y1 into
 * SH_NEW with its compensations. */
void integrate32(sh_ctx *ctx, sh_level *L, int type, double dt, double dx,
                 const double *params, int nparams, int ko_order) {
    require(type == SH_INTEGRATOR_RKN4, "FP32 levels integrate with RKN4 (type 21)");
    require(ko_order == 0, "FP32 levels have no Kreiss-Oliger dissipation");
    require(params && nparams >= 2, "FP32 axion levels need the parameters (lambda, c)");
    const int order = stage32_family(L->ops);
    require(order != 0, "no FP32 stage kernel for this project");
    ensure_kbuf(ctx, L, (size_t)L->total_gvol, 2); /* two K of 2 FP32 components */
    float *k0 = (float *)L->kbuf, *k1 = k0 + (size_t)L->total_gvol * 2;
    const double t0 = L->t[SH_OLD];
    Stage32Args a;
    std::memset(&a, 0, sizeof(a));
    a.tiles = L->d_tiles;
    a.boxes = L->d_boxes;
    a.y0 = (const float *)L->buf[SH_OLD];
    a.k0 = k0;
    a.k1 = k1;
    a.c_old = L->cmp[SH_OLD];
    a.c_new = L->cmp[SH_NEW];
    a.h = (float)dt;
    a.h2 = (float)(dt * dt);
    const float inv_dx2 = (float)(1. / (dx * dx));
    a.inv = order == 1 ? inv_dx2 : inv_dx2 / 12.f;
    a.lam = (float)params[0];
    a.cst = (float)params[1];
    double *const src[3] = {L->buf[SH_OLD], L->buf[SH_NEW], L->buf[2]};
    double *const dst[3] = {L->buf[SH_NEW], L->buf[2], L->buf[SH_NEW]};
    const double node[3] = {0., 0.5, 1.};
    for (int st = 0; st < 3; ++st) {
        const double ts = t0 + dt * node[st];
        a.state = (const float *)src[st];
        a.out = (float *)dst[st];
        a.friction = (float)(-2. / ts);
        a.eta2 = (float)(ts * ts);
        a.kout = st == 0 ? k0 : (st == 1 ? k1 : nullptr);
        a.cm = (float)(st == 0 ? 0.5 * dt : dt);
        a.ck = (float)(st == 0 ? dt * dt / 8. : dt * dt / 2.);
        {
            ProfScope ps(ctx, kProfRhs);
            if (L->ntiles > 0) {
                dim3 block(kTileX, kTileY, 1);
#define SH_STAGE32(O, S) stage32_axion_kernel<O, S><<<L->ntiles, block, 0, ctx->stream>>>(a)
                if (order == 1) {
                    if (st == 0) SH_STAGE32(1, 0);
                    else if (st == 1) SH_STAGE32(1, 1);
                    else SH_STAGE32(1, 2);
                } else {
                    if (st == 0) SH_STAGE32(2, 0);
                    else if (st == 1) SH_STAGE32(2, 1);
                    else SH_STAGE32(2, 2);
                }
#undef SH_STAGE32
                ctx->launches++;
                ck(cudaGetLastError(), "FP32 stage kernel launch");
            }
        }
        if (st < 2)
            fill_patch_stage(ctx, L, dst[st], t0 + dt * node[st + 1], 2);
        else
            fill_patch(ctx, L, dst[st], t0 + dt);
    }
}

void move(sh_ctx *ctx, const sh_level *L, int which, double *arr, int layout, int dir) {
    require(layout == 0 || layout == 1, "layout must be 0 (canonical) or 1 (boxes)");
    if (layout == 0) {
        long long dv = 1;
        for (int d = 0; d < 3; ++d) dv *= (L->dhi[d] - L->dlo[d] + 1);
        require(dv == L->nvalid, "canonical layout needs boxes covering the whole domain");
    }
    const long long work = L->nvalid * L->ncomp;
    ProfScope ps(ctx, kProfMove);
    const int n0 = L->dhi[0] - L->dlo[0] + 1, n1 = L->dhi[1] - L->dlo[1] + 1,
              n2 = L->dhi[2] - L->dlo[2] + 1;
    if (L->esize == 4) {
        require(which == SH_NEW || which == SH_OLD, "FP32 levels move their two time levels");
        move_kernel<float><<<grid_for(work), 256, 0, ctx->stream>>>(
            L->d_boxes, L->d_vbase, (int)L->boxes.size(), L->ncomp, L->nvalid,
            (float *)L->buf[which], L->cmp[which], arr, layout, dir, n0, n1, n2, L->dlo[0],
            L->dlo[1], L->dlo[2]);
    } else {
        move_kernel<double><<<grid_for(work), 256, 0, ctx->stream>>>(
            L->d_boxes, L->d_vbase, (int)L->boxes.size(), L->ncomp, L->nvalid, L->buf[which],
            nullptr, arr, layout, dir, n0, n1, n2, L->dlo[0], L->dlo[1], L->dlo[2]);
    }
    ctx->launches++;
    ck(cudaGetLastError(), "data movement launch");
}

/* Rectangles of coarse cells under the fine boxes, one per (fine box,
 * coarse box) overlap, found through the coarse level's block map. */
std::vector<AvgRect> avg_plan(const sh_level *F, const sh_level *C, long long &ncells) {
    std::vector<AvgRect> r;
    ncells = 0;
    const int R = C->owner_res;
    std::vector<int> owners;
    for (size_t fb = 0; fb < F->boxes.size(); ++fb) {
        int clo[3], chi[3], b0[3], b1[3];
        for (int d = 0; d < 3; ++d) {
            auto cdiv = [](int a) { return a >= 0 ? a / 2 : -((-a + 1) / 2); };
            clo[d] = cdiv(F->boxes[fb].lo[d]);
            chi[d] = cdiv(F->boxes[fb].hi[d]);
            b0[d] = floordiv(std::max(clo[d], C->dlo[d]) - C->dlo[d], R);
            b1[d] = floordiv(std::min(chi[d], C->dhi[d]) - C->dlo[d], R);
        }
        owners.clear();
        for (int z = b0[2]; z <= b1[2]; ++z)
            for (int y = b0[1]; y <= b1[1]; ++y)
                for (int x = b0[0]; x <= b1[0]; ++x) {
                    const int o = C->owner[((size_t)z * C->owner_nb[1] + y) * C->owner_nb[0] + x];
                    if (o >= 0) owners.push_back(o);
                }
        std::sort(owners.begin(), owners.end());
        owners.erase(std::unique(owners.begin(), owners.end()), owners.end());
        for (int cb : owners) {
            int lo[3], hi[3];
            if (!box_intersect(clo, chi, C->boxes[cb].lo, C->boxes[cb].hi, lo, hi)) continue;
            AvgRect a;
            a.fbox = (int)fb;
            a.cbox = cb;
            for (int d = 0; d < 3; ++d) {
                a.lo[d] = lo[d];
                a.hi[d] = hi[d];
            }
            a.first = ncells;
            ncells += (long long)(hi[0] - lo[0] + 1) * (hi[1] - lo[1] + 1) * (hi[2] - lo[2] + 1);
            r.push_back(a);
        }
    }
    return r;
}

void average_down_impl(sh_ctx *ctx, const sh_level *F, int which_f, sh_level *C, int which_c,
                       bool with_te) {
    require(F->ncomp == C->ncomp, "fine and coarse levels differ in components");
    require(F->esize == C->esize, "fine and coarse levels differ in precision");
    if (F->avg_for != C->uid) {
        for (const sh_box &b : F->boxes)
            for (int d = 0; d < 3; ++d)
                require(b.lo[d] % 2 == 0 && b.hi[d] % 2 != 0 && b.lo[d] >= 0,
                        "fine boxes must be aligned to the refinement ratio 2");
        long long ncells = 0;
        std::vector<AvgRect> plan = avg_plan(F, C, ncells);
        dfree_async(ctx, F->d_avg);
        F->d_avg = upload_async(ctx, plan.data(), plan.size(), "average-down plan");
        F->navg = (int)plan.size();
        F->avg_cells = ncells;
        F->avg_for = C->uid;
    }
    if (F->avg_cells == 0) return;
    ProfScope ps(ctx, kProfAvg);
    if (F->esize == 4) {
        /* truncation errors of an FP32 level go to its FP64 array */
        double *te = nullptr;
        if (with_te) {
            sh_level *Fm = const_cast<sh_level *>(F);
            if (!Fm->te64) {
                const size_t bytes = (size_t)F->total_gvol * F->ncomp * sizeof(double);
                Fm->te64 = (double *)dmalloc_async(ctx, bytes, "truncation errors");
                ck(cudaMemsetAsync(Fm->te64, 0, bytes, ctx->stream), "truncation errors clear");
            }
            te = Fm->te64;
        }
        avgdown_kernel<float><<<grid_for(F->avg_cells), 256, 0, ctx->stream>>>(
            (const AvgRect *)F->d_avg, F->navg, F->avg_cells, F->d_boxes, C->d_boxes, F->ncomp,
            (const float *)F->buf[which_f], F->cmp[which_f], (float *)C->buf[which_c],
            C->cmp[which_c], te, (float *)F->buf[SH_OLD], F->cmp[SH_OLD]);
    } else {
        avgdown_kernel<double><<<grid_for(F->avg_cells), 256, 0, ctx->stream>>>(
            (const AvgRect *)F->d_avg, F->navg, F->avg_cells, F->d_boxes, C->d_boxes, F->ncomp,
            F->buf[which_f], nullptr, C->buf[which_c], nullptr,
            with_te ? F->buf[SH_OLD] : nullptr, nullptr, nullptr);
    }
    ctx->launches++;
    ck(cudaGetLastError(), "average-down launch");
}

} // namespace

namespace sh {
void set_ctx_error(::sh_ctx *ctx, const std::string &msg) {
    if (ctx) ctx->err = msg;
}
} // namespace sh

/* ====================================================================== */
extern "C" {

int sh_ctx_create(int device, sh_ctx **out) {
    if (!out) return SH_ERR_ARG;
    *out = nullptr;
    sh_ctx *ctx = new (std::nothrow) sh_ctx();
    if (!ctx) return SH_ERR_NOMEM;
    ctx->device = device;
    int rc = guarded(ctx, [&] {
        int n = 0;
        ck(cudaGetDeviceCount(&n), "cudaGetDeviceCount");
        require(device >= 0 && device < n, "no such CUDA device");
        set_device(ctx);
        ck(cudaStreamCreateWithFlags(&ctx->own_stream, cudaStreamNonBlocking), "stream create");
        ctx->stream = ctx->own_stream;
        /* keep freed level memory in this process's pool for reuse */
        cudaMemPool_t pool;
        ck(cudaDeviceGetDefaultMemPool(&pool, device), "default memory pool");
        uint64_t thr = UINT64_MAX;
        ck(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr),
           "memory pool threshold");
    });
    if (rc != SH_OK) {
        std::fprintf(stderr, "sh_ctx_create: %s\n", ctx->err.c_str());
        delete ctx;
        return rc;
    }
    *out = ctx;
    return SH_OK;
}

int sh_ctx_destroy(sh_ctx *ctx) {
    if (!ctx) return SH_ERR_ARG;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, ctx->device) == cudaSuccess)
        cudaMemPoolTrimTo(pool, 0);
    cudaFree(ctx->scratch);
    ctx->gw.release();
    for (const ProfRecord &r : ctx->prof) {
        cudaEventDestroy(r.start);
        cudaEventDestroy(r.stop);
    }
    for (cudaEvent_t e : ctx->event_pool) cudaEventDestroy(e);
    if (ctx->own_stream) cudaStreamDestroy(ctx->own_stream);
    delete ctx;
    return SH_OK;
}

const char *sh_ctx_last_error(const sh_ctx *ctx) { return ctx ? ctx->err.c_str() : "no context"; }

int sh_ctx_set_stream(sh_ctx *ctx, void *s) {
    if (!ctx) return SH_ERR_ARG;
    ctx->stream = s ? (cudaStream_t)s : ctx->own_stream;
    return SH_OK;
}

void *sh_ctx_stream(sh_ctx *ctx) { return ctx ? (void *)ctx->stream : nullptr; }

int sh_ctx_synchronize(sh_ctx *ctx) {
    if (!ctx) return SH_ERR_ARG;
    return guarded(ctx, [&] { ck(cudaStreamSynchronize(ctx->stream), "synchronize"); });
}

long long sh_ctx_kernel_launches(const sh_ctx *ctx) { return ctx ? ctx->launches : 0; }

int sh_ctx_profile(sh_ctx *ctx, int enable) {
    if (!ctx) return SH_ERR_ARG;
    return guarded(ctx, [&] {
        set_device(ctx);
        profile_resolve(ctx);
        if (enable) {
            for (int c = 0; c < kProfCount; ++c) {
                ctx->prof_ms[c] = 0;
                ctx->prof_n[c] = 0;
            }
        }
        ctx->profiling = enable != 0;
    });
}

int sh_ctx_profile_read(sh_ctx *ctx, const char *category, double *total_ms,
                        long long *launches) {
    if (!ctx || !category) return SH_ERR_ARG;
    return guarded(ctx, [&] {
        set_device(ctx);
        profile_resolve(ctx);
        for (int c = 0; c < kProfCount; ++c)
            if (std::strcmp(kProfCategories[c], category) == 0) {
                if (total_ms) *total_ms = ctx->prof_ms[c];
                if (launches) *launches = ctx->prof_n[c];
                return;
            }
        throw ShError(SH_ERR_ARG, std::string("unknown profile category ") + category);
    });
}

int sh_project_count(void) { return project_count(); }

const char *sh_project_name(int id) {
    const ProjectOps *p = project_by_id(id);
    return p ? p->name : nullptr;
}

int sh_project_find(const char *name, int *id) {
    if (!name || !id) return SH_ERR_ARG;
    for (int q = 0; q < project_count(); ++q)
        if (std::strcmp(project_by_id(q)->name, name) == 0) {
            *id = q;
            return SH_OK;
        }
    return SH_ERR_PROJECT;
}

int sh_project_ncomp(int id, int with_gw, int *ncomp, int *npairs) {
    const ProjectOps *p = project_by_id(id);
    if (!p) return SH_ERR_PROJECT;
    if (with_gw && !p->has_gw) return SH_ERR_UNSUPPORTED;
    if (ncomp) *ncomp = p->nscalars + (with_gw ? 12 : 0);
    if (npairs) *npairs = p->nscalars / 2 + (with_gw ? 6 : 0);
    return SH_OK;
}

int sh_project_comp_name(int id, int comp, const char **name) {
    const ProjectOps *p = project_by_id(id);
    if (!p) return SH_ERR_PROJECT;
    if (!name) return SH_ERR_ARG;
    /* appended after the user fields (gravitational_waves.cpp:20-31) */
    static const char *const kGw[12] = {"u_xx",  "u_yy",  "u_zz",  "u_xy",  "u_xz",  "u_yz",
                                        "du_xx", "du_yy", "du_zz", "du_xy", "du_xz", "du_yz"};
    if (comp >= 0 && comp < p->nscalars) {
        *name = p->field_name(comp);
        return *name ? SH_OK : SH_ERR_PROJECT;
    }
    if (p->has_gw && comp >= p->nscalars && comp < p->nscalars + 12) {
        *name = kGw[comp - p->nscalars];
        return SH_OK;
    }
    return SH_ERR_ARG;
}

int sh_level_create(sh_ctx *ctx, int project, int with_gw, const int domain_lo[3],
                    const int domain_hi[3], const sh_box *boxes, int nbox, int nghost,
                    sh_level **out) {
    return sh_level_create_prec(ctx, project, with_gw, domain_lo, domain_hi, boxes, nbox, nghost,
                                SH_PREC_FP64, out);
}

int sh_level_precision(const sh_level *L, int *precision) {
    if (!L || !precision) return SH_ERR_ARG;
    *precision = L->esize == 8 ? SH_PREC_FP64 : SH_PREC_FP32_KAHAN;
    return SH_OK;
}

int sh_level_create_prec(sh_ctx *ctx, int project, int with_gw, const int domain_lo[3],
                         const int domain_hi[3], const sh_box *boxes, int nbox, int nghost,
                         int precision, sh_level **out) {
    if (!ctx || !out) return SH_ERR_ARG;
    if (precision != SH_PREC_FP64 && precision != SH_PREC_FP32_KAHAN) return SH_ERR_ARG;
    *out = nullptr;
    sh_level *L = new (std::nothrow) sh_level();
    static std::atomic<long long> next_uid{1};
    if (L) L->uid = next_uid++;
    if (!L) return SH_ERR_NOMEM;
    int rc = guarded(ctx, [&] {
        set_device(ctx);
        L->ops = project_by_id(project);
        if (!L->ops) throw ShError(SH_ERR_PROJECT, "unknown project id");
        if (with_gw && !L->ops->has_gw)
            throw ShError(SH_ERR_UNSUPPORTED, "project has no gravitational-wave hooks");
        require(boxes && nbox > 0 && domain_lo && domain_hi, "boxes and domain required");
        require(nghost >= L->ops->reach && nghost <= 8,
                "nghost must cover the project's stencil reach and be at most 8");
        L->project = project;
        L->with_gw = with_gw != 0;
        if (precision == SH_PREC_FP32_KAHAN) {
            const int fam = stage32_family(L->ops);
            require(fam != 0,
                    "FP32 levels are available for AxionStringsLap1, AxionStringsLap2 and "
                    "FirstOrderPhaseTransition");
            require(!L->with_gw || fam == kFam32Fopt,
                    "FP32 axion-string levels carry no GW tensor");
            L->esize = 4;
        }
        L->ncomp = L->ops->nscalars + (L->with_gw ? 12 : 0);
        L->npairs = L->ops->nscalars / 2 + (L->with_gw ? 6 : 0);
        require(L->ncomp <= kMaxComp, "too many components");
        L->nghost = nghost;
        for (int d = 0; d < 3; ++d) {
            L->dlo[d] = domain_lo[d];
            L->dhi[d] = domain_hi[d];
            require(domain_hi[d] >= domain_lo[d], "empty domain");
        }
        L->boxes.assign(boxes, boxes + nbox);
        long long base = 0, vb = 0;
        std::vector<TileDev> tiles;
        L->vbase.push_back(0);
        for (int b = 0; b < nbox; ++b) {
            BoxDev bd;
            std::memset(&bd, 0, sizeof(bd));
            bd.off = base;
            long long gv = 1;
            for (int d = 0; d < 3; ++d) {
                require(boxes[b].hi[d] >= boxes[b].lo[d], "empty box");
                require(boxes[b].lo[d] >= domain_lo[d] && boxes[b].hi[d] <= domain_hi[d],
                        "box outside the domain");
                bd.lo[d] = boxes[b].lo[d];
                bd.hi[d] = boxes[b].hi[d];
                bd.glo[d] = boxes[b].lo[d] - nghost;
                bd.gdim[d] = boxes[b].hi[d] - boxes[b].lo[d] + 1 + 2 * nghost;
                gv *= bd.gdim[d];
            }
            bd.gvol = gv;
            base += gv;
            const long long nv = (long long)(bd.hi[0] - bd.lo[0] + 1) *
                                 (bd.hi[1] - bd.lo[1] + 1) * (bd.hi[2] - bd.lo[2] + 1);
            vb += nv;
            L->vbase.push_back(vb);
            L->hboxes.push_back(bd);
        }
        /* deep tiles amortise the per-column set-up of the hooks; a level
         * whose deep tiles would not fill two waves of seven blocks per SM
         * gets shallow ones */
        auto make_tiles = [&](int depth) {
            tiles.clear();
            for (int b = 0; b < nbox; ++b) {
                const BoxDev &bd = L->hboxes[b];
                for (int z = bd.lo[2]; z <= bd.hi[2]; z += depth)
                    for (int x = bd.lo[0]; x <= bd.hi[0]; x += kTileX) {
                        const int nx = std::min(kTileX, bd.hi[0] - x + 1);
                        const int rows = kThreads / nx;
                        const int nz = std::min(depth, bd.hi[2] - z + 1);
                        for (int y = bd.lo[1]; y <= bd.hi[1]; y += rows)
                            tiles.push_back(TileDev{b, x, y, z, nx, nz});
                    }
            }
        };
        int nsm = 0;
        ck(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, ctx->device),
           "SM count");
        make_tiles(kTileZ);
        if (L->esize == 8) {
            if ((long long)tiles.size() < 2LL * 7 * nsm) make_tiles(kTileZShallow);
        } else {
            /* the FP32 stage kernels (32-40 registers, up to 16 blocks per
             * SM) wait on memory: shallower tiles until the level gives
             * four waves of them */
            for (int depth = kTileZ / 2; depth >= 1 && (long long)tiles.size() < 4LL * 16 * nsm;
                 depth /= 2)
                make_tiles(depth);
        }
        L->total_gvol = base;
        L->nvalid = vb;
        if (L->esize == 8 && nbox == 1) {
            bool whole = true;
            for (int d = 0; d < 3; ++d)
                whole = whole && boxes[0].lo[d] == domain_lo[d] && boxes[0].hi[d] == domain_hi[d] &&
                        2 * nghost <= domain_hi[d] - domain_lo[d] + 1;
            L->self_periodic = whole;
        }
        L->ntiles = (int)tiles.size();
        L->d_boxes = upload_async(ctx, L->hboxes.data(), L->hboxes.size(), "box table");
        L->d_tiles = upload_async(ctx, tiles.data(), tiles.size(), "tile table");
        L->d_vbase = upload_async(ctx, L->vbase.data(), L->vbase.size(), "box prefix");
        build_owner_map(ctx, L);
        build_ghost_plan(ctx, L);
        const size_t bytes = (size_t)L->total_gvol * L->ncomp * L->esize;
        for (int q = 0; q < 3; ++q) {
            L->buf[q] = (double *)dmalloc_async(ctx, bytes, "level buffer");
            ck(cudaMemsetAsync(L->buf[q], 0, bytes, ctx->stream), "level buffer clear");
        }
        if (L->esize == 4)
            for (int q = 0; q < 2; ++q) {
                L->cmp[q] = (float *)dmalloc_async(ctx, bytes, "level compensations");
                ck(cudaMemsetAsync(L->cmp[q], 0, bytes, ctx->stream), "compensations clear");
            }
    });
    if (rc != SH_OK) {
        level_free(ctx, L);
        delete L;
        return rc;
    }
    *out = L;
    return SH_OK;
}

int sh_level_destroy(sh_ctx *ctx, sh_level *L) {
    if (!ctx || !L) return SH_ERR_ARG;
    cudaSetDevice(ctx->device);
    level_free(ctx, L); /* stream-ordered: after the work queued on the level */
    delete L;
    return SH_OK;
}

int sh_level_project(const sh_level *L, int *project, int *with_gw) {
    if (!L) return SH_ERR_ARG;
    if (project) *project = L->project;
    if (with_gw) *with_gw = L->with_gw ? 1 : 0;
    return SH_OK;
}

int sh_level_domain(const sh_level *L, int lo[3], int hi[3]) {
    if (!L || !lo || !hi) return SH_ERR_ARG;
    for (int d = 0; d < 3; ++d) {
        lo[d] = L->dlo[d];
        hi[d] = L->dhi[d];
    }
    return SH_OK;
}

int sh_level_info(const sh_level *L, int *ncomp, int *nbox, long long *nvalid) {
    if (!L) return SH_ERR_ARG;
    if (ncomp) *ncomp = L->ncomp;
    if (nbox) *nbox = (int)L->boxes.size();
    if (nvalid) *nvalid = L->nvalid;
    return SH_OK;
}

int sh_level_time(const sh_level *L, int which, double *t, int *istep) {
    if (!L || (which != SH_NEW && which != SH_OLD)) return SH_ERR_ARG;
    if (t) *t = L->t[which];
    if (istep) *istep = L->istep[which];
    return SH_OK;
}

int sh_level_boxes(const sh_level *L, sh_box *out, int capacity, int *nbox) {
    if (!L || !nbox) return SH_ERR_ARG;
    *nbox = (int)L->boxes.size();
    if (!out) return SH_OK;
    if (capacity < (int)L->boxes.size()) return SH_ERR_ARG;
    std::copy(L->boxes.begin(), L->boxes.end(), out);
    return SH_OK;
}

int sh_level_set_index(sh_level *L, int lev) {
    if (!L) return SH_ERR_ARG;
    L->lev_index = lev;
    return SH_OK;
}

int sh_level_set_time(sh_level *L, int which, double t, int istep) {
    if (!L || (which != SH_NEW && which != SH_OLD)) return SH_ERR_ARG;
    L->t[which] = t;
    L->istep[which] = istep;
    return SH_OK;
}

int sh_level_write(sh_ctx *ctx, sh_level *L, int which, int layout, const double *host) {
    if (!ctx || !L || !host || (which != SH_NEW && which != SH_OLD)) return SH_ERR_ARG;
    return guarded(ctx, [&] {
        L->version++;
        set_device(ctx);
        const size_t bytes = (size_t)L->nvalid * L->ncomp * sizeof(double);
        double *stage = (double *)ctx_scratch(ctx, bytes);
        ck(cudaMemcpyAsync(stage, host, bytes, cudaMemcpyHostToDevice, ctx->stream), "upload");
        move(ctx, L, which, stage, layout, 0);
        ck(cudaStreamSynchronize(ctx->stream), "upload");
    });
}

int sh_level_read(sh_ctx *ctx, const sh_level *L, int which, int layout, double *host) {
    if (!ctx || !L || !host || (which != SH_NEW && which != SH_OLD)) return SH_ERR_ARG;
    return guarded(ctx, [&] {
        set_device(ctx);
        const size_t bytes = (size_t)L->nvalid * L->ncomp * sizeof(double);
        double *stage = (double *)ctx_scratch(ctx, bytes);
        move(ctx, L, which, stage, layout, 1);
        ck(cudaMemcpyAsync(host, stage, bytes, cudaMemcpyDeviceToHost, ctx->stream), "download");
        ck(cudaStreamSynchronize(ctx->stream), "download");
    });
}

int sh_level_write_device(sh_ctx *ctx, sh_level *L, int which, int layout, const double *dev) {
    if (!ctx || !L || !dev || (which != SH_NEW && which != SH_OLD)) return SH_ERR_ARG;
    return guarded(ctx, [&] {
        L->version++;
        set_device(ctx);
        move(ctx, L, which, const_cast<double *>(dev), layout, 0);
    });
}

int sh_level_read_device(sh_ctx *ctx, const sh_level *L, int which, int layout, double *dev) {
    if (!ctx || !L || !dev || (which != SH_NEW && which != SH_OLD)) return SH_ERR_ARG;
    return guarded(ctx, [&] {
        set_device(ctx);
        move(ctx, L, which, dev, layout, 1);
    });
}

int sh_level_fill_patch(sh_ctx *ctx, sh_level *L, int which) {
    if (!ctx || !L || (which != SH_NEW && which != SH_OLD)) return SH_ERR_ARG;
    return guarded(ctx, [&] {
        L->version++;
        set_device(ctx);
        fill_patch(ctx, L, L->buf[which], L->t[which]);
    });
}

int sh_level_set_coarse(sh_ctx *ctx, sh_level *fine, sh_level *coarse) {
    if (!ctx || !fine) return SH_ERR_ARG;
    return guarded(ctx, [&] {
        set_device(ctx);
        dfree_async(ctx, fine->d_cf);
        fine->d_cf = nullptr;
        dfree_async(ctx, fine->cf_old);
        dfree_async(ctx, fine->cf_new);
        fine->cf_old = fine->cf_new = nullptr;
        fine->cf_uid = fine->cf_ver = -1;
        fine->ncf = 0;
        fine->ncf_items = 0;
        fine->coarse = nullptr;
        if (!coarse) return;
        require(coarse != fine, "a level cannot be its own coarse level");
        require(coarse->esize == fine->esize, "fine and coarse levels differ in precision");
        FillPlan P = build_fill_plan(fine, fine, coarse, true, false);
        const std::vector<CfItem> items = cf_items(P.cf, fine);
        fine->d_cf = upload_items(ctx, items, "coarse-fine plan");
        fine->ncf_items = (int)items.size();
        fine->ncf = P.cf_cells;
        fine->coarse = coarse;
    });
}

int sh_level_fill_from(sh_ctx *ctx, sh_level *dst, int which_dst, const sh_level *src,
                       int which_src, sh_level *coarse, double time) {
    if (!ctx || !dst || (which_dst != SH_NEW && which_dst != SH_OLD)) return SH_ERR_ARG;
    if (src && which_src != SH_NEW && which_src != SH_OLD) return SH_ERR_ARG;
    return guarded(ctx, [&] {
        dst->version++;
        set_device(ctx);
        require(src != dst, "source and destination must differ");
        if (src) require(src->ncomp == dst->ncomp, "source differs in components");
        if (src) require(src->esize == dst->esize, "source differs in precision");
        if (coarse) require(coarse->esize == dst->esize, "coarse level differs in precision");
        const bool f32 = dst->esize == 4;
        FillPlan P = build_fill_plan(dst, src, coarse, false);
        CopyItem *d_rects = nullptr;
        CfItem *d_cf = nullptr;
        if (!P.rects.empty()) {
            const std::vector<CopyItem> items = copy_items(P.rects, dst, src);
            d_rects = upload_items(ctx, items, "fill plan");
            ProfScope ps(ctx, kProfFill);
            if (f32) {
                /* values and their compensations */
                copy_items_kernel<float><<<(int)items.size(), kItemThreads, 0, ctx->stream>>>(
                    d_rects, (float *)dst->buf[which_dst], (const float *)src->buf[which_src],
                    dst->ncomp);
                copy_items_kernel<float><<<(int)items.size(), kItemThreads, 0, ctx->stream>>>(
                    d_rects, dst->cmp[which_dst], src->cmp[which_src], dst->ncomp);
                ctx->launches++;
            } else {
                copy_items_kernel<double><<<(int)items.size(), kItemThreads, 0, ctx->stream>>>(
                    d_rects, dst->buf[which_dst], src->buf[which_src], dst->ncomp);
            }
            ctx->launches++;
            ck(cudaGetLastError(), "fill copy launch");
        }
        if (!P.cf.empty()) {
            require(coarse != nullptr, "cells not covered by the source need a coarse level");
            const std::vector<CfItem> items = cf_items(P.cf, dst);
            d_cf = upload_items(ctx, items, "coarse fill plan");
            int mode;
            double alpha, beta;
            coarse_time_weights(coarse, time, mode, alpha, beta);
            ProfScope ps(ctx, kProfCf);
            if (f32)
                cf_interp_kernel<float><<<(int)items.size(), 128, 0, ctx->stream>>>(
                    d_cf, coarse->d_boxes, (float *)dst->buf[which_dst], owner_map_dev(coarse),
                    (const float *)coarse->buf[SH_OLD], (const float *)coarse->buf[SH_NEW], mode,
                    alpha, beta, dst->ncomp, nullptr, 0, dst->cmp[which_dst]);
            else
                cf_interp_kernel<double><<<(int)items.size(), 128, 0, ctx->stream>>>(
                    d_cf, coarse->d_boxes, dst->buf[which_dst], owner_map_dev(coarse),
                    coarse->buf[SH_OLD], coarse->buf[SH_NEW], mode, alpha, beta, dst->ncomp,
                    nullptr, 0, nullptr);
            ctx->launches++;
            ck(cudaGetLastError(), "coarse fill launch");
        }
        dfree_async(ctx, d_rects);
        dfree_async(ctx, d_cf);
    });
}

int sh_level_advance(sh_ctx *ctx, sh_level *L, int integrator, const double *tableau,
                     int nstages, double dt, double dx, const double *params, int nparams,
                     const double *gw_params, int ngw, int ko_order, const double *ko_strength,
                     int flags) {
    if (!ctx || !L) return SH_ERR_ARG;
    return guarded(ctx, [&] {
        const long long ver = L->version;
        L->version++;
        set_device(ctx);
        require(dt > 0 && dx > 0, "dt and dx must be positive");
        if (!(flags & SH_ADVANCE_NO_SWAP)) {
            std::swap(L->buf[SH_NEW], L->buf[SH_OLD]);
            std::swap(L->cmp[SH_NEW], L->cmp[SH_OLD]);
            std::swap(L->t[SH_NEW], L->t[SH_OLD]);
            std::swap(L->istep[SH_NEW], L->istep[SH_OLD]);
        }
        /* FillPatch at t_old, unless the last stage of the previous step
         * filled this buffer for the same time and neither this level nor
         * its coarse level changed since (the finest level between its two
         * sub-steps): the ghost values would be the same */
        if (!fill_current(L, L->buf[SH_OLD], L->t[SH_OLD], ver))
            fill_patch(ctx, L, L->buf[SH_OLD], L->t[SH_OLD]);
        if (L->esize == 4) {
            require(ko_order == 0, "FP32 levels have no Kreiss-Oliger dissipation");
            if (stage32_family(L->ops) == kFam32Fopt)
                integrate32_fopt(ctx, L, integrator, dt, dx, params, nparams);
            else
                integrate32(ctx, L, integrator, dt, dx, params, nparams, ko_order);
        } else {
            integrate(ctx, L, integrator, tableau, nstages, dt, dx, params, nparams, gw_params,
                      ngw, ko_order, ko_strength);
        }
        L->t[SH_NEW] = L->t[SH_OLD] + dt;
        L->istep[SH_NEW] = L->istep[SH_OLD] + 1;
        ck(cudaGetLastError(), "advance");
    });
}

int sh_level_rhs(sh_ctx *ctx, sh_level *L, int which, double time, int lev, double dt,
                 double dx, const double *params, int nparams, const double *gw_params, int ngw,
                 int ko_order, const double *ko_strength, double *host_rhs) {
    if (!ctx || !L || !host_rhs || (which != SH_NEW && which != SH_OLD)) return SH_ERR_ARG;
    return guarded(ctx, [&] {
        L->version++;
        set_device(ctx);
        require_fp64(L, "the Rhs through the project hooks");
        StageArgs a;
        fill_common(a, L, dt, dx, params, nparams, gw_params, ngw, ko_order, ko_strength);
        a.state = L->buf[which];
        a.out = L->buf[2];
        a.epi = kEpiPlainRhs;
        a.time = time;
        a.lev = lev;
        launch_stage(ctx, L, a, ko_order);
        const size_t bytes = (size_t)L->nvalid * L->ncomp * sizeof(double);
        double *stage = (double *)ctx_scratch(ctx, bytes);
        move(ctx, L, 2, stage, 1, 1);
        ck(cudaMemcpyAsync(host_rhs, stage, bytes, cudaMemcpyDeviceToHost, ctx->stream),
           "download");
        ck(cudaStreamSynchronize(ctx->stream), "rhs");
    });
}

int sh_level_add_bubbles(sh_ctx *ctx, sh_level *L, int which, int comp_phi, int comp_dphi,
                         int nb, const double *xyz, const double *profile, int nbins,
                         double inv_dx, double Lcut, double dx) {
    if (!ctx || !L || (which != SH_NEW && which != SH_OLD) || nb < 0 ||
        (nb > 0 && (!xyz || !profile)) || nbins < 2 || !(inv_dx > 0) || !(Lcut > 0) ||
        !(dx > 0))
        return SH_ERR_ARG;
    if (nb == 0) return SH_OK;
    return guarded(ctx, [&] {
        L->version++;
        set_device(ctx);
        require(comp_phi >= 0 && comp_phi < L->ncomp && comp_dphi >= 0 &&
                    comp_dphi < L->ncomp,
                "component index out of range");
        require((long long)(Lcut * inv_dx) + 2 <= nbins,
                "profile needs at least floor(Lcut * inv_dx) + 2 bins");
        const int N = L->dhi[0] - L->dlo[0] + 1;
        for (int d = 0; d < 3; ++d)
            require(L->dhi[d] - L->dlo[d] + 1 == N, "bubbles need a cubic domain");
        const size_t nx = 3 * (size_t)nb, np = 2 * (size_t)nbins;
        double *d = (double *)ctx_scratch(ctx, (nx + np) * sizeof(double));
        ck(cudaMemcpyAsync(d, xyz, nx * sizeof(double), cudaMemcpyHostToDevice, ctx->stream),
           "bubble upload");
        ck(cudaMemcpyAsync(d + nx, profile, np * sizeof(double), cudaMemcpyHostToDevice,
                           ctx->stream),
           "bubble upload");
        BubbleList bl{d, d + nx, nb, nbins, inv_dx, Lcut};
        if (L->esize == 4)
            level_bubbles_kernel<float><<<grid_for(L->nvalid), 256, 0, ctx->stream>>>(
                L->d_boxes, L->d_vbase, (int)L->boxes.size(), L->nvalid, L->ncomp, comp_phi,
                comp_dphi, (float *)L->buf[which], L->cmp[which], bl, dx, N * dx);
        else
            level_bubbles_kernel<double><<<grid_for(L->nvalid), 256, 0, ctx->stream>>>(
                L->d_boxes, L->d_vbase, (int)L->boxes.size(), L->nvalid, L->ncomp, comp_phi,
                comp_dphi, L->buf[which], nullptr, bl, dx, N * dx);
        ctx->launches++;
        ck(cudaGetLastError(), "bubble launch");
        ck(cudaStreamSynchronize(ctx->stream), "bubbles");
    });
}

int sh_scalar_spectrum(sh_ctx *ctx, const sh_level *L, int fn, int comp, double dx,
                       double *bins_out, long long *ks_out, int max_bins, int *nbins) {
    if (!ctx || !L || !bins_out || !nbins || !(dx > 0)) return SH_ERR_ARG;
    return guarded(ctx, [&] {
        set_device(ctx);
        require(fn >= SH_OUT_COMPONENT && fn <= SH_OUT_R_PRIME2, "unknown output function");
        require(fn > SH_OUT_COMPONENT_SQ ? L->ncomp >= 4 : (comp >= 0 && comp < L->ncomp),
                "component index out of range");
        const int N = L->dhi[0] - L->dlo[0] + 1;
        long long dv = 1;
        for (int d = 0; d < 3; ++d) {
            require(L->dhi[d] - L->dlo[d] + 1 == N, "spectrum needs a cubic domain");
            dv *= N;
        }
        require(dv == L->nvalid, "spectrum needs a level covering its whole domain");
        const size_t sbytes = (gw_scratch_bytes(N, 1) + 255) & ~size_t(255);
        const size_t maxb = (size_t)3 * (N / 2 + 1) * (N / 2 + 1) + 16;
        char *base = (char *)ctx_scratch(ctx, sbytes + maxb * sizeof(double));
        double *bins_dev = (double *)(base + sbytes);
        const double fac = std::pow(1. / N, 6);
        const double dk = 2. * M_PI / (N * dx);
        const double pre = fac * L->t[SH_NEW] / dk;
        int nb = 0;
        std::string err;
        ProfScope ps(ctx, kProfGw);
        cudaError_t e = scalar_spectrum_packed(
            ctx->gw, ctx->stream, N, pre, (double *)base, bins_dev, &nb, &ctx->launches, err,
            [&](double *real) {
                out_pack_kernel<<<grid_for(L->nvalid), 256, 0, ctx->stream>>>(
                    L->d_boxes, L->d_vbase, (int)L->boxes.size(), L->nvalid, L->ncomp, fn, comp,
                    state64(ctx, L, SH_NEW), real, N, L->dlo[0], L->dlo[1], L->dlo[2]);
            });
        if (!err.empty()) throw ShError(SH_ERR_CUDA, err);
        ck(e, "scalar spectrum");
        *nbins = nb;
        require(nb <= max_bins, "bins_out too small");
        ck(cudaMemcpyAsync(bins_out, bins_dev, nb * sizeof(double), cudaMemcpyDeviceToHost,
                           ctx->stream),
           "bins download");
        ck(cudaStreamSynchronize(ctx->stream), "scalar spectrum");
        if (ks_out) std::copy(ctx->gw.ks().begin(), ctx->gw.ks().end(), ks_out);
    });
}

int sh_projection(sh_ctx *ctx, const sh_level *const *levels, int nlev, int fn, int comp,
                  int mode, double *data_out, int *n_out) {
    if (!ctx || !levels || nlev <= 0 || !data_out || !n_out) return SH_ERR_ARG;
    return guarded(ctx, [&] {
        set_device(ctx);
        require(nlev <= kMaxProjLevels, "at most 8 levels");
        require(fn >= SH_OUT_COMPONENT && fn <= SH_OUT_R_PRIME2, "unknown output function");
        require(mode == 0 || mode == 1, "mode must be 0 (sum) or 1 (maximum)");
        ProjArgs a;
        std::memset(&a, 0, sizeof(a));
        a.nlev = nlev;
        a.fn = fn;
        a.comp = comp;
        a.mode = mode;
        for (int l = 0; l < nlev; ++l) {
            const sh_level *L = levels[l];
            require(L != nullptr, "null level");
            require(fn > SH_OUT_COMPONENT_SQ ? L->ncomp >= 4 : (comp >= 0 && comp < L->ncomp),
                    "component index out of range");
            const int N = L->dhi[0] - L->dlo[0] + 1;
            for (int d = 0; d < 3; ++d)
                require(L->dlo[d] == 0 && L->dhi[d] + 1 == N,
                        "projection levels need cubic domains starting at 0");
            if (l > 0) require(N == 2 * a.lev[l - 1].dimN, "levels must refine by 2");
            a.lev[l].map = owner_map_dev(L);
            a.lev[l].boxes = L->d_boxes;
            a.lev[l].buf = state64(ctx, L, SH_NEW);
            a.lev[l].ncomp = L->ncomp;
            a.lev[l].dimN = N;
        }
        a.dimN = a.lev[nlev - 1].dimN;
        const long long npix = (long long)a.dimN * a.dimN;
        char *base = (char *)ctx_scratch(ctx, npix * (sizeof(double) + sizeof(int)) + 256);
        double *d_data = (double *)base;
        int *d_n = (int *)(base + ((npix * sizeof(double) + 255) & ~255LL));
        projection_kernel<<<grid_for(npix), 256, 0, ctx->stream>>>(a, d_data, d_n);
        ctx->launches++;
        ck(cudaGetLastError(), "projection launch");
        ck(cudaMemcpyAsync(data_out, d_data, npix * sizeof(double), cudaMemcpyDeviceToHost,
                           ctx->stream),
           "projection download");
        ck(cudaMemcpyAsync(n_out, d_n, npix * sizeof(int), cudaMemcpyDeviceToHost, ctx->stream),
           "projection download");
        ck(cudaStreamSynchronize(ctx->stream), "projection");
    });
}

int sh_level_reduce(sh_ctx *ctx, const sh_level *L, int which, int op, int comp, double *out) {
    if (!ctx || !L || !out || (which != SH_NEW && which != SH_OLD)) return SH_ERR_ARG;
    if (op < SH_REDUCE_MAX_ABS || op > SH_REDUCE_SUM_MODULUS) return SH_ERR_ARG;
    if (comp < 0 || comp >= L->ncomp) return SH_ERR_ARG;
    if (op == SH_REDUCE_SUM_MODULUS && comp + 1 >= L->ncomp) return SH_ERR_ARG;
    return guarded(ctx, [&] {
        set_device(ctx);
        const int nbox = (int)L->boxes.size();
        double *d = (double *)ctx_scratch(ctx, ((size_t)nbox + 1) * sizeof(double));
        reduce_boxes_kernel<<<nbox, kReduceThreads, 0, ctx->stream>>>(
            L->d_boxes, state64(ctx, L, which), L->ncomp, comp, op, d + 1);
        reduce_final_kernel<<<1, kReduceThreads, 0, ctx->stream>>>(d + 1, nbox, op, d);
        ctx->launches += 2;
        ck(cudaGetLastError(), "reduce launch");
        ck(cudaMemcpyAsync(out, d, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream),
           "reduce download");
        ck(cudaStreamSynchronize(ctx->stream), "reduce");
    });
}

int sh_level_check_finite(sh_ctx *ctx, const sh_level *L, int which, long long *nonfinite) {
    if (nonfinite) *nonfinite = 0;
    if (!ctx || !L || (which != SH_NEW && which != SH_OLD)) return SH_ERR_ARG;
    std::vector<double> counts(L->ncomp, 0.);
    int rc = guarded(ctx, [&] {
        set_device(ctx);
        const int nbox = (int)L->boxes.size();
        double *d = (double *)ctx_scratch(ctx, ((size_t)nbox + L->ncomp) * sizeof(double));
        const double *st = state64(ctx, L, which);
        for (int c = 0; c < L->ncomp; ++c) {
            reduce_boxes_kernel<<<nbox, kReduceThreads, 0, ctx->stream>>>(
                L->d_boxes, st, L->ncomp, c, SH_REDUCE_COUNT_NONFINITE, d + L->ncomp);
            reduce_final_kernel<<<1, kReduceThreads, 0, ctx->stream>>>(
                d + L->ncomp, nbox, SH_REDUCE_COUNT_NONFINITE, d + c);
            ctx->launches += 2;
        }
        ck(cudaGetLastError(), "finite check launch");
        ck(cudaMemcpyAsync(counts.data(), d, L->ncomp * sizeof(double), cudaMemcpyDeviceToHost,
                           ctx->stream),
           "finite check download");
        ck(cudaStreamSynchronize(ctx->stream), "finite check");
    });
    if (rc != SH_OK) return rc;
    long long total = 0;
    int first = -1;
    for (int c = 0; c < L->ncomp; ++c) {
        total += (long long)counts[c];
        if (counts[c] > 0 && first < 0) first = c;
    }
    if (nonfinite) *nonfinite = total;
    if (total == 0) return SH_OK;
    const char *name = L->ops->field_name ? L->ops->field_name(first) : nullptr;
    ctx->err = std::to_string(total) + " non-finite values, the first in component " +
               std::to_string(first) + (name ? std::string(" (") + name + ")" : std::string());
    return SH_ERR_NONFINITE;
}

int sh_level_string_tags(sh_ctx *ctx, sh_level *L, double time, int lev, double dt, double dx,
                         const double *params_tag, int nparams_tag, long long *ntags) {
    if (!ctx || !L || !ntags) return SH_ERR_ARG;
    return guarded(ctx, [&] {
        set_device(ctx);
        require(L->nghost >= 1, "string tags read the +1 neighbours: nghost >= 1");
        require(nparams_tag >= 0 && nparams_tag <= kMaxParams, "at most 32 tag parameters");
        require(nparams_tag == 0 || params_tag, "params_tag required");
        TagArgs a;
        std::memset(&a, 0, sizeof(a));
        a.boxes = L->d_boxes;
        a.tiles = L->d_tiles;
        a.state = state64(ctx, L, SH_NEW);
        a.te = nullptr;
        a.ncomp = L->ncomp;
        a.lev = lev;
        a.time = time;
        a.dt = dt;
        a.dx = dx;
        for (int q = 0; q < nparams_tag; ++q) a.params_tag[q] = params_tag[q];
        const size_t cnt_bytes = (2 + kMaxComp) * sizeof(unsigned long long);
        const size_t mask_off = (cnt_bytes + 255) & ~size_t(255);
        char *base = (char *)ctx_scratch(ctx, mask_off + (size_t)L->nvalid);
        a.counts = (unsigned long long *)base;
        a.mask = (unsigned char *)(base + mask_off);
        a.mask_off = L->d_vbase;
        ck(cudaMemsetAsync(a.counts, 0, cnt_bytes, ctx->stream), "count clear");
        {
            ProfScope ps(ctx, kProfTag);
            ck(L->ops->launch_tag(a, L->ntiles, ctx->stream), "tag launch");
            ctx->launches++;
        }
        unsigned long long counts[2];
        ck(cudaMemcpyAsync(counts, a.counts, sizeof(counts), cudaMemcpyDeviceToHost, ctx->stream),
           "count download");
        ck(cudaStreamSynchronize(ctx->stream), "string tags");
        *ntags = (long long)counts[1];
    });
}

int sh_string_xi(long long string_tags, double dx, double L, double eta, double *xi) {
    if (!xi || !(eta > 0.) || !(dx > 0.) || !(L > 0.) || string_tags < 0) return SH_ERR_ARG;
    /* Cosmology::Xi with BoxToPhysical, Hubble, XiTemp and XiTime */
    const double T1 = 5.4954174414835757e+17, mpl = 1.22e19, gstar = 106.;
    const double hubble =
        std::sqrt(4. * std::pow(M_PI, 3) / 45. * gstar * std::pow(T1, 4) / std::pow(mpl, 2));
    const double length_sim = static_cast<double>(string_tags) * 2. / 3. * dx;
    const double length_phys = length_sim * eta / hubble;
    const double box_phys = L * eta / hubble;
    const double T = T1 / eta;
    const double time = 0.3012 / std::sqrt(gstar) * mpl / std::pow(T, 2);
    *xi = length_phys * std::pow(time, 2) / std::pow(box_phys, 3);
    return SH_OK;
}

int sh_average_down(sh_ctx *ctx, const sh_level *F, int which_f, sh_level *C, int which_c) {
    if (!ctx || !F || !C) return SH_ERR_ARG;
    if ((which_f != SH_NEW && which_f != SH_OLD) || (which_c != SH_NEW && which_c != SH_OLD))
        return SH_ERR_ARG;
    return guarded(ctx, [&] {
        C->version++;
        set_device(ctx);
        average_down_impl(ctx, F, which_f, C, which_c, false);
    });
}

int sh_average_down_te(sh_ctx *ctx, sh_level *F, sh_level *C) {
    if (!ctx || !F || !C) return SH_ERR_ARG;
    return guarded(ctx, [&] {
        C->version++;
        F->version++;
        set_device(ctx);
        average_down_impl(ctx, F, SH_NEW, C, SH_NEW, true);
    });
}

int sh_tag(sh_ctx *ctx, sh_level *L, int use_te, double time, int lev, double dt, double dx,
           const double *te_crit, const double *params_tag, int nparams_tag,
           const double *params_mod, int nparams_mod, uint8_t *mask_out, long long *counts_out,
           int32_t *list_out, long long list_capacity, long long *ntagged) {
    if (!ctx || !L || !mask_out) return SH_ERR_ARG;
    return guarded(ctx, [&] {
        set_device(ctx);
        require(L->nghost >= 1, "tagging reads the +1 neighbours: nghost >= 1");
        require(nparams_tag >= 0 && nparams_tag <= kMaxParams, "at most 32 tag parameters");
        require(nparams_mod >= 0 && nparams_mod <= kMaxComp, "at most 32 modifier parameters");
        require(!use_te || te_crit, "te_crit required with truncation errors");
        require(L->nvalid < (1LL << 31), "tag list indices are 32-bit");
        if (L->nvalid == 0) { /* nothing to tag (and no empty launch) */
            if (ntagged) *ntagged = 0;
            if (counts_out)
                for (int n = 0; n < 2 + L->ncomp; ++n) counts_out[n] = 0;
            return;
        }
        TagArgs a;
        std::memset(&a, 0, sizeof(a));
        a.boxes = L->d_boxes;
        a.tiles = L->d_tiles;
        a.state = state64(ctx, L, SH_NEW);
        a.te = use_te ? te_of(L) : nullptr;
        a.ncomp = L->ncomp;
        a.lev = lev;
        a.time = time;
        a.dt = dt;
        a.dx = dx;
        for (int n = 0; n < L->ncomp; ++n) a.te_crit[n] = use_te ? te_crit[n] : 0.0;
        for (int q = 0; q < nparams_tag; ++q) a.params_tag[q] = params_tag[q];
        for (int q = 0; q < nparams_mod; ++q) a.params_mod[q] = params_mod[q];
        const int nbox = (int)L->boxes.size();
        const long long nchunks = (L->nvalid + kChunk - 1) / kChunk;
        /* scratch: mask | mask offsets | counts | chunk counts | chunk bases | total | list */
        size_t off = 0;
        auto carve = [&](size_t bytes) {
            size_t o = off;
            off += (bytes + 255) & ~size_t(255);
            return o;
        };
        const size_t o_mask = carve(L->nvalid);
        const size_t o_moff = carve(nbox * sizeof(long long));
        const size_t o_cnt = carve((2 + kMaxComp) * sizeof(unsigned long long));
        const size_t o_cc = carve(nchunks * sizeof(int));
        const size_t o_cb = carve(nchunks * sizeof(long long));
        const size_t o_tot = carve(sizeof(long long));
        const size_t o_list = carve((list_out ? std::max<long long>(list_capacity, 1) : 1) *
                                    sizeof(int));
        char *base = (char *)ctx_scratch(ctx, off);
        a.mask = (unsigned char *)(base + o_mask);
        a.mask_off = (const long long *)(base + o_moff);
        a.counts = (unsigned long long *)(base + o_cnt);
        ck(cudaMemcpyAsync(base + o_moff, L->vbase.data(), nbox * sizeof(long long),
                           cudaMemcpyHostToDevice, ctx->stream),
           "mask offsets");
        ck(cudaMemsetAsync(a.counts, 0, (2 + kMaxComp) * sizeof(unsigned long long), ctx->stream),
           "count clear");
        ProfScope ps(ctx, kProfTag);
        ck(L->ops->launch_tag(a, L->ntiles, ctx->stream), "tag launch");
        ctx->launches++;
        int *cc = (int *)(base + o_cc);
        long long *cb = (long long *)(base + o_cb);
        long long *tot = (long long *)(base + o_tot);
        int *list = (int *)(base + o_list);
        tag_count_kernel<<<(unsigned)nchunks, 256, 0, ctx->stream>>>(a.mask, L->nvalid, cc);
        tag_scan_kernel<<<1, 1024, 0, ctx->stream>>>(cc, (int)nchunks, cb, tot);
        ctx->launches += 2;
        if (list_out && list_capacity > 0) {
            tag_write_kernel<<<(unsigned)nchunks, 256, 0, ctx->stream>>>(a.mask, L->nvalid, cb,
                                                                         list, list_capacity);
            ctx->launches++;
        }
        ck(cudaGetLastError(), "tag compaction launch");
        ck(cudaMemcpyAsync(mask_out, a.mask, L->nvalid, cudaMemcpyDeviceToHost, ctx->stream),
           "mask download");
        unsigned long long counts[2 + kMaxComp];
        ck(cudaMemcpyAsync(counts, a.counts, sizeof(counts), cudaMemcpyDeviceToHost, ctx->stream),
           "count download");
        long long total = 0;
        ck(cudaMemcpyAsync(&total, tot, sizeof(long long), cudaMemcpyDeviceToHost, ctx->stream),
           "tag total download");
        ck(cudaStreamSynchronize(ctx->stream), "tag");
        if (list_out && list_capacity > 0) {
            const long long nl = std::min(total, list_capacity);
            ck(cudaMemcpy(list_out, list, nl * sizeof(int), cudaMemcpyDeviceToHost),
               "tag list download");
        }
        if (ntagged) *ntagged = total;
        if (counts_out)
            for (int n = 0; n < 2 + L->ncomp; ++n) counts_out[n] = (long long)counts[n];
    });
}

int sh_tag_blocks(sh_ctx *ctx, sh_level *L, int use_te, double time, int lev, double dt,
                  double dx, const double *te_crit, const double *params_tag, int nparams_tag,
                  const double *params_mod, int nparams_mod, int block, int buffer,
                  uint8_t *blocks_out, long long *ntagged) {
    if (!ctx || !L || !blocks_out || block <= 0 || buffer < 0) return SH_ERR_ARG;
    return guarded(ctx, [&] {
        set_device(ctx);
        require(L->nghost >= 1, "tagging reads the +1 neighbours: nghost >= 1");
        require(nparams_tag >= 0 && nparams_tag <= kMaxParams, "at most 32 tag parameters");
        require(nparams_mod >= 0 && nparams_mod <= kMaxComp, "at most 32 modifier parameters");
        require(!use_te || te_crit, "te_crit required with truncation errors");
        const int N = L->dhi[0] - L->dlo[0] + 1;
        for (int d = 0; d < 3; ++d)
            require(L->dhi[d] - L->dlo[d] + 1 == N, "block tags need a cubic domain");
        require(N % block == 0, "the domain must be a whole number of blocks");
        const int nb = N / block;
        const long long nblk = (long long)nb * nb * nb;
        TagArgs a;
        std::memset(&a, 0, sizeof(a));
        a.boxes = L->d_boxes;
        a.tiles = L->d_tiles;
        a.state = state64(ctx, L, SH_NEW);
        a.te = use_te ? te_of(L) : nullptr;
        a.ncomp = L->ncomp;
        a.lev = lev;
        a.time = time;
        a.dt = dt;
        a.dx = dx;
        for (int n = 0; n < L->ncomp; ++n) a.te_crit[n] = use_te ? te_crit[n] : 0.0;
        for (int q = 0; q < nparams_tag; ++q) a.params_tag[q] = params_tag[q];
        for (int q = 0; q < nparams_mod; ++q) a.params_mod[q] = params_mod[q];
        const int nbox = (int)L->boxes.size();
        size_t off = 0;
        auto carve = [&](size_t bytes) {
            size_t o = off;
            off += (bytes + 255) & ~size_t(255);
            return o;
        };
        const size_t o_mask = carve(L->nvalid);
        const size_t o_moff = carve(nbox * sizeof(long long));
        const size_t o_cnt = carve((2 + kMaxComp) * sizeof(unsigned long long));
        const size_t o_blk = carve(nblk);
        char *base = (char *)ctx_scratch(ctx, off);
        a.mask = (unsigned char *)(base + o_mask);
        a.mask_off = (const long long *)(base + o_moff);
        a.counts = (unsigned long long *)(base + o_cnt);
        unsigned char *blk = (unsigned char *)(base + o_blk);
        ck(cudaMemcpyAsync(base + o_moff, L->vbase.data(), nbox * sizeof(long long),
                           cudaMemcpyHostToDevice, ctx->stream),
           "mask offsets");
        ck(cudaMemsetAsync(a.counts, 0, (2 + kMaxComp) * sizeof(unsigned long long), ctx->stream),
           "count clear");
        ck(cudaMemsetAsync(blk, 0, nblk, ctx->stream), "block clear");
        ProfScope ps(ctx, kProfTag);
        ck(L->ops->launch_tag(a, L->ntiles, ctx->stream), "tag launch");
        tag_blocks_kernel<<<grid_for(L->nvalid), 256, 0, ctx->stream>>>(
            L->d_boxes, L->d_vbase, nbox, L->nvalid, a.mask, L->dlo[0], L->dlo[1], L->dlo[2],
            block, buffer, nb, blk);
        ctx->launches += 2;
        ck(cudaGetLastError(), "block tag launch");
        ck(cudaMemcpyAsync(blocks_out, blk, nblk, cudaMemcpyDeviceToHost, ctx->stream),
           "block download");
        unsigned long long counts[2 + kMaxComp];
        ck(cudaMemcpyAsync(counts, a.counts, sizeof(counts), cudaMemcpyDeviceToHost, ctx->stream),
           "count download");
        ck(cudaStreamSynchronize(ctx->stream), "block tags");
        if (ntagged) *ntagged = (long long)counts[0];
    });
}

int sh_gw_spectrum(sh_ctx *ctx, const sh_level *L, const int *comps, int zero_padding,
                   int projection_type, int unbinned, double *bins_out, long long *ks_out,
                   int max_bins, int *nbins) {
    if (!ctx || !L || !bins_out || !nbins) return SH_ERR_ARG;
    return guarded(ctx, [&] {
        set_device(ctx);
        require(L->with_gw || comps, "level has no GW components; pass comps");
        require(zero_padding >= 1, "zero_padding must be >= 1");
        require(projection_type >= 1 && projection_type <= 3, "projection_type must be 1..3");
        const int N = L->dhi[0] - L->dlo[0] + 1;
        long long dv = 1;
        for (int d = 0; d < 3; ++d) {
            require(L->dhi[d] - L->dlo[d] + 1 == N, "spectrum needs a cubic domain");
            dv *= N;
        }
        require(dv == L->nvalid, "spectrum needs a level covering its whole domain");
        require((N * zero_padding) % 2 == 0, "spectrum grid size must be even");
        int c6[6];
        const int ns = L->ops->nscalars;
        const int dflt[6] = {ns + 6, ns + 9, ns + 10, ns + 7, ns + 11, ns + 8};
        for (int q = 0; q < 6; ++q) {
            c6[q] = comps ? comps[q] : dflt[q];
            require(c6[q] >= 0 && c6[q] < L->ncomp, "component index out of range");
        }
        const size_t sbytes = gw_scratch_bytes(N, zero_padding);
        const int P = N * zero_padding;
        const size_t maxbins = (size_t)3 * (P / 2 + 1) * (P / 2 + 1) + 16;
        char *base = (char *)ctx_scratch(ctx, sbytes + maxbins * sizeof(double) + 256);
        double *bins_dev = (double *)(base + ((sbytes + 255) & ~size_t(255)));
        int nb = 0;
        std::string err;
        ProfScope ps(ctx, kProfGw);
        cudaError_t e = gw_spectrum_device(ctx->gw, ctx->stream, L->d_boxes, L->d_vbase,
                                           (int)L->boxes.size(), L->nvalid, L->ncomp,
                                           state64(ctx, L, SH_NEW), c6, N, L->dlo, zero_padding,
                                           projection_type, unbinned, (double *)base, bins_dev,
                                           &nb, &ctx->launches, err);
        if (!err.empty()) throw ShError(SH_ERR_CUDA, err);
        ck(e, "gw spectrum");
        *nbins = nb;
        require(nb <= max_bins, "bins_out too small");
        ck(cudaMemcpyAsync(bins_out, bins_dev, nb * sizeof(double), cudaMemcpyDeviceToHost,
                           ctx->stream),
           "spectrum download");
        ck(cudaStreamSynchronize(ctx->stream), "gw spectrum");
        if (ks_out) std::copy(ctx->gw.ks().begin(), ctx->gw.ks().end(), ks_out);
    });
}

int sh_evolve_periodic(sh_ctx *ctx, int project, int integrator, const double *tableau,
                       int nstages, int N, int max_grid, int nghost, int ncomp, int with_gw,
                       const double *state_in, const double *init_new, double *state_out,
                       double t0, double dt, double dx, int nsteps, const double *params,
                       int nparams, const double *gw_params, int ngw, int ko_order,
                       const double *ko_strength) {
    if (!ctx || !state_in || !state_out || N <= 0 || nsteps < 0) return SH_ERR_ARG;
    int nc = 0;
    int rc = sh_project_ncomp(project, with_gw, &nc, nullptr);
    if (rc != SH_OK) return rc;
    if (nc != ncomp) {
        ctx->err = "ncomp does not match the project";
        return SH_ERR_ARG;
    }
    std::vector<sh_box> boxes;
    const int mg = (max_grid <= 0 || max_grid >= N) ? N : max_grid;
    for (int z = 0; z < N; z += mg)
        for (int y = 0; y < N; y += mg)
            for (int x = 0; x < N; x += mg)
                boxes.push_back(sh_box{{x, y, z},
                                       {std::min(x + mg, N) - 1, std::min(y + mg, N) - 1,
                                        std::min(z + mg, N) - 1}});
    const int dlo[3] = {0, 0, 0}, dhi[3] = {N - 1, N - 1, N - 1};
    sh_level *L = nullptr;
    rc = sh_level_create(ctx, project, with_gw, dlo, dhi, boxes.data(), (int)boxes.size(), nghost,
                         &L);
    if (rc != SH_OK) return rc;
    rc = sh_level_write(ctx, L, SH_NEW, 0, state_in);
    if (rc == SH_OK && init_new) rc = sh_level_write(ctx, L, SH_OLD, 0, init_new);
    if (rc == SH_OK) sh_level_set_time(L, SH_NEW, t0, 0);
    for (int s = 0; s < nsteps && rc == SH_OK; ++s)
        rc = sh_level_advance(ctx, L, integrator, tableau, nstages, dt, dx, params, nparams,
                              gw_params, ngw, ko_order, ko_strength, 0);
    if (rc == SH_OK) rc = sh_level_read(ctx, L, SH_NEW, 0, state_out);
    sh_level_destroy(ctx, L);
    return rc;
}

} /* extern "C" */

/* ---- allocation-free tagging ------------------------------------------------
 * Working memory of sh_tag_static: one fixed array per GPU, laid out as
 *   [0, 512)                counters (total, user, per component)
 *   [512, 768)              number of tagged cells
 *   [768, 5120)             per-chunk tag counts (up to 1024 chunks)
 *   [5120, 16384)           per-chunk list offsets
 *   [16384, +4 MiB)         tag mask, one byte per valid cell
 *   [16384 + 4 MiB, +16 MiB) tag list, one int per cell
 */
namespace {
constexpr size_t kStaticCountsOff = 0;
constexpr size_t kStaticTotalOff = 512;
constexpr size_t kStaticChunkCntOff = 768;
constexpr size_t kStaticChunkBaseOff = 5120;
constexpr size_t kStaticMaskOff = 16384;
constexpr size_t kStaticListOff = kStaticMaskOff + (size_t)SH_TAG_STATIC_MAX_CELLS;
constexpr size_t kStaticBytes = kStaticListOff + (size_t)SH_TAG_STATIC_MAX_CELLS * sizeof(int);
static_assert((SH_TAG_STATIC_MAX_CELLS + kChunk - 1) / kChunk * sizeof(int) <=
                  kStaticChunkBaseOff - kStaticChunkCntOff,
              "chunk counts do not fit");
static_assert((SH_TAG_STATIC_MAX_CELLS + kChunk - 1) / kChunk * sizeof(long long) <=
                  kStaticMaskOff - kStaticChunkBaseOff,
              "chunk offsets do not fit");

static __device__ __align__(256) unsigned char g_tag_static[kStaticBytes];

constexpr int kMaxDevices = 64;
std::mutex g_tag_static_mutex;
void *g_tag_static_ptr[kMaxDevices] = {nullptr};

/* Device address of g_tag_static on the context's device (looked up once per
 * device, with that device current). */
unsigned char *tag_static_base(sh_ctx *ctx) {
    require(ctx->device >= 0 && ctx->device < kMaxDevices, "device index out of range");
    std::lock_guard<std::mutex> lock(g_tag_static_mutex);
    if (!g_tag_static_ptr[ctx->device]) {
        void *p = nullptr;
        ck(cudaGetSymbolAddress(&p, g_tag_static), "cudaGetSymbolAddress(g_tag_static)");
        g_tag_static_ptr[ctx->device] = p;
    }
    return (unsigned char *)g_tag_static_ptr[ctx->device];
}
} // namespace

extern "C" int sh_tag_static(sh_ctx *ctx, sh_level *L, int use_te, double time, int lev,
                             double dt, double dx, const double *te_crit,
                             const double *params_tag, int nparams_tag,
                             const double *params_mod, int nparams_mod, uint8_t *mask_out,
                             long long *counts_out, int32_t *list_out, long long list_capacity,
                             long long *ntagged) {
    if (!ctx || !L || !mask_out) return SH_ERR_ARG;
    return guarded(ctx, [&] {
        set_device(ctx);
        require(L->nvalid <= SH_TAG_STATIC_MAX_CELLS,
                "sh_tag_static: level has " + std::to_string(L->nvalid) +
                    " valid cells, more than SH_TAG_STATIC_MAX_CELLS (" +
                    std::to_string(SH_TAG_STATIC_MAX_CELLS) + ")");
        require(L->nghost >= 1, "tagging reads the +1 neighbours: nghost >= 1");
        require(nparams_tag >= 0 && nparams_tag <= kMaxParams, "at most 32 tag parameters");
        require(nparams_mod >= 0 && nparams_mod <= kMaxComp, "at most 32 modifier parameters");
        require(!use_te || te_crit, "te_crit required with truncation errors");
        if (L->nvalid == 0) { /* nothing to tag (and no empty launch) */
            if (ntagged) *ntagged = 0;
            if (counts_out)
                for (int n = 0; n < 2 + L->ncomp; ++n) counts_out[n] = 0;
            return;
        }
        unsigned char *base = tag_static_base(ctx);
        TagArgs a;
        std::memset(&a, 0, sizeof(a));
        a.boxes = L->d_boxes;
        a.tiles = L->d_tiles;
        require_fp64(L, "tagging without allocations");
        a.state = L->buf[SH_NEW];
        a.te = use_te ? L->buf[SH_OLD] : nullptr;
        a.ncomp = L->ncomp;
        a.lev = lev;
        a.time = time;
        a.dt = dt;
        a.dx = dx;
        for (int n = 0; n < L->ncomp; ++n) a.te_crit[n] = use_te ? te_crit[n] : 0.0;
        for (int q = 0; q < nparams_tag; ++q) a.params_tag[q] = params_tag[q];
        for (int q = 0; q < nparams_mod; ++q) a.params_mod[q] = params_mod[q];
        a.mask = base + kStaticMaskOff;
        a.mask_off = L->d_vbase; /* prefix sums of valid cells = mask offsets */
        a.counts = (unsigned long long *)(base + kStaticCountsOff);
        const long long nchunks = (L->nvalid + kChunk - 1) / kChunk;
        int *cc = (int *)(base + kStaticChunkCntOff);
        long long *cb = (long long *)(base + kStaticChunkBaseOff);
        long long *tot = (long long *)(base + kStaticTotalOff);
        int *list = (int *)(base + kStaticListOff);
        const long long dev_cap =
            std::min<long long>(list_out ? list_capacity : 0, SH_TAG_STATIC_MAX_CELLS);
        /* the array keeps the previous call's contents: the counters must
         * start at zero (mask, chunk counts and offsets are fully rewritten) */
        ck(cudaMemsetAsync(base + kStaticCountsOff, 0, kStaticChunkCntOff, ctx->stream),
           "static counters clear");
        ck(L->ops->launch_tag(a, L->ntiles, ctx->stream), "tag launch");
        ctx->launches++;
        tag_count_kernel<<<(unsigned)nchunks, 256, 0, ctx->stream>>>(a.mask, L->nvalid, cc);
        tag_scan_kernel<<<1, 1024, 0, ctx->stream>>>(cc, (int)nchunks, cb, tot);
        ctx->launches += 2;
        if (dev_cap > 0) {
            tag_write_kernel<<<(unsigned)nchunks, 256, 0, ctx->stream>>>(a.mask, L->nvalid, cb,
                                                                         list, dev_cap);
            ctx->launches++;
        }
        ck(cudaGetLastError(), "tag compaction launch");
        ck(cudaMemcpyAsync(mask_out, a.mask, L->nvalid, cudaMemcpyDeviceToHost, ctx->stream),
           "mask download");
        unsigned long long counts[2 + kMaxComp];
        ck(cudaMemcpyAsync(counts, a.counts, sizeof(counts), cudaMemcpyDeviceToHost, ctx->stream),
           "count download");
        long long total = 0;
        ck(cudaMemcpyAsync(&total, tot, sizeof(long long), cudaMemcpyDeviceToHost, ctx->stream),
           "tag total download");
        ck(cudaStreamSynchronize(ctx->stream), "tag");
        if (dev_cap > 0) {
            const long long nl = std::min(total, dev_cap);
            ck(cudaMemcpyAsync(list_out, list, nl * sizeof(int), cudaMemcpyDeviceToHost,
                               ctx->stream),
               "tag list download");
            ck(cudaStreamSynchronize(ctx->stream), "tag list");
        }
        if (ntagged) *ntagged = total;
        if (counts_out)
            for (int n = 0; n < 2 + L->ncomp; ++n) counts_out[n] = (long long)counts[n];
    });
}
