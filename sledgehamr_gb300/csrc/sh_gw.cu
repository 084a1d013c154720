/* Gravitational-wave spectrum (GravitationalWaves::ComputeSpectrum,
 * source/gravitational_waves.cpp:52-322) and the spectrum binning data
 * (Sledgehamr::ReadSpectrumKs/ReadProj, sledgehamr.cpp:554-615, whose
 * arrays pySledgehamr/Sledgehamr.py:7-27 generates).
 *
 * Pipeline on the device, per call:
 *   1. pack each of the six selected tensor components of time level NEW
 *      into a (pN)^3 real array, zero padded (utils::Fft, fft.h:143-262);
 *   2. cuFFT D2Z, unnormalised, giving (pN/2+1) x pN x pN complex values
 *      with the x index halved;
 *   3. projection kernel: for every k-cell the TT-projected power
 *        multpl * sum_{ijlm} L_ijlm (Re u_ij Re u_lm + Im u_ij Im u_lm),
 *        L_ijlm = P_il P_jm - 1/2 P_ij P_lm,  P_ij = delta_ij - k_i k_j/|k|^2
 *      with k_i = index_to_k[index] and multpl = 1 for a in {0, pN/2}, else
 *      2.  The 81-term sum is evaluated in the equivalent contracted form
 *        Re sum_lm (P U P)_lm conj(U_lm) - 1/2 |sum_ij P_ij U_ij|^2
 *      (U the symmetric complex 3x3 tensor), about 150 FP64 operations per
 *      cell instead of the reference's 81 x 4 projections;
 *   4. deterministic binning: every bin sums its cells in ascending cell
 *      order with a fixed warp tree (bin lists built once per grid size and
 *      cached), then divides by (pN)^6.  Binned mode uses bin
 *      round(|n|); unbinned mode the position of |n|^2 in the sorted list of
 *      unique k^2.
 */
#include <cufft.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include <functional>
#include <new>

#ifdef _OPENMP
#include <omp.h>
#endif

#include "sh_gw.h"
#include "sledgehamr_gb300.h"

namespace sh {

std::vector<long long> unique_k2_host(int dim) {
    std::vector<long long> sq;
    for (int a = 0; a < dim; ++a) {
        long long f = a < (dim + 1) / 2 ? a : a - dim;
        sq.push_back(f * f);
    }
    std::sort(sq.begin(), sq.end());
    sq.erase(std::unique(sq.begin(), sq.end()), sq.end());
    const long long maxs = 3 * sq.back();
    std::vector<char> hit((size_t)maxs + 1, 0);
    for (long long x : sq)
        for (long long y : sq)
            for (long long z : sq) hit[(size_t)(x + y + z)] = 1;
    std::vector<long long> out;
    for (long long v = 0; v <= maxs; ++v)
        if (hit[(size_t)v]) out.push_back(v);
    return out;
}

std::vector<double> index_to_k_host(int N, int type) {
    std::vector<double> r(N);
    for (int a = 0; a < N; ++a) {
        double nt = (double)a;
        if ((double)a - N > -N / 2.0 - 1) nt -= N;
        const double x = 2. * M_PI / N * nt;
        if (type == 1) r[a] = std::sin(x);
        else if (type == 2) r[a] = (8. * std::sin(x) - std::sin(2. * x)) / 6.;
        else r[a] = (45. * std::sin(x) - 9. * std::sin(2. * x) + std::sin(3. * x)) / 30.;
    }
    return r;
}

namespace {

/* Pack components ca (real part) and cb (imaginary part) of a level buffer
 * (valid cells, any box layout covering [0,N)^3) into the first N^3 block
 * of a zero-initialised complex (pN)^3 array. */
__global__ void gw_pack_kernel(const BoxDev *boxes, const long long *vbase, int nbox,
                               long long nvalid, int ncomp, int ca, int cb, const double *buf,
                               double2 *dst, int P, int dlo0, int dlo1, int dlo2) {
    for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < nvalid;
         v += (long long)gridDim.x * blockDim.x) {
        int lo = 0, hi = nbox - 1;
        while (lo < hi) {
            int mid = (lo + hi + 1) >> 1;
            if (vbase[mid] <= v) lo = mid;
            else hi = mid - 1;
        }
        const BoxDev &b = boxes[lo];
        const long long lv = v - vbase[lo];
        const int vx = b.hi[0] - b.lo[0] + 1, vy = b.hi[1] - b.lo[1] + 1;
        const int i = b.lo[0] + (int)(lv % vx);
        const int j = b.lo[1] + (int)((lv / vx) % vy);
        const int k = b.lo[2] + (int)(lv / ((long long)vx * vy));
        const long long bi = b.off * ncomp + (i - b.glo[0]) +
                             (long long)(j - b.glo[1]) * b.gdim[0] +
                             (long long)(k - b.glo[2]) * b.gdim[0] * b.gdim[1];
        dst[((long long)(k - dlo2) * P + (j - dlo1)) * P + (i - dlo0)] =
            make_double2(buf[bi + (long long)ca * b.gvol], buf[bi + (long long)cb * b.gvol]);
    }
}

/* Per k-cell TT power, four times unnormalised; layout ((c*P + b)*H + a).
 *
 * The six real components arrive in pairs, each pair transformed as one
 * complex field Z = u + i u' (a complex-to-complex transform costs what the
 * two real-to-complex ones cost together, and runs faster than cuFFT's
 * real-to-complex pass); with conj Z(-k) the conjugate of the transform's
 * value at -k,
 *     2 U(k) = Z(k) + conj Z(-k),   2 U'(k) = -i (Z(k) - conj Z(-k)),
 * and the factor 2 (4 in the power) is taken out by the bins' scale.
 *
 * The reference sums Lambda_ijlm(k) u_lm conj(u_ij) over i,j,l,m
 * (gravitational_waves.cpp:251-276) with Lambda_ijlm = P_il P_jm -
 * 1/2 P_ij P_lm and P = 1 - k k^T / k^2 (gravitational_waves.h:101-133).  As
 * Lambda is the TT projector this equals |W|^2 - 1/2 |tr W|^2 with
 * W = P U P, which is formed here without the 3x3 products: with v = U k,
 * s = k.v and w = v / k^2 - (s / 2k^4) k,
 *     W = U - k w^T - w k^T,
 * about 100 FP64 operations per cell instead of the ~170 of P U P.  W is
 * the projected tensor itself, so |W|^2 carries rounding of the order of
 * eps |U| |W| (not eps |U|^2), as the explicit form does. */
template <class C>
__device__ __forceinline__ void split_pair(C z, C m, C &u, C &v) {
    u.x = z.x + m.x;
    u.y = z.y - m.y;
    v.x = z.y + m.y;
    v.y = m.x - z.x;
}

/* C, R: double2, double for FP64 transforms; float2, float for FP32 ones
 * (the per-cell value is widened to FP64 for the bin sums). */
template <class C, class R>
__global__ void gw_project_kernel(const C *__restrict__ Z0, const C *__restrict__ Z1,
                                  const C *__restrict__ Z2, const R *__restrict__ index_to_k,
                                  int P, double *out) {
    const int H = P / 2 + 1;
    const long long n = (long long)H * P * P;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n;
         e += (long long)gridDim.x * blockDim.x) {
        const int a = (int)(e % H);
        const int b = (int)((e / H) % P);
        const int c = (int)(e / ((long long)H * P));
        if (a == 0 && b == 0 && c == 0) {
            out[e] = 0.;
            continue;
        }
        const long long f = ((long long)c * P + b) * P + a;
        const long long g =
            ((long long)(c ? P - c : 0) * P + (b ? P - b : 0)) * P + (a ? P - a : 0);
        /* twice the transforms of the slots xx xy xz yy yz zz */
        C s6[6];
        split_pair(Z0[f], Z0[g], s6[0], s6[1]);
        split_pair(Z1[f], Z1[g], s6[2], s6[3]);
        split_pair(Z2[f], Z2[g], s6[4], s6[5]);
        R k[3] = {index_to_k[a], index_to_k[b], index_to_k[c]};
        R inv;
        if constexpr (sizeof(R) == 4) {
            /* FP32: the unit vector k / |k| (near the Nyquist planes |k| is
             * ~1e-16, and 1 / |k|^4 would overflow) */
            const R rn = rsqrtf(k[0] * k[0] + k[1] * k[1] + k[2] * k[2]);
            k[0] *= rn;
            k[1] *= rn;
            k[2] *= rn;
            inv = (R)1;
        } else {
            inv = (R)1 / (k[0] * k[0] + k[1] * k[1] + k[2] * k[2]);
        }
        const int slot[3][3] = {{0, 1, 2}, {1, 3, 4}, {2, 4, 5}};
        C v[3];
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            v[i].x = s6[slot[i][0]].x * k[0] + s6[slot[i][1]].x * k[1] + s6[slot[i][2]].x * k[2];
            v[i].y = s6[slot[i][0]].y * k[0] + s6[slot[i][1]].y * k[1] + s6[slot[i][2]].y * k[2];
        }
        const R sx = k[0] * v[0].x + k[1] * v[1].x + k[2] * v[2].x;
        const R sy = k[0] * v[0].y + k[1] * v[1].y + k[2] * v[2].y;
        const R h = (R)0.5 * inv * inv;
        C w[3];
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            w[i].x = inv * v[i].x - h * sx * k[i];
            w[i].y = inv * v[i].y - h * sy * k[i];
        }
        R first = 0, tr_re = 0, tr_im = 0;
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = i; j < 3; ++j) {
                const C u = s6[slot[i][j]];
                const R re = u.x - (k[i] * w[j].x + w[i].x * k[j]);
                const R im = u.y - (k[i] * w[j].y + w[i].y * k[j]);
                const R wt = i == j ? (R)1 : (R)2;
                first += wt * (re * re + im * im);
                if (i == j) {
                    tr_re += re;
                    tr_im += im;
                }
            }
        const R multpl = (a == 0 || a == P / 2) ? (R)1 : (R)2;
        out[e] = (double)(multpl * (first - (R)0.5 * (tr_re * tr_re + tr_im * tr_im)));
    }
}

/* Deterministic sums of the bins' cells, scaled: a block of kBinThreads
 * threads per bin (blocks loop over bins), thread t summing the cells t,
 * t + kBinThreads, ... of the bin in order, then a fixed warp-shuffle and
 * shared-memory tree.  A whole block per bin keeps the 85 K-cell bins of a
 * 384^3 binned spectrum from running on a few hundred warps. */
constexpr int kBinThreads = 256;
__global__ void __launch_bounds__(kBinThreads)
    gw_bin_kernel(const double *val, const long long *bin_off, const int *bin_cells, int nbins,
                  double scale, double *bins) {
    __shared__ double part[kBinThreads / 32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int bin = blockIdx.x; bin < nbins; bin += gridDim.x) {
        const long long o0 = bin_off[bin], o1 = bin_off[bin + 1];
        double s = 0.;
        for (long long q = o0 + threadIdx.x; q < o1; q += kBinThreads) s += val[bin_cells[q]];
        for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
        if (lane == 0) part[wid] = s;
        __syncthreads();
        if (wid == 0) {
            double t = lane < kBinThreads / 32 ? part[lane] : 0.;
            for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
            if (lane == 0) bins[bin] = t * scale;
        }
        __syncthreads();
    }
}

void launch_bins(const double *vals, const GwBins &g, double scale, double *bins_dev,
                 cudaStream_t stream) {
    const int nb = (int)g.ks.size();
    const int grid = std::max(1, std::min(nb, 152 * 8));
    gw_bin_kernel<<<grid, kBinThreads, 0, stream>>>(vals, g.d_off, g.d_cells, nb, scale,
                                                    bins_dev);
}

/* multpl |F|^2 per k-cell of a scalar field's R2C transform, with
 * |F| = sqrt(re^2 + im^2) as utils::Fft forms it (fft.h:244-250). */
__global__ void scalar_power_kernel(const double2 *F, int P, double *out) {
    const int H = P / 2 + 1;
    const long long n = (long long)H * P * P;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n;
         e += (long long)gridDim.x * blockDim.x) {
        const int a = (int)(e % H);
        const double multpl = (a == 0 || a == P / 2) ? 1. : 2.;
        const double2 z = F[e];
        const double absF = sqrt(__dadd_rn(__dmul_rn(z.x, z.x), __dmul_rn(z.y, z.y)));
        out[e] = multpl * absF * absF;
    }
}

} // namespace

/* Builds (or reuses) the bin lists of a P^3 spectrum. */
void GwCache::prepare(int P, int unbinned, int projection_type) {
    ++clock;
    for (GwBins &b : bins)
        if (b.P == P && b.unbinned == unbinned && b.projection_type == projection_type) {
            b.used = clock;
            cur = &b;
            return;
        }
    if ((int)bins.size() >= kMaxBins) { /* evict the least recently used */
        size_t lru = 0;
        for (size_t q = 1; q < bins.size(); ++q)
            if (bins[q].used < bins[lru].used) lru = q;
        cudaFree(bins[lru].d_off);
        cudaFree(bins[lru].d_cells);
        cudaFree(bins[lru].d_itk);
        cudaFree(bins[lru].d_itk32);
        bins.erase(bins.begin() + lru);
    }
    GwBins g;
    g.P = P;
    g.unbinned = unbinned;
    g.projection_type = projection_type;
    g.used = clock;
    const int H = P / 2 + 1;
    const long long ncell = (long long)H * P * P;
    if (unbinned) {
        g.ks = unique_k2_host(P);
    } else {
        for (int k = 0; k <= std::sqrt(3.) / 2. * static_cast<double>(P) + .5; ++k)
            g.ks.push_back((long long)k * k);
    }
    const int nb = (int)g.ks.size();
    const long long maxsq = 3LL * (P / 2) * (P / 2);
    std::vector<int> lut((size_t)maxsq + 1, -1);
    if (unbinned) {
        for (int q = 0; q < nb; ++q) lut[(size_t)g.ks[q]] = q;
    } else {
        for (long long sq = 0; sq <= maxsq; ++sq) {
            long long r = (long long)std::llround(std::sqrt((double)sq));
            /* round(sqrt(sq)) == r  <=>  r^2 - r < sq <= r^2 + r */
            while (r * r + r < sq) ++r;
            while (r > 0 && r * r - r >= sq) --r;
            lut[(size_t)sq] = (int)r;
        }
    }
    auto bin_of = [&](long long e) {
        const int a = (int)(e % H), b = (int)((e / H) % P), c = (int)(e / ((long long)H * P));
        const long long li = a >= P / 2 ? a - P : a;
        const long long lj = b >= P / 2 ? b - P : b;
        const long long lk = c >= P / 2 ? c - P : c;
        return lut[(size_t)(li * li + lj * lj + lk * lk)];
    };
    /* stable counting sort over contiguous chunks of cells, one per thread */
    int nt = 1;
#ifdef _OPENMP
    nt = std::max(1, std::min(omp_get_max_threads(), 64));
#endif
    const long long chunk = (ncell + nt - 1) / nt;
    std::vector<long long> cnt((size_t)nt * nb, 0);
#pragma omp parallel for num_threads(nt) schedule(static, 1)
    for (int t = 0; t < nt; ++t) {
        long long *c = cnt.data() + (size_t)t * nb;
        const long long e1 = std::min(ncell, (t + 1) * chunk);
        for (long long e = t * chunk; e < e1; ++e) c[bin_of(e)]++;
    }
    std::vector<long long> off(nb + 1, 0);
    for (int q = 0; q < nb; ++q) {
        long long run = off[q];
        for (int t = 0; t < nt; ++t) {
            const long long c = cnt[(size_t)t * nb + q];
            cnt[(size_t)t * nb + q] = run; /* start of thread t's cells in bin q */
            run += c;
        }
        off[q + 1] = run;
    }
    std::vector<int> cells((size_t)ncell);
#pragma omp parallel for num_threads(nt) schedule(static, 1)
    for (int t = 0; t < nt; ++t) {
        long long *pos = cnt.data() + (size_t)t * nb;
        const long long e1 = std::min(ncell, (t + 1) * chunk);
        for (long long e = t * chunk; e < e1; ++e) cells[(size_t)pos[bin_of(e)]++] = (int)e;
    }
    std::vector<double> itk = index_to_k_host(P, projection_type);
    std::vector<float> itk32(itk.begin(), itk.end());
    if (cudaMalloc(&g.d_off, off.size() * sizeof(long long)) != cudaSuccess ||
        cudaMalloc(&g.d_cells, cells.size() * sizeof(int)) != cudaSuccess ||
        cudaMalloc(&g.d_itk, itk.size() * sizeof(double)) != cudaSuccess ||
        cudaMalloc(&g.d_itk32, itk32.size() * sizeof(float)) != cudaSuccess) {
        cudaGetLastError();
        cudaFree(g.d_off);
        cudaFree(g.d_cells);
        cudaFree(g.d_itk);
        cudaFree(g.d_itk32);
        throw std::bad_alloc();
    }
    cudaMemcpy(g.d_off, off.data(), off.size() * sizeof(long long), cudaMemcpyHostToDevice);
    cudaMemcpy(g.d_cells, cells.data(), cells.size() * sizeof(int), cudaMemcpyHostToDevice);
    cudaMemcpy(g.d_itk, itk.data(), itk.size() * sizeof(double), cudaMemcpyHostToDevice);
    cudaMemcpy(g.d_itk32, itk32.data(), itk32.size() * sizeof(float), cudaMemcpyHostToDevice);
    bins.push_back(std::move(g));
    cur = &bins.back();
}

bool GwCache::plan(int P, int kind, cufftHandle *out) {
    ++clock;
    for (Plan &p : plans)
        if (p.P == P && p.kind == kind) {
            p.used = clock;
            *out = p.h;
            return true;
        }
    if ((int)plans.size() >= kMaxPlans) {
        size_t lru = 0;
        for (size_t q = 1; q < plans.size(); ++q)
            if (plans[q].used < plans[lru].used) lru = q;
        cufftDestroy(plans[lru].h);
        plans.erase(plans.begin() + lru);
    }
    Plan p;
    p.P = P;
    p.kind = kind;
    p.used = clock;
    if (cufftCreate(&p.h) != CUFFT_SUCCESS) return false;
    long long n[3] = {P, P, P};
    const long long dist = (long long)P * P * P;
    size_t work = 0;
    const cufftResult r =
        kind == kPlanD2Z
            ? cufftMakePlanMany64(p.h, 3, n, nullptr, 1, 0, nullptr, 1, 0, CUFFT_D2Z, 1, &work)
            : cufftMakePlanMany64(p.h, 3, n, nullptr, 1, dist, nullptr, 1, dist,
                                  kind == kPlanZ2Z3 ? CUFFT_Z2Z : CUFFT_C2C, 3, &work);
    if (r != CUFFT_SUCCESS) {
        cufftDestroy(p.h);
        return false;
    }
    plans.push_back(p);
    *out = p.h;
    return true;
}

void GwCache::release() {
    for (GwBins &b : bins) {
        cudaFree(b.d_off);
        cudaFree(b.d_cells);
        cudaFree(b.d_itk);
        cudaFree(b.d_itk32);
    }
    bins.clear();
    for (Plan &p : plans) cufftDestroy(p.h);
    plans.clear();
    cur = nullptr;
}

cudaError_t gw_spectrum_packed(GwCache &cache, cudaStream_t stream, int P, int N,
                               int projection_type, int unbinned, double *scratch,
                               double *bins_dev, int *nbins, long long *launches,
                               std::string &err,
                               const std::function<void(int, double2 *)> &pack) {
    cache.prepare(P, unbinned, projection_type);
    const int H = P / 2 + 1;
    const long long nfull = (long long)P * P * P;
    const long long nhalf = (long long)H * P * P;
    cufftHandle plan;
    if (!cache.plan(P, GwCache::kPlanZ2Z3, &plan)) {
        err = "cuFFT plan of three P^3 complex transforms failed";
        return cudaErrorUnknown;
    }
    cufftSetStream(plan, stream);
    /* scratch: three complex P^3 arrays (component pairs) | per-cell values */
    double2 *Z = (double2 *)scratch;
    double *vals = (double *)(Z + 3 * nfull);
    /* the pack covers all of P^3 without zero padding */
    if (P != N) cudaMemsetAsync(Z, 0, 3 * nfull * sizeof(double2), stream);
    for (int p = 0; p < 3; ++p) {
        pack(p, Z + p * nfull);
        (*launches)++;
    }
    if (cufftExecZ2Z(plan, (cufftDoubleComplex *)Z, (cufftDoubleComplex *)Z, CUFFT_FORWARD) !=
        CUFFT_SUCCESS) {
        err = "cufftExecZ2Z failed";
        return cudaErrorUnknown;
    }
    int g = (int)std::min<long long>((nhalf + 255) / 256, 152LL * 32);
    gw_project_kernel<double2, double><<<std::max(g, 1), 256, 0, stream>>>(
        Z, Z + nfull, Z + 2 * nfull, cache.cur->d_itk, P, vals);
    (*launches)++;
    const int nb = (int)cache.ks().size();
    /* 1/P^6, and 1/4 for the pairs' factor 2 (exact) */
    const double scale = 0.25 / std::pow((double)P, 6);
    launch_bins(vals, *cache.cur, scale, bins_dev, stream);
    (*launches)++;
    *nbins = nb;
    return cudaGetLastError();
}

cudaError_t gw_spectrum_packed32(GwCache &cache, cudaStream_t stream, int P, int N,
                                 int projection_type, int unbinned, double *scratch,
                                 double *bins_dev, int *nbins, long long *launches,
                                 std::string &err,
                                 const std::function<void(int, float2 *)> &pack) {
    cache.prepare(P, unbinned, projection_type);
    const int H = P / 2 + 1;
    const long long nfull = (long long)P * P * P;
    const long long nhalf = (long long)H * P * P;
    cufftHandle plan;
    if (!cache.plan(P, GwCache::kPlanC2C3, &plan)) {
        err = "cuFFT plan of three P^3 FP32 complex transforms failed";
        return cudaErrorUnknown;
    }
    cufftSetStream(plan, stream);
    /* scratch: three complex FP32 P^3 arrays (component pairs) | per-cell values */
    float2 *Z = (float2 *)scratch;
    double *vals = (double *)(Z + 3 * nfull);
    if (P != N) cudaMemsetAsync(Z, 0, 3 * nfull * sizeof(float2), stream);
    for (int p = 0; p < 3; ++p) {
        pack(p, Z + p * nfull);
        (*launches)++;
    }
    if (cufftExecC2C(plan, (cufftComplex *)Z, (cufftComplex *)Z, CUFFT_FORWARD) != CUFFT_SUCCESS) {
        err = "cufftExecC2C failed";
        return cudaErrorUnknown;
    }
    int g = (int)std::min<long long>((nhalf + 255) / 256, 152LL * 32);
    gw_project_kernel<float2, float><<<std::max(g, 1), 256, 0, stream>>>(
        Z, Z + nfull, Z + 2 * nfull, cache.cur->d_itk32, P, vals);
    (*launches)++;
    const int nb = (int)cache.ks().size();
    const double scale = 0.25 / std::pow((double)P, 6);
    launch_bins(vals, *cache.cur, scale, bins_dev, stream);
    (*launches)++;
    *nbins = nb;
    return cudaGetLastError();
}

cudaError_t scalar_spectrum_packed(GwCache &cache, cudaStream_t stream, int P, double pre,
                                   double *scratch, double *bins_dev, int *nbins,
                                   long long *launches, std::string &err,
                                   const std::function<void(double *)> &pack) {
    /* unbinned bins of k^2 (the k-map of the entry is not used) */
    cache.prepare(P, 1, 2);
    const int H = P / 2 + 1;
    const long long nreal = (long long)P * P * P;
    const long long ncplx = (long long)H * P * P;
    cufftHandle plan;
    if (!cache.plan(P, GwCache::kPlanD2Z, &plan)) {
        err = "cuFFT plan of a P^3 real-to-complex transform failed";
        return cudaErrorUnknown;
    }
    cufftSetStream(plan, stream);
    double *real = scratch;
    double2 *cplx = (double2 *)(scratch + nreal);
    double *vals = (double *)(cplx + ncplx);
    cudaMemsetAsync(real, 0, nreal * sizeof(double), stream);
    pack(real);
    (*launches)++;
    if (cufftExecD2Z(plan, real, (cufftDoubleComplex *)cplx) != CUFFT_SUCCESS) {
        err = "cufftExecD2Z failed";
        return cudaErrorUnknown;
    }
    int g = (int)std::min<long long>((ncplx + 255) / 256, 152LL * 32);
    scalar_power_kernel<<<std::max(g, 1), 256, 0, stream>>>(cplx, P, vals);
    (*launches)++;
    const int nb = (int)cache.ks().size();
    launch_bins(vals, *cache.cur, pre, bins_dev, stream);
    (*launches)++;
    *nbins = nb;
    return cudaGetLastError();
}

cudaError_t gw_spectrum_device(GwCache &cache, cudaStream_t stream, const BoxDev *boxes,
                               const long long *vbase, int nbox, long long nvalid, int ncomp,
                               const double *buf, const int comps[6], int N, const int dlo[3],
                               int zero_padding, int projection_type, int unbinned,
                               double *scratch, double *bins_dev, int *nbins, long long *launches,
                               std::string &err) {
    const int P = N * zero_padding;
    return gw_spectrum_packed(
        cache, stream, P, N, projection_type, unbinned, scratch, bins_dev, nbins, launches, err,
        [&](int p, double2 *dst) {
            int g = (int)std::min<long long>((nvalid + 255) / 256, 152LL * 32);
            gw_pack_kernel<<<std::max(g, 1), 256, 0, stream>>>(
                boxes, vbase, nbox, nvalid, ncomp, comps[2 * p], comps[2 * p + 1], buf, dst, P,
                dlo[0], dlo[1], dlo[2]);
        });
}

size_t gw_scratch_bytes(int N, int zero_padding) {
    const long long P = (long long)N * zero_padding;
    const long long H = P / 2 + 1;
    /* GW: three complex P^3 arrays + per-cell values; scalar spectra: a real
     * P^3 array + a half-spectrum + per-cell values (smaller) */
    return (size_t)(6 * P * P * P + H * P * P) * sizeof(double);
}

} // namespace sh

extern "C" {

int sh_spectrum_bins(int dim, long long *out, int capacity, int *nbins) {
    if (dim <= 0 || !nbins) return SH_ERR_ARG;
    std::vector<long long> v = sh::unique_k2_host(dim);
    *nbins = (int)v.size();
    if (!out) return SH_OK;
    if ((int)v.size() > capacity) return SH_ERR_ARG;
    std::copy(v.begin(), v.end(), out);
    return SH_OK;
}

int sh_index_to_k(int dim, int projection_type, double *out) {
    if (dim <= 0 || !out || projection_type < 1 || projection_type > 3) return SH_ERR_ARG;
    std::vector<double> v = sh::index_to_k_host(dim, projection_type);
    std::copy(v.begin(), v.end(), out);
    return SH_OK;
}

} /* extern "C" */
