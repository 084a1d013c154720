/* Internal interface of the GW spectrum module (sh_gw.cu). */
#ifndef SH_GW_H_
#define SH_GW_H_

#include <cufft.h>

#include <functional>
#include <string>
#include <vector>

#include "sh_internal.h"

namespace sh {

/* Bin lists of one spectrum kind: grid size P, binned or unbinned, with the
 * index_to_k table of a projection type. */
struct GwBins {
    int P = 0, unbinned = -1, projection_type = -1;
    std::vector<long long> ks; /* k^2 of every bin */
    long long *d_off = nullptr; /* nbins + 1 */
    int *d_cells = nullptr;     /* cells sorted by bin, ascending within a bin */
    double *d_itk = nullptr;    /* index_to_k[P] */
    float *d_itk32 = nullptr;   /* the same in FP32 (FP32 transforms) */
    long long used = 0;         /* last use (for eviction) */
};

/* Bin lists and cuFFT plans of the recent spectrum kinds, kept per context
 * (or ensemble) so that alternating binned and unbinned spectra, or several
 * grid sizes, reuse them.  Bin lists are built on the host threads (a
 * stable parallel counting sort, so cells stay in ascending order within a
 * bin and sums are reproducible). */
struct GwCache {
    static constexpr int kMaxBins = 4, kMaxPlans = 3;
    /* plan kinds: one real-to-complex P^3 transform (scalar spectra), three
     * in-place complex P^3 transforms (the GW components in pairs), in FP64
     * or in FP32 */
    static constexpr int kPlanD2Z = 0, kPlanZ2Z3 = 1, kPlanC2C3 = 2;
    std::vector<GwBins> bins;
    struct Plan {
        int P = 0, kind = 0;
        cufftHandle h = 0;
        long long used = 0;
    };
    std::vector<Plan> plans;
    long long clock = 0;
    GwBins *cur = nullptr;
    /* k^2 of the bins of the last prepared kind */
    const std::vector<long long> &ks() const { return cur->ks; }
    void prepare(int P, int unbinned, int projection_type);
    /* cuFFT plan of a kind for P^3 (created on first use); false if cuFFT
     * fails */
    bool plan(int P, int kind, cufftHandle *out);
    void release();
};

std::vector<long long> unique_k2_host(int dim);
std::vector<double> index_to_k_host(int N, int type);
size_t gw_scratch_bytes(int N, int zero_padding);
/* Scalar power spectrum of one P^3 real field that `pack(real)` writes into
 * the zeroed `real`: bins of the sorted unique k^2, pre * sum multpl |F|^2. */
cudaError_t scalar_spectrum_packed(GwCache &cache, cudaStream_t stream, int P, double pre,
                                   double *scratch, double *bins_dev, int *nbins,
                                   long long *launches, std::string &err,
                                   const std::function<void(double *)> &pack);
/* FFT, TT projection and binning of six P^3 real fields, which
 * `pack(p, dst)` writes (enqueued on `stream`) in pairs p = 0..2 as the real
 * and imaginary parts of a complex array, element (x, y, z) at
 * dst[(z P + y) P + x]: (du_xx, du_xy), (du_xz, du_yy), (du_yz, du_zz); the
 * destination is zeroed first only when the packed N^3 block does not fill
 * it (N < P). */
cudaError_t gw_spectrum_packed(GwCache &cache, cudaStream_t stream, int P, int N,
                               int projection_type, int unbinned, double *scratch,
                               double *bins_dev, int *nbins, long long *launches,
                               std::string &err,
                               const std::function<void(int, double2 *)> &pack);
/* gw_spectrum_packed with FP32 transforms and an FP32 projection (the
 * precision form's spectra: FP32 state, FP64 bin sums): `pack(p, dst)`
 * writes the pairs into complex FP32 arrays. */
cudaError_t gw_spectrum_packed32(GwCache &cache, cudaStream_t stream, int P, int N,
                                 int projection_type, int unbinned, double *scratch,
                                 double *bins_dev, int *nbins, long long *launches,
                                 std::string &err,
                                 const std::function<void(int, float2 *)> &pack);
cudaError_t gw_spectrum_device(GwCache &cache, cudaStream_t stream, const BoxDev *boxes,
                               const long long *vbase, int nbox, long long nvalid, int ncomp,
                               const double *buf, const int comps[6], int N, const int dlo[3],
                               int zero_padding, int projection_type, int unbinned,
                               double *scratch, double *bins_dev, int *nbins, long long *launches,
                               std::string &err);

} // namespace sh

#endif
