/* Internal interface of the GW spectrum module (sh_gw.cu). */
#ifndef SH_GW_H_
#define SH_GW_H_

#include <cufft.h>

#include <functional>
#include <string>
#include <vector>

#include "sh_internal.h"

namespace sh {

/* Bin lists, index_to_k table and cuFFT plan of the last spectrum size,
 * kept per context. */
struct GwCache {
    int P = 0, unbinned = -1, projection_type = -1;
    std::vector<long long> ks;
    long long *d_off = nullptr; /* nbins + 1 */
    int *d_cells = nullptr;     /* cells sorted by bin, ascending within a bin */
    double *d_itk = nullptr;    /* index_to_k[P] */
    cufftHandle plan = 0;
    bool plan_ok = false;
    int plan_P = 0;
    void prepare(int P, int unbinned, int projection_type);
    void release();
};

std::vector<long long> unique_k2_host(int dim);
std::vector<double> index_to_k_host(int N, int type);
size_t gw_scratch_bytes(int N, int zero_padding);
/* FFT, TT projection and binning of six P^3 real arrays that `pack(q, real)`
 * writes (enqueued on `stream`) into the zeroed `real` for q = 0..5 in the
 * order du_xx, du_xy, du_xz, du_yy, du_yz, du_zz. */
/* Scalar power spectrum of one P^3 real field that `pack(real)` writes into
 * the zeroed `real`: bins of the sorted unique k^2, pre * sum multpl |F|^2. */
cudaError_t scalar_spectrum_packed(GwCache &cache, cudaStream_t stream, int P, double pre,
                                   double *scratch, double *bins_dev, int *nbins,
                                   long long *launches, std::string &err,
                                   const std::function<void(double *)> &pack);
cudaError_t gw_spectrum_packed(GwCache &cache, cudaStream_t stream, int P, int projection_type,
                               int unbinned, double *scratch, double *bins_dev, int *nbins,
                               long long *launches, std::string &err,
                               const std::function<void(int, double *)> &pack);
cudaError_t gw_spectrum_device(GwCache &cache, cudaStream_t stream, const BoxDev *boxes,
                               const long long *vbase, int nbox, long long nvalid, int ncomp,
                               const double *buf, const int comps[6], int N, const int dlo[3],
                               int zero_padding, int projection_type, int unbinned,
                               double *scratch, double *bins_dev, int *nbins, long long *launches,
                               std::string &err);

} // namespace sh

#endif
