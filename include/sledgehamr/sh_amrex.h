/* Minimal stand-ins for the AMReX types and macros that sledgehamr project
 * kernel headers use (amrex::Array4, amrex::Real, amrex::Dim3, amrex::min/max,
 * AMREX_GPU_DEVICE, AMREX_GPU_HOST_DEVICE, AMREX_FORCE_INLINE).
 *
 * Only the public indexing semantics of AMReX's Array4 are kept, because
 * project hooks rely on them: state(i, j, k, n) addresses absolute cell
 * indices (ghost cells included) of a box whose x index runs fastest, then y,
 * then z, then the component n.  Everything else about the storage is up to
 * the caller that builds the accessor: a view of a box in HBM, a shared-memory
 * tile, or a per-thread register array (all strides zero, one component
 * stride) for the Rhs output of a single cell.
 *
 * Reference interface: amrex::Array4 as used by
 *   source/utils/sledgehamr_utils.h:50-188 and projects/<Name>/kernels_*.h.
 */
#ifndef SH_AMREX_SHIM_H_
#define SH_AMREX_SHIM_H_

#include <cmath>
#include <cstdint>
#include <type_traits>

#if defined(__CUDACC__)
#define AMREX_GPU_DEVICE __device__
#define AMREX_GPU_HOST_DEVICE __host__ __device__
#define AMREX_FORCE_INLINE __forceinline__
#else
#define AMREX_GPU_DEVICE
#define AMREX_GPU_HOST_DEVICE
#define AMREX_FORCE_INLINE inline __attribute__((always_inline))
#endif
#define AMREX_GPU_HOST
#define AMREX_RESTRICT __restrict__
#ifndef AMREX_SPACEDIM
#define AMREX_SPACEDIM 3
#endif
#define AMREX_PRAGMA_SIMD

namespace amrex {

using Real = double;
using Long = long long;

struct Dim3 {
    int x, y, z;
};

template <class T>
AMREX_GPU_HOST_DEVICE AMREX_FORCE_INLINE constexpr const T &min(const T &a,
                                                                const T &b) {
    return (b < a) ? b : a;
}
template <class T>
AMREX_GPU_HOST_DEVICE AMREX_FORCE_INLINE constexpr const T &max(const T &a,
                                                                const T &b) {
    return (a < b) ? b : a;
}

/* Four-index accessor: p[(i-begin.x) + (j-begin.y)*jstride
 *                       + (k-begin.z)*kstride + n*nstride]. */
template <class T>
struct Array4 {
    T *AMREX_RESTRICT p = nullptr;
    Long jstride = 0;
    Long kstride = 0;
    Long nstride = 0;
    Dim3 begin{0, 0, 0};
    Dim3 end{0, 0, 0}; /* one past the last cell, as in AMReX */
    int ncomp = 0;

    constexpr Array4() = default;

    AMREX_GPU_HOST_DEVICE AMREX_FORCE_INLINE constexpr Array4(
        T *ptr, Dim3 lo, Dim3 hi_plus_one, int nc)
        : p(ptr),
          jstride(Long(hi_plus_one.x - lo.x)),
          kstride(Long(hi_plus_one.x - lo.x) * (hi_plus_one.y - lo.y)),
          nstride(Long(hi_plus_one.x - lo.x) * (hi_plus_one.y - lo.y) *
                  (hi_plus_one.z - lo.z)),
          begin(lo), end(hi_plus_one), ncomp(nc) {}

    AMREX_GPU_HOST_DEVICE AMREX_FORCE_INLINE constexpr Array4(
        T *ptr, Long js, Long ks, Long ns, Dim3 lo, Dim3 hi_plus_one, int nc)
        : p(ptr), jstride(js), kstride(ks), nstride(ns), begin(lo),
          end(hi_plus_one), ncomp(nc) {}

    /* Array4<const T> from Array4<T>. */
    template <class U,
              class = typename std::enable_if<
                  std::is_same<T, const U>::value>::type>
    AMREX_GPU_HOST_DEVICE AMREX_FORCE_INLINE constexpr Array4(
        const Array4<U> &rhs)
        : p(rhs.p), jstride(rhs.jstride), kstride(rhs.kstride),
          nstride(rhs.nstride), begin(rhs.begin), end(rhs.end),
          ncomp(rhs.ncomp) {}

    AMREX_GPU_HOST_DEVICE AMREX_FORCE_INLINE T &operator()(int i, int j, int k,
                                                           int n = 0) const {
        return p[(i - begin.x) + (j - begin.y) * jstride +
                 (k - begin.z) * kstride + n * nstride];
    }

    AMREX_GPU_HOST_DEVICE AMREX_FORCE_INLINE T *ptr(int i, int j, int k,
                                                   int n = 0) const {
        return p + ((i - begin.x) + (j - begin.y) * jstride +
                    (k - begin.z) * kstride + n * nstride);
    }

    AMREX_GPU_HOST_DEVICE AMREX_FORCE_INLINE int nComp() const {
        return ncomp;
    }
};

template <class T>
AMREX_GPU_HOST_DEVICE AMREX_FORCE_INLINE Dim3 lbound(const Array4<T> &a) {
    return a.begin;
}
template <class T>
AMREX_GPU_HOST_DEVICE AMREX_FORCE_INLINE Dim3 ubound(const Array4<T> &a) {
    return Dim3{a.end.x - 1, a.end.y - 1, a.end.z - 1};
}

} // namespace amrex

#endif // SH_AMREX_SHIM_H_
