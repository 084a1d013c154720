/* ORACLE (test infrastructure only).
 *
 * Prelude force-included (-include) when the reference's own per-cell
 * headers (source/utils/sledgehamr_utils.h, source/kernels.h and the
 * projects' kernels_*.h) are compiled into oracle/_ref by
 * oracle/build_ref.sh.  It provides the handful of AMReX names those headers
 * use: amrex::Real, amrex::Array4, amrex::min/max, the AMREX_* function
 * qualifiers, and no-op stand-ins for amrex::ParallelDescriptor::Barrier and
 * amrex::Print that the headers' unused timer helpers mention.
 */
#ifndef SH_REF_PRELUDE_H_
#define SH_REF_PRELUDE_H_

#include <cfloat>
#include <cmath>
#include <functional>
#include <iostream>
#include <string>
#include <vector>

#define AMREX_GPU_DEVICE
#define AMREX_GPU_HOST_DEVICE
#define AMREX_FORCE_INLINE inline
#define AMREX_PRAGMA_SIMD
#define AMREX_SPACEDIM 3

namespace amrex {
using Real = double;
using Long = long long;
struct Dim3 { int x, y, z; };
template <class T> inline const T &min(const T &a, const T &b) { return b < a ? b : a; }
template <class T> inline const T &max(const T &a, const T &b) { return a < b ? b : a; }
template <class T>
struct Array4 {
    T *p = nullptr;
    Long jstride = 0, kstride = 0, nstride = 0;
    Dim3 begin{0, 0, 0};
    int ncomp = 0;
    Array4() = default;
    Array4(T *ptr, Long js, Long ks, Long ns, Dim3 b, int nc)
        : p(ptr), jstride(js), kstride(ks), nstride(ns), begin(b), ncomp(nc) {}
    template <class U, class = typename std::enable_if<std::is_same<T, const U>::value>::type>
    Array4(const Array4<U> &o)
        : p(o.p), jstride(o.jstride), kstride(o.kstride), nstride(o.nstride), begin(o.begin),
          ncomp(o.ncomp) {}
    T &operator()(int i, int j, int k, int n = 0) const {
        return p[(i - begin.x) + (j - begin.y) * jstride + (k - begin.z) * kstride + n * nstride];
    }
    int nComp() const { return ncomp; }
};
namespace ParallelDescriptor {
inline void Barrier() {}
} // namespace ParallelDescriptor
struct PrintStub {
    template <class T> PrintStub &operator<<(const T &) { return *this; }
    PrintStub &operator<<(std::ostream &(*)(std::ostream &)) { return *this; }
};
inline PrintStub Print() { return PrintStub(); }
} // namespace amrex

#endif // SH_REF_PRELUDE_H_
