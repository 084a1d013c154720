/* ORACLE (test infrastructure only).
 *
 * Stand-in for the few AMReX types the reference's integrators
 * (source/integrators/rkn.cpp, lsssprk3.cpp, leapfrog.cpp) and
 * source/level_data.h use, when they are compiled unchanged into
 * oracle/_ref by oracle/build_ref.sh: a MultiFab of one box covering a
 * periodic cubic domain with ghost cells (FArrayBox layout: x fastest, then
 * y, z, component), with MultiFab::Copy, Saxpy and LinComb as AMReX
 * documents them (over the valid cells and nghost ghost layers:
 * dst = src; dst += a src; dst = a x + b y), an MFIter over that one box,
 * and no-op ParmParse / Error / AllPrint.  Storage starts zeroed.
 * Force-included after ref_prelude.h (amrex::Array4, Dim3, Real).
 */
#ifndef SH_REF_SHIM_INT_MULTIFAB_H_
#define SH_REF_SHIM_INT_MULTIFAB_H_

#include <cfloat>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

namespace amrex {

template <class T>
using Vector = std::vector<T>;

struct Box {
    Dim3 lo{0, 0, 0}, hi{-1, -1, -1};
};
inline Dim3 lbound(const Box &b) { return b.lo; }
inline Dim3 ubound(const Box &b) { return b.hi; }

/* the valid box of the single-box level */
struct BoxArray {
    Box box;
};
struct DistributionMapping {};

class MultiFab;
class MFIter {
  public:
    MFIter(const MultiFab &, bool = true) {}
    bool isValid() const { return !done_; }
    MFIter &operator++() {
        done_ = true;
        return *this;
    }
    Box tilebox() const;
    const MultiFab *mf_ = nullptr;

  private:
    bool done_ = false;
    friend class MultiFab;
};

class MultiFab {
  public:
    MultiFab() = default;
    MultiFab(const BoxArray &ba, const DistributionMapping &, int ncomp, int nghost) {
        define(ba, DistributionMapping{}, ncomp, nghost);
    }
    void define(const BoxArray &ba, const DistributionMapping &, int ncomp, int nghost) {
        ba_ = ba;
        nc_ = ncomp;
        ng_ = nghost;
        n_ = ba.box.hi.x - ba.box.lo.x + 1;
        g_ = n_ + 2 * nghost;
        data_.assign((size_t)g_ * g_ * g_ * nc_, 0.);
    }
    void clear() { data_.clear(); }
    const BoxArray &boxArray() const { return ba_; }
    DistributionMapping DistributionMap() const { return {}; }
    int nComp() const { return nc_; }
    int nGrow() const { return ng_; }
    int size() const { return n_; }
    /* element of cell (i, j, k) of component n, ghost cells included */
    double &at(int i, int j, int k, int n) {
        return data_[(((size_t)n * g_ + (k + ng_)) * g_ + (j + ng_)) * g_ + (i + ng_)];
    }
    double at(int i, int j, int k, int n) const {
        return data_[(((size_t)n * g_ + (k + ng_)) * g_ + (j + ng_)) * g_ + (i + ng_)];
    }
    Array4<double> array(const MFIter &) {
        return Array4<double>(data_.data(), g_, (Long)g_ * g_, (Long)g_ * g_ * g_,
                              Dim3{-ng_, -ng_, -ng_}, nc_);
    }
    Array4<const double> array(const MFIter &) const {
        return Array4<const double>(data_.data(), g_, (Long)g_ * g_, (Long)g_ * g_ * g_,
                                    Dim3{-ng_, -ng_, -ng_}, nc_);
    }
    /* dst(dstcomp..) = src(srccomp..) */
    static void Copy(MultiFab &dst, const MultiFab &src, int srccomp, int dstcomp, int numcomp,
                     int nghost) {
        dst.each(nghost, numcomp, [&](int i, int j, int k, int n) {
            dst.at(i, j, k, dstcomp + n) = src.at(i, j, k, srccomp + n);
        });
    }
    /* dst(dstcomp..) += a src(srccomp..) */
    static void Saxpy(MultiFab &dst, double a, const MultiFab &src, int srccomp, int dstcomp,
                      int numcomp, int nghost) {
        dst.each(nghost, numcomp, [&](int i, int j, int k, int n) {
            dst.at(i, j, k, dstcomp + n) += a * src.at(i, j, k, srccomp + n);
        });
    }
    /* dst(dstcomp..) = a x(xcomp..) + b y(ycomp..) */
    static void LinComb(MultiFab &dst, double a, const MultiFab &x, int xcomp, double b,
                        const MultiFab &y, int ycomp, int dstcomp, int numcomp, int nghost) {
        dst.each(nghost, numcomp, [&](int i, int j, int k, int n) {
            dst.at(i, j, k, dstcomp + n) = a * x.at(i, j, k, xcomp + n) + b * y.at(i, j, k, ycomp + n);
        });
    }
    /* ghost cells from their periodic images */
    void FillBoundaryPeriodic() {
        for (int n = 0; n < nc_; ++n)
            for (int k = -ng_; k < n_ + ng_; ++k)
                for (int j = -ng_; j < n_ + ng_; ++j)
                    for (int i = -ng_; i < n_ + ng_; ++i) {
                        if (i >= 0 && i < n_ && j >= 0 && j < n_ && k >= 0 && k < n_) continue;
                        at(i, j, k, n) = at((i + n_) % n_, (j + n_) % n_, (k + n_) % n_, n);
                    }
    }

  private:
    template <class F>
    void each(int nghost, int numcomp, F &&f) {
        if (nghost > ng_) throw std::runtime_error("more ghost layers than the MultiFab has");
        for (int n = 0; n < numcomp; ++n)
            for (int k = -nghost; k < n_ + nghost; ++k)
                for (int j = -nghost; j < n_ + nghost; ++j)
                    for (int i = -nghost; i < n_ + nghost; ++i) f(i, j, k, n);
    }
    BoxArray ba_;
    int nc_ = 0, ng_ = 0, n_ = 0, g_ = 0;
    std::vector<double> data_;
};

inline Box MFIter::tilebox() const { return Box{}; }

/* user-defined tableaus are not read in these tests */
struct ParmParse {
    explicit ParmParse(const std::string &) {}
    template <class T>
    void getarr(const char *, T &) const {
        throw std::runtime_error("ParmParse is not available in the oracle");
    }
};
inline void Error(const std::string &m) { throw std::runtime_error(m); }
inline PrintStub AllPrint() { return PrintStub(); }

} // namespace amrex

#endif // SH_REF_SHIM_INT_MULTIFAB_H_
