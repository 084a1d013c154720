/* ORACLE (test infrastructure only).
 *
 * CPU restatement, in FP64, of sledgehamr's time-stepping hot path.  It is
 * the checker for the CUDA implementation in sledgehamr_gb300/ and the timed
 * CPU baseline; nothing in the product links or calls it.
 *
 * Data model (restating AMReX MultiFab as sledgehamr uses it): a level is a
 * list of boxes; each box stores every component as a contiguous FP64 array
 * over the ghost-grown box, x fastest, then y, z, component.
 *
 * What each part follows (paths relative to the sledgehamr repository):
 *   FillRhs / FillAddRhs loop drivers ..... source/macros.h:301-485
 *   RKN (RKN4, RKN5, user tableau) ........ source/integrators/rkn.cpp:25-120,
 *                                           tableaus :124-156
 *   low-storage SSPRK3 .................... source/integrators/lsssprk3.cpp:14-31
 *   leapfrog KDK .......................... source/integrators/leapfrog.cpp:13-57
 *   Integrator::Advance ................... source/integrators/integrator.cpp:11-31
 *   periodic ghost fill (lev <= 0) ........ source/level_synchronizer.cpp:19-25,
 *                                           :94-144, :156-214, :613-632
 *   average down with truncation error .... source/kernels.h:18-42,
 *                                           source/level_synchronizer.cpp:240-357
 *   plain average down .................... source/level_synchronizer.cpp:219-233
 *                                           (amrex::average_down: 2x2x2 mean;
 *                                           summation order unpinned)
 *   shadow level .......................... source/sledgehamr.cpp:234-251
 *   CPU tagging ........................... source/macros.h:199-220, :489-566,
 *                                           :640-663; source/sledgehamr.cpp:280-348
 *   GW spectrum ........................... source/gravitational_waves.cpp:52-322,
 *                                           source/gravitational_waves.h:101-133,
 *                                           source/utils/fft.h:143-262
 *   spectrum bins and index_to_k .......... pySledgehamr/Sledgehamr.py:7-27
 *
 * The arithmetic of every FP64 expression keeps the operand order of the
 * cited code, and the library is compiled with -ffp-contract=off, so that
 * results are reproducible bit for bit on x86-64 and aarch64 hosts.
 */
#ifndef SH_ORACLE_CORE_H_
#define SH_ORACLE_CORE_H_

#include <algorithm>
#include <cassert>
#include <cfloat>
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstring>
#include <functional>
#include <stdexcept>
#include <utility>
#include <vector>

namespace orc {

struct IV {
    int x, y, z;
};

struct Box {
    IV lo, hi; /* inclusive */
    int len(int d) const {
        return d == 0 ? hi.x - lo.x + 1 : (d == 1 ? hi.y - lo.y + 1 : hi.z - lo.z + 1);
    }
    long long volume() const { return (long long)len(0) * len(1) * len(2); }
    Box grow(int g) const {
        return Box{{lo.x - g, lo.y - g, lo.z - g}, {hi.x + g, hi.y + g, hi.z + g}};
    }
    bool contains(int i, int j, int k) const {
        return i >= lo.x && i <= hi.x && j >= lo.y && j <= hi.y && k >= lo.z &&
               k <= hi.z;
    }
    Box coarsen2() const {
        auto cdiv = [](int a) { return a >= 0 ? a / 2 : -((-a + 1) / 2); };
        return Box{{cdiv(lo.x), cdiv(lo.y), cdiv(lo.z)},
                   {cdiv(hi.x), cdiv(hi.y), cdiv(hi.z)}};
    }
};

/* Four-index view with the semantics of amrex::Array4. */
template <class T>
struct A4 {
    T *p = nullptr;
    long long js = 0, ks = 0, ns = 0;
    IV b{0, 0, 0};
    int nc = 0;
    T &operator()(int i, int j, int k, int n = 0) const {
        return p[(i - b.x) + (j - b.y) * js + (k - b.z) * ks + n * ns];
    }
    operator A4<const T>() const {
        A4<const T> r;
        r.p = p; r.js = js; r.ks = ks; r.ns = ns; r.b = b; r.nc = nc;
        return r;
    }
};

struct Fab {
    Box vbox;
    int ng = 0, nc = 0;
    std::vector<double> d;
    Box gbox() const { return vbox.grow(ng); }
    void define(const Box &b, int ncomp, int nghost) {
        vbox = b; nc = ncomp; ng = nghost;
        d.assign((size_t)gbox().volume() * nc, 0.0);
    }
    A4<double> a() {
        Box g = gbox();
        A4<double> r;
        r.p = d.data(); r.js = g.len(0); r.ks = (long long)g.len(0) * g.len(1);
        r.ns = g.volume(); r.b = g.lo; r.nc = nc;
        return r;
    }
    A4<const double> ca() const { return const_cast<Fab *>(this)->a(); }
};

/* A level's data at one time (MultiFab + time bookkeeping of LevelData). */
struct MF {
    Box domain; /* periodic domain of this level */
    std::vector<Fab> fabs;
    int nc = 0, ng = 0;
    double t = -DBL_MAX;
    int istep = 0;
    bool contains_truncation_errors = false;
    /* owner box of every block of `res` cells of the domain (-1: uncovered) */
    std::vector<int> owner;
    int res = 0, nbx = 0, nby = 0, nbz = 0;

    void define(const Box &dom, const std::vector<Box> &boxes, int ncomp,
                int nghost, double time = -DBL_MAX) {
        domain = dom; nc = ncomp; ng = nghost; t = time; istep = 0;
        contains_truncation_errors = false;
        fabs.assign(boxes.size(), Fab());
        for (size_t b = 0; b < boxes.size(); ++b) fabs[b].define(boxes[b], ncomp, nghost);
        auto gcd = [](int a, int b) {
            a = a < 0 ? -a : a;
            b = b < 0 ? -b : b;
            while (b) { int r = a % b; a = b; b = r; }
            return a;
        };
        res = gcd(gcd(dom.len(0), dom.len(1)), dom.len(2));
        for (const Box &b : boxes) {
            res = gcd(res, b.lo.x - dom.lo.x); res = gcd(res, b.hi.x + 1 - dom.lo.x);
            res = gcd(res, b.lo.y - dom.lo.y); res = gcd(res, b.hi.y + 1 - dom.lo.y);
            res = gcd(res, b.lo.z - dom.lo.z); res = gcd(res, b.hi.z + 1 - dom.lo.z);
        }
        if (res <= 0) res = 1;
        nbx = dom.len(0) / res; nby = dom.len(1) / res; nbz = dom.len(2) / res;
        owner.assign((size_t)nbx * nby * nbz, -1);
        for (size_t q = 0; q < boxes.size(); ++q) {
            const Box &b = boxes[q];
            for (int z = (b.lo.z - dom.lo.z) / res; z <= (b.hi.z - dom.lo.z) / res; ++z)
                for (int y = (b.lo.y - dom.lo.y) / res; y <= (b.hi.y - dom.lo.y) / res; ++y)
                    for (int x = (b.lo.x - dom.lo.x) / res; x <= (b.hi.x - dom.lo.x) / res; ++x)
                        owner[((size_t)z * nby + y) * nbx + x] = (int)q;
        }
    }
    bool defined() const { return !fabs.empty(); }
    std::vector<Box> boxes() const {
        std::vector<Box> r;
        for (auto &f : fabs) r.push_back(f.vbox);
        return r;
    }
    void clear() { fabs.clear(); }
};

/* Find the fab of `mf` whose valid box contains cell (i,j,k), or -1. */
inline int find_fab(const MF &mf, int i, int j, int k) {
    if (!mf.domain.contains(i, j, k) || mf.res <= 0) return -1;
    const int x = (i - mf.domain.lo.x) / mf.res, y = (j - mf.domain.lo.y) / mf.res,
              z = (k - mf.domain.lo.z) / mf.res;
    return mf.owner[((size_t)z * mf.nby + y) * mf.nbx + x];
}

template <class F>
inline void for_cells(const Box &b, F &&f) {
    for (int k = b.lo.z; k <= b.hi.z; ++k)
        for (int j = b.lo.y; j <= b.hi.y; ++j)
            for (int i = b.lo.x; i <= b.hi.x; ++i) f(i, j, k);
}
/* Same visit, with (k, j) rows shared among OpenMP threads; only for bodies
 * that write nothing but their own cell. */
template <class F>
inline void for_cells_par(const Box &b, F &&f) {
    const int nj = b.len(1), nk = b.len(2);
#pragma omp parallel for schedule(static)
    for (int r = 0; r < nj * nk; ++r) {
        const int j = b.lo.y + r % nj, k = b.lo.z + r / nj;
        for (int i = b.lo.x; i <= b.hi.x; ++i) f(i, j, k);
    }
}

/* ---- MultiFab linear algebra (valid region grown by ngrow) ------------ */
inline void mf_copy(MF &dst, const MF &src, int scomp, int dcomp, int ncomp, int ngrow) {
    for (size_t b = 0; b < dst.fabs.size(); ++b) {
        auto d = dst.fabs[b].a();
        auto s = src.fabs[b].ca();
        for (int n = 0; n < ncomp; ++n)
            for_cells_par(dst.fabs[b].vbox.grow(ngrow),
                          [&](int i, int j, int k) { d(i, j, k, dcomp + n) = s(i, j, k, scomp + n); });
    }
}
/* dst[dcomp..] += a * src[scomp..] (amrex::MultiFab::Saxpy) */
inline void mf_saxpy(MF &dst, double a, const MF &src, int scomp, int dcomp, int ncomp, int ngrow) {
    for (size_t b = 0; b < dst.fabs.size(); ++b) {
        auto d = dst.fabs[b].a();
        auto s = src.fabs[b].ca();
        for (int n = 0; n < ncomp; ++n)
            for_cells_par(dst.fabs[b].vbox.grow(ngrow), [&](int i, int j, int k) {
                d(i, j, k, dcomp + n) += a * s(i, j, k, scomp + n);
            });
    }
}
/* dst[dcomp..] = a * x[xcomp..] + b * y[ycomp..] (amrex::MultiFab::LinComb) */
inline void mf_lincomb(MF &dst, double a, const MF &x, int xcomp, double bcoef, const MF &y,
                       int ycomp, int dcomp, int ncomp, int ngrow) {
    for (size_t b = 0; b < dst.fabs.size(); ++b) {
        auto d = dst.fabs[b].a();
        auto xa = x.fabs[b].ca();
        auto ya = y.fabs[b].ca();
        for (int n = 0; n < ncomp; ++n)
            for_cells_par(dst.fabs[b].vbox.grow(ngrow), [&](int i, int j, int k) {
                d(i, j, k, dcomp + n) = a * xa(i, j, k, xcomp + n) + bcoef * ya(i, j, k, ycomp + n);
            });
    }
}

inline int pmod(int a, int n) {
    int r = a % n;
    return r < 0 ? r + n : r;
}

/* Single-level ghost fill with periodic boundaries in every direction
 * (FillPatchSingleLevel with int_dir BCs): each ghost cell takes the value of
 * the valid cell, in any box of the same level, that is its periodic image.
 * Ghost cells whose image is not covered by the level are left untouched
 * (on a fine level they are filled by coarse-fine interpolation). */
inline void fill_boundary_periodic(MF &mf) {
    const int NX = mf.domain.len(0), NY = mf.domain.len(1), NZ = mf.domain.len(2);
    const IV dlo = mf.domain.lo;
    for (size_t b = 0; b < mf.fabs.size(); ++b) {
        Fab &fab = mf.fabs[b];
        auto d = fab.a();
        const Box vb = fab.vbox;
        for_cells_par(fab.gbox(), [&](int i, int j, int k) {
            if (vb.contains(i, j, k)) return;
            int si = dlo.x + pmod(i - dlo.x, NX);
            int sj = dlo.y + pmod(j - dlo.y, NY);
            int sk = dlo.z + pmod(k - dlo.z, NZ);
            const int s = find_fab(mf, si, sj, sk);
            if (s < 0) return;
            auto sa = mf.fabs[s].ca();
            for (int n = 0; n < mf.nc; ++n) d(i, j, k, n) = sa(si, sj, sk, n);
        });
    }
}

/* ---- project hook policy ------------------------------------------------
 * P::NScalars (user fields incl. momenta), P::NFields (position fields),
 * P::rhs(...), P::gw_rhs(...), P::tag(...), P::te_modifier(n, ...).       */

struct RhsConfig {
    int lev = 0;
    double dt = 0, dx = 0;
    const double *params = nullptr;
    const double *gw_params = nullptr;
    bool with_gw = false;
    int ko_order = 0;                  /* 0: off, 2 or 3 */
    const double *ko_strength = nullptr; /* per component */
};

template <class P>
inline void cell_rhs_full(const A4<double> &r, const A4<const double> &s, int i, int j, int k,
                          double time, const RhsConfig &c, int ncomp) {
    P::rhs(r, s, i, j, k, c.lev, time, c.dt, c.dx, c.params);
    if (c.with_gw) {
        P::gw_rhs(r, s, i, j, k, c.lev, time, c.dt, c.dx, c.gw_params);
        P::gw_backreaction(r, s, i, j, k, c.lev, time, c.dt, c.dx, c.params, c.gw_params);
    }
    if (c.ko_order == 2 || c.ko_order == 3) {
        for (int n = 0; n < ncomp; ++n)
            r(i, j, k, n) += P::ko(c.ko_order, s, i, j, k, n, c.dx, c.ko_strength[n]);
    }
}

/* FillRhs: rhs = f(state) on the valid cells of every box. */
template <class P>
inline void fill_rhs(MF &rhs, const MF &state, double time, const RhsConfig &c) {
    for (size_t b = 0; b < rhs.fabs.size(); ++b) {
        auto r = rhs.fabs[b].a();
        auto s = state.fabs[b].ca();
        for_cells_par(rhs.fabs[b].vbox, [&](int i, int j, int k) {
            cell_rhs_full<P>(r, s, i, j, k, time, c, rhs.nc);
        });
    }
}

/* FillAddRhs: rhs = f(state) + weight * rhs_old. */
template <class P>
inline void fill_add_rhs(MF &rhs, const MF &state, double time, const RhsConfig &c,
                         double weight) {
    for (size_t b = 0; b < rhs.fabs.size(); ++b) {
        auto r = rhs.fabs[b].a();
        auto s = state.fabs[b].ca();
        for_cells_par(rhs.fabs[b].vbox, [&](int i, int j, int k) {
            double tmp[64];
            for (int n = 0; n < rhs.nc; ++n) tmp[n] = r(i, j, k, n);
            cell_rhs_full<P>(r, s, i, j, k, time, c, rhs.nc);
            for (int n = 0; n < rhs.nc; ++n) r(i, j, k, n) += weight * tmp[n];
        });
    }
}

/* ---- integrators --------------------------------------------------------*/
enum IntegratorType {
    Lsssprk3 = 10,
    Leapfrog = 11,
    RknButcherTableau = 20,
    Rkn4 = 21,
    Rkn5 = 22
};

struct RknTableau {
    std::vector<double> nodes;
    std::vector<std::vector<double>> a; /* lower triangle incl. diagonal */
    std::vector<double> bbar, b;
};

/* Tableaus of source/integrators/rkn.cpp:130-152. */
inline RknTableau rkn_tableau(int type) {
    RknTableau t;
    if (type == Rkn4) {
        t.nodes = {0.0, 0.5, 1.0};
        t.a = {{0.0}, {1. / 8., 0.0}, {0.0, 0.5, 0.0}};
        t.bbar = {1. / 6., 1. / 3., 0.0};
        t.b = {1. / 6., 4. / 6., 1. / 6.};
    } else if (type == Rkn5) {
        t.nodes = {0.0, 1. / 5., 2. / 3., 1.0};
        t.a = {{0.0}, {1. / 50., 0.0}, {-1. / 27., 7. / 27., 0.0}, {3. / 10., -2. / 35., 9. / 35., 0.0}};
        t.bbar = {14. / 336., 100. / 336., 54. / 336., 0.0};
        t.b = {14. / 336., 125. / 336., 162. / 336., 35. / 336.};
    } else {
        throw std::runtime_error("rkn_tableau: unknown type");
    }
    return t;
}

/* Ghost fill for a level during a step.  The periodic single-level fill is
 * built in; a two-level fill is supplied by the AMR driver. */
using GhostFill = std::function<void(MF &, double)>;

struct StepContext {
    int ncomp_user = 0; /* Nf = user fields incl. momenta */
    bool with_gw = false;
    GhostFill fill;    /* FillIntermediatePatch(lev, time, mf) */
};

/* IntegratorRkn::Integrate, source/integrators/rkn.cpp:25-120. */
template <class P>
inline void integrate_rkn(MF &mf_old, MF &mf_new, const RknTableau &tab, double dt,
                          const RhsConfig &c, const StepContext &sc) {
    const double t = mf_old.t;
    const int nghost = mf_old.ng;
    const int N = mf_old.nc;
    const int Ngrav = sc.with_gw ? 12 : 0;
    const int Nf = N - Ngrav;
    const int uN = Nf / 2, uN0 = 0, uN1 = uN0 + uN;
    const int gN = Ngrav / 2, gN0 = Nf, gN1 = gN0 + gN;
    const int S = (int)tab.b.size();

    std::vector<MF> F(S);
    for (int i = 0; i < S; ++i) F[i].define(mf_old.domain, mf_old.boxes(), N, nghost);

    for (int i = 0; i < S; ++i) {
        double stage_time = t + dt * tab.nodes[i];
        mf_copy(mf_new, mf_old, 0, 0, N, nghost);
        mf_saxpy(mf_new, dt * tab.nodes[i], mf_old, uN1, uN0, uN, nghost);
        if (Ngrav > 0) mf_saxpy(mf_new, dt * tab.nodes[i], mf_old, gN1, gN0, gN, nghost);
        for (int j = 0; j < i; ++j) {
            mf_saxpy(mf_new, dt * dt * tab.a[i][j], F[j], uN1, uN0, uN, nghost);
            if (Ngrav == 0) continue;
            mf_saxpy(mf_new, dt * dt * tab.a[i][j], F[j], gN1, gN0, gN, nghost);
        }
        sc.fill(mf_new, stage_time);
        fill_rhs<P>(F[i], mf_new, stage_time, c);
    }
    mf_copy(mf_new, mf_old, 0, 0, N, nghost);
    mf_saxpy(mf_new, dt, mf_new, uN1, uN0, uN, nghost);
    if (Ngrav > 0) mf_saxpy(mf_new, dt, mf_new, gN1, gN0, gN, nghost);
    for (int i = 0; i < S; ++i) {
        mf_saxpy(mf_new, dt * dt * tab.bbar[i], F[i], uN1, uN0, uN, nghost);
        mf_saxpy(mf_new, dt * tab.b[i], F[i], uN1, uN1, uN, nghost);
        if (Ngrav == 0) continue;
        mf_saxpy(mf_new, dt * dt * tab.bbar[i], F[i], gN1, gN0, gN, nghost);
        mf_saxpy(mf_new, dt * tab.b[i], F[i], gN1, gN1, gN, nghost);
    }
    sc.fill(mf_new, t + dt);
}

/* IntegratorLsssprk3::Integrate, source/integrators/lsssprk3.cpp:14-31. */
template <class P>
inline void integrate_lsssprk3(MF &mf_old, MF &mf_new, double dt, const RhsConfig &c,
                               const StepContext &sc) {
    const int ncomp = mf_old.nc;
    const double t0 = mf_old.t, t1 = t0 + dt;
    MF k1;
    k1.define(mf_old.domain, mf_old.boxes(), ncomp, mf_old.ng);
    fill_rhs<P>(k1, mf_old, t0, c);
    mf_lincomb(mf_new, 1, mf_old, 0, dt, k1, 0, 0, ncomp, 0);
    sc.fill(mf_new, t1);
    fill_add_rhs<P>(k1, mf_new, t1, c, 1.);
    mf_lincomb(mf_new, 1, mf_old, 0, dt / 4., k1, 0, 0, ncomp, 0);
    sc.fill(mf_new, t0 + dt / 2.);
    fill_add_rhs<P>(k1, mf_new, t0 + dt / 2., c, 0.25);
    mf_lincomb(mf_new, 1, mf_old, 0, dt * 2. / 3., k1, 0, 0, ncomp, 0);
    sc.fill(mf_new, t1);
}

/* IntegratorLeapfrog::Integrate, source/integrators/leapfrog.cpp:13-57.
 * The second force evaluation reads the momentum components that mf_new
 * held before the step (it is not refreshed), as in the reference. */
template <class P>
inline void integrate_leapfrog(MF &mf_old, MF &mf_new, double dt, const RhsConfig &c,
                               const StepContext &sc) {
    const double t0 = mf_old.t, t1 = t0 + dt;
    const int N = mf_old.nc;
    const int Ngrav = sc.with_gw ? 12 : 0;
    const int Nf = N - Ngrav;
    const int uN = Nf / 2, uN0 = 0, uN1 = uN0 + uN;
    const int gN = Ngrav / 2, gN0 = Nf, gN1 = gN0 + gN;
    MF a, vh;
    a.define(mf_old.domain, mf_old.boxes(), N, mf_old.ng);
    vh.define(mf_old.domain, mf_old.boxes(), N, mf_old.ng);
    fill_rhs<P>(a, mf_old, t0, c);
    mf_lincomb(vh, 1, mf_old, 0, dt / 2., a, 0, 0, N, 0);
    mf_lincomb(mf_new, 1, mf_old, uN0, dt, vh, uN1, uN0, uN, 0);
    if (Ngrav > 0) mf_lincomb(mf_new, 1, mf_old, gN0, dt, vh, gN1, gN0, gN, 0);
    sc.fill(mf_new, t1);
    fill_rhs<P>(a, mf_new, t1, c);
    mf_lincomb(mf_new, 1, vh, uN1, dt / 2., a, uN1, uN1, uN, 0);
    if (Ngrav > 0) mf_lincomb(mf_new, 1, vh, gN1, dt / 2., a, gN1, gN1, gN, 0);
    sc.fill(mf_new, t1);
}

struct IntegratorSpec {
    int type = Rkn4;
    RknTableau user; /* for RknButcherTableau */
};

/* Integrate(mf_old -> mf_new) with the scheme selected by integrator.type. */
template <class P>
inline void integrate(const IntegratorSpec &spec, MF &mf_old, MF &mf_new, double dt,
                      const RhsConfig &c, const StepContext &sc) {
    switch (spec.type) {
    case Lsssprk3: integrate_lsssprk3<P>(mf_old, mf_new, dt, c, sc); break;
    case Leapfrog: integrate_leapfrog<P>(mf_old, mf_new, dt, c, sc); break;
    case Rkn4:
    case Rkn5: integrate_rkn<P>(mf_old, mf_new, rkn_tableau(spec.type), dt, c, sc); break;
    case RknButcherTableau: integrate_rkn<P>(mf_old, mf_new, spec.user, dt, c, sc); break;
    default: throw std::runtime_error("unknown integrator type");
    }
}

/* Integrator::Advance for a single periodic level (lev <= 0):
 * swap(old,new); FillPatch(old at t_old); Integrate; t_new = t_old + dt. */
template <class P>
inline void advance_single_level(const IntegratorSpec &spec, MF &grid_old, MF &grid_new,
                                 double dt, const RhsConfig &c, bool with_gw,
                                 int ncomp_user) {
    grid_old.contains_truncation_errors = false;
    std::swap(grid_old, grid_new);
    fill_boundary_periodic(grid_old);
    StepContext sc;
    sc.ncomp_user = ncomp_user;
    sc.with_gw = with_gw;
    sc.fill = [](MF &mf, double) { fill_boundary_periodic(mf); };
    integrate<P>(spec, grid_old, grid_new, dt, c, sc);
    grid_new.t = grid_old.t + dt;
    grid_new.istep = grid_old.istep + 1;
}

/* ---- average down --------------------------------------------------------*/

/* kernels::AverageDownWithTruncationError, source/kernels.h:18-42. */
inline void avgdown_te_cell(int i, int j, int k, int ncomp, const A4<double> &crse,
                            const A4<const double> &fine, const A4<double> &te) {
    const int ratio = 2;
    const double volfrac = 1.0 / (double)(ratio * ratio * ratio);
    const int ii = i * ratio, jj = j * ratio, kk = k * ratio;
    for (int n = 0; n < ncomp; ++n) {
        double c = fine(ii, jj, kk, n);
        c += fine(ii + 1, jj, kk, n);
        c += fine(ii, jj + 1, kk, n);
        c += fine(ii, jj, kk + 1, n);
        c += fine(ii + 1, jj + 1, kk, n);
        c += fine(ii + 1, jj, kk + 1, n);
        c += fine(ii, jj + 1, kk + 1, n);
        c += fine(ii + 1, jj + 1, kk + 1, n);
        te(ii, jj, kk, n) = std::fabs(crse(i, j, k, n) - volfrac * c);
        crse(i, j, k, n) = volfrac * c;
    }
}


/* Plain 2x2x2 average of fine onto every coarse cell covered by fine
 * (amrex::average_down with ratio 2); sum in k, j, i loop order. */
inline void average_down(const MF &fine, MF &crse, int ncomp) {
    for (const Fab &ff : fine.fabs) {
        auto f = ff.ca();
        Box cb = ff.vbox.coarsen2();
        for_cells(cb, [&](int i, int j, int k) {
            int cf = find_fab(crse, i, j, k);
            if (cf < 0) return;
            auto c = crse.fabs[cf].a();
            for (int n = 0; n < ncomp; ++n) {
                double s = 0.0;
                for (int dk = 0; dk < 2; ++dk)
                    for (int dj = 0; dj < 2; ++dj)
                        for (int di = 0; di < 2; ++di) s += f(2 * i + di, 2 * j + dj, 2 * k + dk, n);
                c(i, j, k, n) = s * 0.125;
            }
        });
    }
}

/* LevelSynchronizer::ComputeTruncationErrors restricted to the cell work:
 * for every coarse cell covered by fine, te_fine(2i,2j,2k) =
 * |crse - avg(fine)| and crse = avg(fine). */
inline void average_down_with_te(const MF &fine, MF &crse, MF &te, int ncomp) {
    for (size_t fb = 0; fb < fine.fabs.size(); ++fb) {
        const Fab &ff = fine.fabs[fb];
        auto f = ff.ca();
        auto t = te.fabs[fb].a();
        Box cb = ff.vbox.coarsen2();
        for_cells(cb, [&](int i, int j, int k) {
            int cf = find_fab(crse, i, j, k);
            if (cf < 0) return;
            auto c = crse.fabs[cf].a();
            avgdown_te_cell(i, j, k, ncomp, c, f, t);
        });
    }
}

/* ---- tagging ---------------------------------------------------------------*/

/* Tag mask of one level with the CPU semantics of
 * SLEDGEHAMR_PRJ_TAG_WITH_TRUNCATION_CPU (macros.h:489-566): cells are
 * visited in k, j, i order within 8x8 (y, z) tiles of every box; each visit
 * clears the cell, sets it if the project tags it, and if the cell has all
 * even indices and some component's modified truncation error reaches its
 * threshold, sets the 2x2x2 block starting at the cell.  mask holds one
 * byte per valid cell of every box (box-major, x fastest); 1 = SET. */
template <class P>
inline void tag_cpu_literal(const MF &state, const MF *te, double time, int lev, double dt,
                            double dx, const double *te_crit, int ncomp_te,
                            const double *params_tag, const double *params_mod,
                            std::vector<std::vector<uint8_t>> &mask, long *ntags_total,
                            long *ntags_user, long *ntags_trunc) {
    mask.assign(state.fabs.size(), {});
    for (size_t b = 0; b < state.fabs.size(); ++b) {
        const Box vb = state.fabs[b].vbox;
        mask[b].assign((size_t)vb.volume(), 0);
        auto s = state.fabs[b].ca();
        auto m = [&](int i, int j, int k) -> uint8_t & {
            return mask[b][(size_t)(i - vb.lo.x) +
                           (size_t)vb.len(0) * ((j - vb.lo.y) + (size_t)vb.len(1) * (k - vb.lo.z))];
        };
        auto setm = [&](int i, int j, int k) {
            if (vb.contains(i, j, k)) m(i, j, k) = 1;
        };
        /* default CPU tiling: full x extent, 8 cells in y and z */
        for (int tz = vb.lo.z; tz <= vb.hi.z; tz += 8)
            for (int ty = vb.lo.y; ty <= vb.hi.y; ty += 8) {
                Box tile{{vb.lo.x, ty, tz}, {vb.hi.x, std::min(ty + 7, vb.hi.y), std::min(tz + 7, vb.hi.z)}};
                for_cells(tile, [&](int i, int j, int k) {
                    m(i, j, k) = 0;
                    bool res = P::tag(s, i, j, k, lev, time, dt, dx, params_tag);
                    if (res) {
                        m(i, j, k) = 1;
                        if (ntags_user) (*ntags_user)++;
                        if (ntags_total) (*ntags_total)++;
                    }
                    if (te == nullptr) return;
                    if (i % 2 != 0 || j % 2 != 0 || k % 2 != 0) return;
                    auto ta = te->fabs[b].ca();
                    bool te_res = false;
                    for (int n = 0; n < ncomp_te; ++n) {
                        double mte = P::te_modifier(n, s, i, j, k, lev, time, dt, dx, ta(i, j, k, n), params_mod);
                        if (mte >= te_crit[n]) {
                            te_res = true;
                            if (ntags_trunc) ntags_trunc[n] += 8;
                        }
                    }
                    if (te_res) {
                        setm(i, j, k); setm(i + 1, j, k); setm(i, j + 1, k); setm(i, j, k + 1);
                        setm(i + 1, j + 1, k); setm(i, j + 1, k + 1); setm(i + 1, j, k + 1);
                        setm(i + 1, j + 1, k + 1);
                        if (ntags_total) (*ntags_total) += 8 - (int)res;
                    }
                });
            }
    }
}

/* ---- GW spectrum ------------------------------------------------------------*/

/* pySledgehamr/Sledgehamr.py:7-12: sorted unique i^2+j^2+k^2 over the
 * integer FFT frequencies of a grid of size dim. */
inline std::vector<long long> unique_k2(int dim) {
    std::vector<long long> sq;
    for (int a = 0; a < dim; ++a) {
        long long f = a < (dim + 1) / 2 ? a : a - dim; /* numpy fftfreq * dim */
        sq.push_back(f * f);
    }
    std::sort(sq.begin(), sq.end());
    sq.erase(std::unique(sq.begin(), sq.end()), sq.end());
    std::vector<long long> out;
    for (long long x : sq)
        for (long long y : sq)
            for (long long z : sq) out.push_back(x + y + z);
    std::sort(out.begin(), out.end());
    out.erase(std::unique(out.begin(), out.end()), out.end());
    return out;
}

/* pySledgehamr/Sledgehamr.py:18-27 (types 1 and 2); type 3 is the
 * eigenvalue of the 6th-order central first difference. */
inline std::vector<double> index_to_k(int N, int projection_type) {
    std::vector<double> r(N);
    for (int a = 0; a < N; ++a) {
        double nt = (double)a;
        if ((double)a - N > -N / 2.0 - 1) nt -= N;
        double x = 2. * M_PI / N * nt;
        if (projection_type == 1) r[a] = std::sin(x);
        else if (projection_type == 2) r[a] = (8. * std::sin(x) - std::sin(2. * x)) / 6.;
        else r[a] = (45. * std::sin(x) - 9. * std::sin(2. * x) + std::sin(3. * x)) / 30.;
    }
    return r;
}

/* In-place complex FFT of length n (forward, e^{-2 pi i jk/n}), mixed radix
 * by recursion on the smallest prime factor, direct DFT for prime n. */
inline void fft1d(std::complex<double> *x, int n, int stride, std::vector<std::complex<double>> &buf) {
    if (n == 1) return;
    int p = 2;
    while (p * p <= n && n % p != 0) ++p;
    if (n % p != 0) p = n;
    const int m = n / p;
    std::vector<std::complex<double>> tmp(n);
    for (int j = 0; j < n; ++j) tmp[j] = x[(long long)j * stride];
    if (p == n) {
        for (int k = 0; k < n; ++k) {
            std::complex<double> s = 0;
            for (int j = 0; j < n; ++j) {
                double ang = -2. * M_PI * (double)((long long)j * k % n) / n;
                s += tmp[j] * std::complex<double>(std::cos(ang), std::sin(ang));
            }
            x[(long long)k * stride] = s;
        }
        return;
    }
    /* split into p subsequences of length m: sub_r[q] = tmp[q*p + r] */
    std::vector<std::complex<double>> sub((size_t)p * m);
    for (int r = 0; r < p; ++r)
        for (int q = 0; q < m; ++q) sub[(size_t)r * m + q] = tmp[(size_t)q * p + r];
    for (int r = 0; r < p; ++r) fft1d(sub.data() + (size_t)r * m, m, 1, buf);
    for (int k = 0; k < n; ++k) {
        std::complex<double> s = 0;
        for (int r = 0; r < p; ++r) {
            double ang = -2. * M_PI * (double)((long long)r * k % n) / n;
            s += sub[(size_t)r * m + (k % m)] * std::complex<double>(std::cos(ang), std::sin(ang));
        }
        x[(long long)k * stride] = s;
    }
}

/* Unnormalised forward R2C transform of an N^3 real field (x fastest):
 * out[(c*N + b)*(N/2+1) + a] for a in [0, N/2], b, c in [0, N). */
inline void rfft3d(const double *in, int N, std::vector<std::complex<double>> &out) {
    const int H = N / 2 + 1;
    std::vector<std::complex<double>> full((size_t)N * N * N);
    for (size_t i = 0; i < full.size(); ++i) full[i] = in[i];
    std::vector<std::complex<double>> buf;
    for (int c = 0; c < N; ++c)
        for (int b = 0; b < N; ++b) fft1d(full.data() + ((size_t)c * N + b) * N, N, 1, buf);
    for (int c = 0; c < N; ++c)
        for (int a = 0; a < N; ++a) fft1d(full.data() + (size_t)c * N * N + a, N, N, buf);
    for (int b = 0; b < N; ++b)
        for (int a = 0; a < N; ++a) fft1d(full.data() + (size_t)b * N + a, N, N * N, buf);
    out.assign((size_t)H * N * N, 0);
    for (int c = 0; c < N; ++c)
        for (int b = 0; b < N; ++b)
            for (int a = 0; a < H; ++a) out[((size_t)c * N + b) * H + a] = full[((size_t)c * N + b) * N + a];
}

/* gw_GetProjection / gw_GetLambda, source/gravitational_waves.h:101-133. */
inline double gw_projection(int i, int j, const double abc[3]) {
    double norm = abc[0] * abc[0] + abc[1] * abc[1] + abc[2] * abc[2];
    int l = std::min(i, j), m = std::max(i, j);
    double proj = abc[l] * abc[m];
    return static_cast<double>(l == m) - proj / norm;
}
inline double gw_lambda(int i, int j, int l, int m, const int abc[3], const double *index_to_k) {
    if (abc[0] == 0 && abc[1] == 0 && abc[2] == 0) return 0.;
    double d[3] = {index_to_k[abc[0]], index_to_k[abc[1]], index_to_k[abc[2]]};
    return gw_projection(i, l, d) * gw_projection(j, m, d) -
           gw_projection(i, j, d) * gw_projection(l, m, d) / 2.;
}

/* GravitationalWaves::ComputeSpectrum (CPU branch), for the six selected
 * tensor components given as N^3 arrays (x fastest) of a single periodic
 * level.  zero_padding p embeds each field in the first N^3 block of a
 * (pN)^3 zero grid.  Returns the spectrum per bin and fills ks with k^2 of
 * the bins. */
inline std::vector<double> gw_spectrum(const std::vector<const double *> &comps6, int N,
                                       int zero_padding, int projection_type, bool unbinned,
                                       std::vector<long long> &ks) {
    const int dimN = N * zero_padding;
    const int H = dimN / 2 + 1;
    std::vector<std::vector<std::complex<double>>> spec(6);
    std::vector<double> padded((size_t)dimN * dimN * dimN);
    for (int q = 0; q < 6; ++q) {
        std::fill(padded.begin(), padded.end(), 0.0);
        for (int c = 0; c < N; ++c)
            for (int b = 0; b < N; ++b)
                for (int a = 0; a < N; ++a)
                    padded[((size_t)c * dimN + b) * dimN + a] = comps6[q][((size_t)c * N + b) * N + a];
        rfft3d(padded.data(), dimN, spec[q]);
    }
    const double dimN6 = std::pow((double)dimN, 6);
    const int mat[3][3] = {{0, 1, 2}, {1, 3, 4}, {2, 4, 5}};
    std::vector<double> itk = index_to_k(dimN, projection_type);
    if (unbinned) {
        ks = unique_k2(dimN);
    } else {
        ks.clear();
        for (int k = 0; k <= std::sqrt(3.) / 2. * static_cast<double>(dimN) + .5; ++k) ks.push_back((long long)k * k);
    }
    const int kmax = (int)ks.size();
    std::vector<double> out(kmax, 0.0);
    for (int c = 0; c < dimN; ++c)
        for (int b = 0; b < dimN; ++b)
            for (int a = 0; a < H; ++a) {
                double multpl = (a == 0 || a == dimN / 2) ? 1. : 2.;
                int abc[3] = {a, b, c};
                double running_sum = 0;
                int li = a >= dimN / 2 ? a - dimN : a;
                int lj = b >= dimN / 2 ? b - dimN : b;
                int lk = c >= dimN / 2 ? c - dimN : c;
                unsigned int sq = li * li + lj * lj + lk * lk;
                size_t index;
                if (unbinned)
                    index = std::lower_bound(ks.begin(), ks.end(), (long long)sq) - ks.begin();
                else
                    index = static_cast<long>(std::sqrt(static_cast<double>(sq)) + .5);
                size_t off = ((size_t)c * dimN + b) * H + a;
                for (int i = 0; i < 3; ++i)
                    for (int j = 0; j < 3; ++j)
                        for (int l = 0; l < 3; ++l)
                            for (int m = 0; m < 3; ++m) {
                                const auto &u = spec[mat[i][j]][off];
                                const auto &v = spec[mat[l][m]][off];
                                running_sum += gw_lambda(i, j, l, m, abc, itk.data()) * multpl *
                                               (u.real() * v.real() + u.imag() * v.imag());
                            }
                out[index] += running_sum;
            }
    for (int c = 0; c < kmax; ++c) out[c] /= dimN6;
    return out;
}


/* Per-cell output functions of the projects (values for projections and
 * scalar spectra), components of the AxionStrings layout Psi1 Psi2 Pi1 Pi2
 * (0..3) or one component `comp`:
 *   0 state(comp)                    1 state(comp)^2 (FOPT dPhi2 with comp 1,
 *                                      projects/FirstOrderPhaseTransition/
 *                                      kernels_misc.h:10-18)
 *   2 a'^2 = ((Psi1 Pi2 - Psi2 Pi1) / r^2)^2, r^2 = Psi1^2 + Psi2^2
 *     (projects/AxionStrings/kernels_energy_densities.h:21-33; also
 *     NextToMinimalExample a_dot_sq, NextToMinimalExample.h:49-61)
 *   3 a'_screened = Psi1 Pi2 - Psi2 Pi1 (kernels_energy_densities.h:48-58)
 *   4 r'^2 = (Psi1 Pi1 + Psi2 Pi2)^2 / r^2 (kernels_energy_densities.h:73-85) */
inline double out_function(int fn, int comp, const double *v, long long stride) {
    if (fn == 0) return v[comp * stride];
    if (fn == 1) return v[comp * stride] * v[comp * stride];
    const double Psi1 = v[0], Psi2 = v[stride], Pi1 = v[2 * stride], Pi2 = v[3 * stride];
    if (fn == 2) {
        double r2 = Psi1 * Psi1 + Psi2 * Psi2;
        double prime_a = (Psi1 * Pi2 - Psi2 * Pi1) / r2;
        return prime_a * prime_a;
    }
    if (fn == 3) return Psi1 * Pi2 - Psi2 * Pi1;
    double r2 = Psi1 * Psi1 + Psi2 * Psi2;
    double prime_r = Psi1 * Pi1 + Psi2 * Pi2;
    return prime_r * prime_r / r2;
}

/* Spectrum::Compute (source/output_types/spectrum.cpp:12-113) for a
 * periodic N^3 level given as a canonical array (ncomp components): the
 * output function per cell, its R2C FFT, |F| (utils::Fft with abs,
 * fft.h:244-250) and the sum of multpl * pre * |F| * |F| into the bins of
 * the sorted unique k^2 (lower_bound), multpl = 1 on the x planes 0 and
 * N/2, else 2, pre = t / (N^6 dk), dk = 2 pi / L. */
inline std::vector<double> scalar_spectrum(const double *state, int N, int ncomp, int fn,
                                           int comp, double L, double t,
                                           std::vector<long long> &ks) {
    (void)ncomp;
    const long long n3 = (long long)N * N * N;
    std::vector<double> f((size_t)n3);
    for (long long q = 0; q < n3; ++q) f[q] = out_function(fn, comp, state + q, n3);
    std::vector<std::complex<double>> F;
    rfft3d(f.data(), N, F);
    const int H = N / 2 + 1;
    double fac = std::pow(1. / N, 6);
    double dk = 2. * M_PI / L;
    double pre = fac * t / dk;
    ks = unique_k2(N);
    std::vector<double> spectrum(ks.size(), 0.0);
    /* loop order of the reference on one thread: i (x) outer, k (z) inner */
    for (int a = 0; a < H; ++a)
        for (int b = 0; b < N; ++b)
            for (int c = 0; c < N; ++c) {
                double multpl = (a == 0 || a == N / 2) ? 1. : 2.;
                int li = a >= N / 2 ? a - N : a;
                int lj = b >= N / 2 ? b - N : b;
                int lk = c >= N / 2 ? c - N : c;
                long long sq = (long long)li * li + (long long)lj * lj + (long long)lk * lk;
                size_t index = std::lower_bound(ks.begin(), ks.end(), sq) - ks.begin();
                const std::complex<double> &z = F[((size_t)c * N + b) * H + a];
                double absF = std::sqrt(z.real() * z.real() + z.imag() * z.imag());
                spectrum[index] += multpl * pre * absF * absF;
            }
    return spectrum;
}

/* Projection::Compute and Projection::Add (source/output_types/
 * projection.cpp:10-118): line-of-sight projection along z onto the pixel
 * grid of the finest of the given levels (levels[0..mlevel]); a cell of
 * level lev not covered by level lev+1 (the cell (2i, 2j, 2k) in none of its
 * boxes) covers ratio x ratio pixels, ratio = dimN / dimN_lev; mode 0 adds
 * ratio * value, mode 1 keeps the maximum (data starts at 0); n counts the
 * contributions.  Pixel index (i ratio + a) dimN + (j ratio + b). */
inline void projection(const std::vector<const MF *> &levels, int fn, int comp, int mode,
                       std::vector<double> &data, std::vector<int> &nproj) {
    const int mlevel = (int)levels.size() - 1;
    const int dimN = levels[mlevel]->domain.len(0);
    data.assign((size_t)dimN * dimN, 0.0);
    nproj.assign((size_t)dimN * dimN, 0);
    for (int lev = 0; lev <= mlevel; ++lev) {
        const MF &mf = *levels[lev];
        const int ratio = dimN / mf.domain.len(0);
        for (const Fab &f : mf.fabs) {
            auto a = f.ca();
            for (int k = f.vbox.lo.z; k <= f.vbox.hi.z; ++k)
                for (int j = f.vbox.lo.y; j <= f.vbox.hi.y; ++j)
                    for (int i = f.vbox.lo.x; i <= f.vbox.hi.x; ++i) {
                        bool contd = lev == mlevel ||
                                     find_fab(*levels[lev + 1], 2 * i, 2 * j, 2 * k) < 0;
                        if (!contd) continue;
                        const double val = out_function(fn, comp, &a(i, j, k, 0), a.ns);
                        const int ii = i * ratio, jj = j * ratio;
                        for (int ia = 0; ia < ratio; ++ia)
                            for (int ja = 0; ja < ratio; ++ja) {
                                const long long ind = (long long)(ii + ia) * dimN + (jj + ja);
                                if (mode == 0) data[ind] += ratio * val;
                                else if (mode == 1) data[ind] = std::max(data[ind], val);
                                nproj[ind] += 1;
                            }
                    }
        }
    }
}

} // namespace orc

#endif // SH_ORACLE_CORE_H_
