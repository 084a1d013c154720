/* ORACLE (test infrastructure only): AMR hierarchy on the CPU.
 *
 * The host time stepper (subcycling, shadow level, regrid scheduling, new
 * grids) is the library's own sh_amr_driver.h, so that both sides take the
 * same decisions; every numerical operation below is the oracle's
 * restatement:
 *   Integrator::Advance with FillPatch / FillIntermediatePatch for lev > 0
 *     (source/integrators/integrator.cpp:11-31,
 *      source/level_synchronizer.cpp:94-214): fine ghost cells take the
 *     valid value of their periodic image on the same level where one
 *     exists; the others are interpolated from the coarse level.
 *   coarse data at time t (GetLevelData, level_synchronizer.cpp:613-632):
 *     new or old when t is within 1e-3 (t_new - t_old) of their time,
 *     otherwise (t_new - t)/(t_new - t_old) old + (t - t_old)/(t_new - t_old) new.
 *   spatial interpolation: the quadratic interpolant through the 3x3x3
 *     coarse cells around the parent, with centred first and second
 *     differences and the four-point mixed differences, evaluated at the
 *     fine-cell centre (offsets -1/4, +1/4 in coarse units).  This restates
 *     AMReX's documented CellQuadratic interpolation (the default
 *     amr.interpolation_type, level_synchronizer.cpp:27-47); AMReX's
 *     operation order is not available here: parity unpinned.
 *   FillCoarsePatch (level_synchronizer.cpp:56-82) and RemakeLevel's
 *     FillPatch (sledgehamr.cpp:173-189) on whole new levels.
 *   average-down, average-down with truncation errors, CPU tagging: as in
 *     oracle_core.h.
 */
#include <memory>

#include "../include/sledgehamr_gb300.h"
#include "../sledgehamr_gb300/csrc/sh_amr_driver.h"
#include "../sledgehamr_gb300/csrc/sh_checkpoint.h"
#include "oracle_projects.h"

namespace orc {

struct CoarseAt {
    const MF *old_ = nullptr, *new_ = nullptr;
    int mode = 1;
    double alpha = 0, beta = 0;
    std::vector<A4<const double>> ao, an;

    CoarseAt(const MF &o, const MF &n, double t) : old_(&o), new_(&n) {
        const double tn = n.t, to = o.t;
        const double teps = std::fabs(tn - to) * 1.e-3;
        if (t > tn - teps && t < tn + teps) {
            mode = 1;
        } else if (t > to - teps && t < to + teps) {
            mode = 0;
        } else {
            mode = 2;
            alpha = (tn - t) / (tn - to);
            beta = (t - to) / (tn - to);
        }
        for (const Fab &f : o.fabs) ao.push_back(f.ca());
        for (const Fab &f : n.fabs) an.push_back(f.ca());
    }
    /* quadratic interpolant at fine cell (fi, fj, fk), all components */
    void interp(int fi, int fj, int fk, int nc, double *out) const {
        auto fl = [](int a) { return a >= 0 ? a / 2 : -((-a + 1) / 2); };
        const int I = fl(fi), J = fl(fj), K = fl(fk);
        const double xi = (fi - 2 * I) ? 0.25 : -0.25;
        const double yi = (fj - 2 * J) ? 0.25 : -0.25;
        const double zi = (fk - 2 * K) ? 0.25 : -0.25;
        const Box &d = new_->domain;
        int fab[27], ii[27], jj[27], kk[27];
        for (int c = -1; c <= 1; ++c)
            for (int b = -1; b <= 1; ++b)
                for (int a = -1; a <= 1; ++a) {
                    const int q = (c + 1) * 9 + (b + 1) * 3 + (a + 1);
                    ii[q] = d.lo.x + pmod(I + a - d.lo.x, d.len(0));
                    jj[q] = d.lo.y + pmod(J + b - d.lo.y, d.len(1));
                    kk[q] = d.lo.z + pmod(K + c - d.lo.z, d.len(2));
                    fab[q] = find_fab(*new_, ii[q], jj[q], kk[q]);
                    if (fab[q] < 0)
                        throw std::runtime_error("coarse level does not cover an interpolation point");
                }
        for (int n = 0; n < nc; ++n) {
            auto u = [&](int a, int b, int c) {
                const int q = (c + 1) * 9 + (b + 1) * 3 + (a + 1);
                const double vn = an[fab[q]](ii[q], jj[q], kk[q], n);
                if (mode == 1) return vn;
                const double vo = ao[fab[q]](ii[q], jj[q], kk[q], n);
                if (mode == 0) return vo;
                return alpha * vo + beta * vn;
            };
            const double u0 = u(0, 0, 0);
            const double dxp = u(1, 0, 0), dxm = u(-1, 0, 0);
            const double dyp = u(0, 1, 0), dym = u(0, -1, 0);
            const double dzp = u(0, 0, 1), dzm = u(0, 0, -1);
            const double Dx = (dxp - dxm) * 0.5, Dy = (dyp - dym) * 0.5, Dz = (dzp - dzm) * 0.5;
            const double Dxx = dxp - 2. * u0 + dxm;
            const double Dyy = dyp - 2. * u0 + dym;
            const double Dzz = dzp - 2. * u0 + dzm;
            const double Dxy = (u(1, 1, 0) - u(1, -1, 0) - u(-1, 1, 0) + u(-1, -1, 0)) * 0.25;
            const double Dxz = (u(1, 0, 1) - u(1, 0, -1) - u(-1, 0, 1) + u(-1, 0, -1)) * 0.25;
            const double Dyz = (u(0, 1, 1) - u(0, 1, -1) - u(0, -1, 1) + u(0, -1, -1)) * 0.25;
            out[n] = u0 + xi * Dx + yi * Dy + zi * Dz +
                     0.5 * (xi * xi * Dxx + yi * yi * Dyy + zi * zi * Dzz) + xi * yi * Dxy +
                     xi * zi * Dxz + yi * zi * Dyz;
        }
    }
};

/* Ghost cells of mf at time t: periodic images on the same level, else the
 * coarse level (if any). */
inline void fill_two_level(MF &mf, double t, const MF *co, const MF *cn) {
    fill_boundary_periodic(mf);
    if (!cn) return;
    CoarseAt c(*co, *cn, t);
    const int NX = mf.domain.len(0), NY = mf.domain.len(1), NZ = mf.domain.len(2);
    const IV dlo = mf.domain.lo;
    for (Fab &fab : mf.fabs) {
        auto d = fab.a();
        for_cells(fab.gbox(), [&](int i, int j, int k) {
            if (fab.vbox.contains(i, j, k)) return;
            int si = dlo.x + pmod(i - dlo.x, NX), sj = dlo.y + pmod(j - dlo.y, NY),
                sk = dlo.z + pmod(k - dlo.z, NZ);
            if (find_fab(mf, si, sj, sk) >= 0) return;
            double v[64];
            c.interp(i, j, k, mf.nc, v);
            for (int n = 0; n < mf.nc; ++n) d(i, j, k, n) = v[n];
        });
    }
}

/* All cells of dst from src's valid cells (periodic images) where they
 * exist, else from the coarse level at time t. */
inline void fill_from(MF &dst, const MF *src, double t, const MF &co, const MF &cn) {
    CoarseAt c(co, cn, t);
    const int NX = dst.domain.len(0), NY = dst.domain.len(1), NZ = dst.domain.len(2);
    const IV dlo = dst.domain.lo;
    for (Fab &fab : dst.fabs) {
        auto d = fab.a();
        for_cells(fab.gbox(), [&](int i, int j, int k) {
            if (src) {
                int si = dlo.x + pmod(i - dlo.x, NX), sj = dlo.y + pmod(j - dlo.y, NY),
                    sk = dlo.z + pmod(k - dlo.z, NZ);
                int f = find_fab(*src, si, sj, sk);
                if (f >= 0) {
                    auto s = src->fabs[f].ca();
                    for (int n = 0; n < dst.nc; ++n) d(i, j, k, n) = s(si, sj, sk, n);
                    return;
                }
            }
            double v[64];
            c.interp(i, j, k, dst.nc, v);
            for (int n = 0; n < dst.nc; ++n) d(i, j, k, n) = v[n];
        });
    }
}

template <class P>
struct CpuBackend {
    struct Lvl {
        MF nw, od;
        int lev = 0;
    };
    using Level = Lvl *;
    sh_amr_config cfg;
    int ncomp = 0;
    IntegratorSpec spec;

    Level create(int lev, const std::vector<shamr::IBox> &boxes, int N) {
        Lvl *l = new Lvl();
        l->lev = lev;
        std::vector<Box> bx;
        for (const auto &b : boxes)
            bx.push_back(Box{{b.lo[0], b.lo[1], b.lo[2]}, {b.hi[0], b.hi[1], b.hi[2]}});
        Box dom{{0, 0, 0}, {N - 1, N - 1, N - 1}};
        l->nw.define(dom, bx, ncomp, cfg.nghost);
        l->od.define(dom, bx, ncomp, cfg.nghost);
        return l;
    }
    void destroy(Level &l) {
        delete l;
        l = nullptr;
    }
    MF &buf(Level l, int which) { return which == shamr::kNew ? l->nw : l->od; }
    double time(const Level &l, int which) { return buf(l, which).t; }
    int istep(const Level &l, int which) { return buf(l, which).istep; }
    void set_time(Level &l, int which, double t, int s) {
        buf(l, which).t = t;
        buf(l, which).istep = s;
    }
    RhsConfig rhs_config(int lev, double dt, double dx) {
        RhsConfig c;
        c.lev = lev;
        c.dt = dt;
        c.dx = dx;
        c.params = cfg.params;
        c.gw_params = cfg.gw_params;
        c.with_gw = cfg.with_gw != 0;
        return c;
    }
    void advance(int lev, Level &l, Level *coarse, double dt, double dx, bool no_swap) {
        if (!no_swap) std::swap(l->nw, l->od);
        const MF *co = coarse ? &(*coarse)->od : nullptr;
        const MF *cn = coarse ? &(*coarse)->nw : nullptr;
        fill_two_level(l->od, l->od.t, co, cn);
        StepContext sc;
        sc.with_gw = cfg.with_gw != 0;
        sc.ncomp_user = ncomp - (cfg.with_gw ? 12 : 0);
        sc.fill = [&](MF &mf, double t) { fill_two_level(mf, t, co, cn); };
        integrate<P>(spec, l->od, l->nw, dt, rhs_config(lev, dt, dx), sc);
        l->nw.t = l->od.t + dt;
        l->nw.istep = l->od.istep + 1;
    }
    void average_down(Level &f, int wf, Level &c, int wc) {
        orc::average_down(buf(f, wf), buf(c, wc), ncomp);
    }
    void average_down_te(Level &f, Level &c) {
        average_down_with_te(f->nw, c->nw, f->od, ncomp);
    }
    std::vector<uint8_t> tag(Level &l, bool use_te, double time, int lev, double dt, double dx) {
        std::vector<std::vector<uint8_t>> m;
        tag_cpu_literal<P>(l->nw, use_te ? &l->od : nullptr, time, lev, dt, dx, cfg.te_crit,
                           ncomp, cfg.params_tag, cfg.params_mod, m, nullptr, nullptr, nullptr);
        std::vector<uint8_t> out;
        for (auto &v : m) out.insert(out.end(), v.begin(), v.end());
        return out;
    }
    std::vector<uint8_t> tag_blocks(Level &l, bool use_te, double time, int lev, double dt,
                                    double dx, int block, int buffer, int nb) {
        std::vector<shamr::IBox> bx;
        for (const Fab &f : l->nw.fabs)
            bx.push_back(shamr::IBox{{f.vbox.lo.x, f.vbox.lo.y, f.vbox.lo.z},
                                     {f.vbox.hi.x, f.vbox.hi.y, f.vbox.hi.z}});
        return shamr::mask_to_blocks(tag(l, use_te, time, lev, dt, dx), bx, block, buffer, nb);
    }
    void fill_from_coarse(Level &f, Level &c, double time) {
        fill_from(f->nw, nullptr, time, c->od, c->nw);
    }
    void remake(Level &fresh, Level &old, Level &c, double time) {
        fill_from(fresh->nw, &old->nw, time, c->od, c->nw);
    }
    void extend(Level &fresh, Level &old, Level &c, double t_new, double t_old) {
        fill_from(fresh->nw, &old->nw, t_new, c->od, c->nw);
        fill_from(fresh->od, &old->od, t_old, c->od, c->nw);
    }
    void refresh_ghosts(Level &l, int which, Level *coarse) {
        MF &m = buf(l, which);
        fill_two_level(m, m.t, coarse ? &(*coarse)->od : nullptr,
                       coarse ? &(*coarse)->nw : nullptr);
    }
    void sync() {}
    /* valid cells in the boxes layout (box after box, comp-major) */
    std::vector<double> read_valid(Level &l, int which) {
        const MF &m = buf(l, which);
        std::vector<double> v;
        for (const Fab &f : m.fabs) {
            auto a = f.ca();
            for (int n = 0; n < m.nc; ++n)
                for_cells(f.vbox, [&](int i, int j, int k) { v.push_back(a(i, j, k, n)); });
        }
        return v;
    }
    void write_valid(Level &l, int which, const std::vector<double> &v) {
        MF &m = buf(l, which);
        size_t q = 0;
        for (Fab &f : m.fabs) {
            auto a = f.a();
            for (int n = 0; n < m.nc; ++n)
                for_cells(f.vbox, [&](int i, int j, int k) {
                    if (q >= v.size()) throw std::runtime_error("checkpoint data too short");
                    a(i, j, k, n) = v[q++];
                });
        }
        if (q != v.size()) throw std::runtime_error("checkpoint data too long");
    }
    /* FirstOrderPhaseTransition.cpp:133-157: params_mod = norm0 of every
     * component of level 0's new data, once per time */
    double maxima_time = -DBL_MAX;
    void params_mod_from_norm0(Level &l0, double time) {
        if (time == maxima_time) return;
        for (int n = 0; n < ncomp; ++n) {
            double m = 0.;
            for (Fab &f : l0->nw.fabs) {
                auto a = f.a();
                for_cells(f.vbox, [&](int i, int j, int k) {
                    const double v = std::fabs(a(i, j, k, n));
                    if (v > m) m = v;
                });
            }
            cfg.params_mod[n] = m;
        }
        cfg.nparams_mod = ncomp;
        maxima_time = time;
    }
};

struct AmrBase {
    virtual ~AmrBase() = default;
    virtual void step(int n) = 0;
    virtual int finest() const = 0;
    virtual long long cell_updates() const = 0;
    virtual int nregrids() const = 0;
    virtual const shamr::RegridRecord &record(int q) const = 0;
    virtual const MF *level(int lev, int which) const = 0;
    virtual const std::vector<shamr::IBox> &boxes(int lev) const = 0;
    virtual void set_tag_params(const double *pt, int nt, const double *pm, int nm) = 0;
    virtual void set_trace(bool on) = 0;
    virtual shamr::Checkpoint checkpoint() = 0;
    virtual void restart(const shamr::Checkpoint &k) = 0;
    virtual const std::vector<std::string> &trace() const = 0;
};

template <class P>
struct Amr : AmrBase {
    CpuBackend<P> backend;
    std::unique_ptr<shamr::Driver<CpuBackend<P>>> drv;
    Amr(const sh_amr_config &cfg, int ncomp, const double *level0) {
        backend.cfg = cfg;
        backend.ncomp = ncomp;
        backend.spec.type = cfg.integrator;
        if (cfg.integrator == RknButcherTableau) throw std::runtime_error("user tableau unsupported");
        shamr::Config d;
        d.N0 = cfg.N0;
        d.L = cfg.L;
        d.cfl = cfg.cfl;
        d.t_start = cfg.t_start;
        d.nghost = cfg.nghost;
        d.max_level = cfg.max_level;
        d.blocking_factor = cfg.blocking_factor;
        d.max_grid_size = cfg.max_grid_size;
        d.n_error_buf = cfg.n_error_buf;
        d.regrid_dt = cfg.regrid_dt;
        d.string_width_threshold = cfg.string_width_threshold;
        d.string_lambda = cfg.string_lambda;
        d.te_crit.assign(cfg.te_crit, cfg.te_crit + ncomp);
        d.clustering = cfg.clustering;
        d.grid_eff = cfg.grid_eff;
        d.params_mod_norm0 = cfg.params_mod_norm0 != 0;
        d.max_local_regrids = cfg.max_local_regrids;
        d.volume_threshold_strong = cfg.volume_threshold_strong;
        d.volume_threshold_weak = cfg.volume_threshold_weak;
        drv.reset(new shamr::Driver<CpuBackend<P>>(backend, d));
        drv->record_regrids = cfg.record_regrids != 0;
        const int N = cfg.N0;
        drv->init_coarse([&](typename CpuBackend<P>::Lvl *&l) {
            for (Fab &f : l->nw.fabs) {
                auto a = f.a();
                for (int n = 0; n < ncomp; ++n)
                    for_cells(f.vbox, [&](int i, int j, int k) {
                        a(i, j, k, n) = level0[(((size_t)n * N + k) * N + j) * N + i];
                    });
            }
        });
    }
    void step(int n) override {
        for (int q = 0; q < n; ++q) drv->step();
    }
    int finest() const override { return drv->finest; }
    long long cell_updates() const override { return drv->cell_updates; }
    int nregrids() const override { return (int)drv->regrids.size(); }
    const shamr::RegridRecord &record(int q) const override { return drv->regrids[q]; }
    const MF *level(int lev, int which) const override {
        return which == 0 ? &drv->levels[lev]->nw : &drv->levels[lev]->od;
    }
    const std::vector<shamr::IBox> &boxes(int lev) const override { return drv->boxes[lev]; }
    void set_trace(bool on) override { drv->record_trace = on; }
    shamr::Checkpoint checkpoint() override { return drv->checkpoint(); }
    void restart(const shamr::Checkpoint &k) override { drv->restart(k); }
    const std::vector<std::string> &trace() const override { return drv->trace; }
    void set_tag_params(const double *pt, int nt, const double *pm, int nm) override {
        for (int q = 0; q < nt; ++q) backend.cfg.params_tag[q] = pt[q];
        for (int q = 0; q < nm; ++q) backend.cfg.params_mod[q] = pm[q];
        backend.cfg.nparams_tag = nt;
        backend.cfg.nparams_mod = nm;
    }
};

} // namespace orc

using namespace orc;

extern "C" {

void *orc_amr_create(const sh_amr_config *cfg, const double *level0) {
    try {
        const int gw = cfg->with_gw ? 12 : 0;
        switch (cfg->project) {
        case 0: return new Amr<AxionStrings>(*cfg, 4 + gw, level0);
        case 1: return new Amr<MinimalExample>(*cfg, 4, level0);
        case 2: return new Amr<NextToMinimalExample>(*cfg, 4, level0);
        case 3: return new Amr<FirstOrderPhaseTransition>(*cfg, 2 + gw, level0);
        case 4: return new Amr<AxionStringsLap<1>>(*cfg, 4, level0);
        case 5: return new Amr<AxionStringsLap<2>>(*cfg, 4, level0);
        case 6: return new Amr<AxionStringsLap<3>>(*cfg, 4, level0);
        default: return nullptr;
        }
    } catch (...) {
        return nullptr;
    }
}

void orc_amr_destroy(void *h) { delete (AmrBase *)h; }

int orc_amr_set_tag_params(void *h, const double *params_tag, int ntag, const double *params_mod,
                           int nmod) {
    if (ntag < 0 || ntag > 32 || nmod < 0 || nmod > 32) return -1;
    ((AmrBase *)h)->set_tag_params(params_tag, ntag, params_mod, nmod);
    return 0;
}

int orc_amr_step(void *h, int n) {
    try {
        ((AmrBase *)h)->step(n);
        return 0;
    } catch (const std::exception &e) {
        fprintf(stderr, "orc_amr_step: %s\n", e.what());
        return -3;
    }
}

int orc_amr_info(void *h, int *finest, long long *cell_updates, int *nregrids) {
    AmrBase *a = (AmrBase *)h;
    if (finest) *finest = a->finest();
    if (cell_updates) *cell_updates = a->cell_updates();
    if (nregrids) *nregrids = a->nregrids();
    return 0;
}

/* The new-grid step alone (shamr::make_boxes): boxes in block coordinates
 * (6 ints each) of the set blocks of tags (nb^3, x fastest) inside the
 * allowed blocks; returns their number, or -1 if cap is too small. */
int orc_make_boxes(const unsigned char *tags, const unsigned char *allowed, int nb,
                   int clustering, double grid_eff, int w, int *out, int cap) {
    const size_t n = (size_t)nb * nb * nb;
    std::vector<uint8_t> t(tags, tags + n), a(allowed, allowed + n);
    const auto b = shamr::make_boxes(t, a, nb, clustering, grid_eff, w);
    if ((int)b.size() > cap) return -1;
    for (size_t q = 0; q < b.size(); ++q)
        for (int d = 0; d < 3; ++d) {
            out[6 * q + d] = b[q].lo[d];
            out[6 * q + 3 + d] = b[q].hi[d];
        }
    return (int)b.size();
}

/* Checkpoint files of the hierarchy (shamr::write_checkpoint) and a new
 * hierarchy restarted from them (level0 of the creation is replaced). */
int orc_amr_checkpoint(void *h, const char *folder) {
    try {
        std::string err;
        if (!shamr::write_checkpoint(((AmrBase *)h)->checkpoint(), folder, &err)) {
            fprintf(stderr, "orc_amr_checkpoint: %s\n", err.c_str());
            return -1;
        }
        return 0;
    } catch (const std::exception &e) {
        fprintf(stderr, "orc_amr_checkpoint: %s\n", e.what());
        return -1;
    }
}
void *orc_amr_restart(const sh_amr_config *cfg, const char *folder) {
    shamr::Checkpoint k;
    std::string err;
    if (!shamr::read_checkpoint(folder, &k, &err)) {
        fprintf(stderr, "orc_amr_restart: %s\n", err.c_str());
        return nullptr;
    }
    std::vector<double> zero((size_t)k.ncomp * cfg->N0 * cfg->N0 * cfg->N0, 0.);
    AmrBase *a = (AmrBase *)orc_amr_create(cfg, zero.data());
    if (!a) return nullptr;
    try {
        a->restart(k);
    } catch (const std::exception &e) {
        fprintf(stderr, "orc_amr_restart: %s\n", e.what());
        delete a;
        return nullptr;
    }
    return a;
}

/* The time stepper's operation trace (shamr::Driver::trace): record_trace
 * on or off, and the events so far as one string, newline-separated, into
 * buf (capacity cap); returns the string's length (-1 if cap is too small). */
int orc_amr_set_trace(void *h, int on) {
    ((AmrBase *)h)->set_trace(on != 0);
    return 0;
}
long long orc_amr_trace(void *h, char *buf, long long cap) {
    std::string all;
    for (const std::string &e : ((AmrBase *)h)->trace()) all += e + "\n";
    if (!buf) return (long long)all.size();
    if ((long long)all.size() + 1 > cap) return -1;
    std::memcpy(buf, all.c_str(), all.size() + 1);
    return (long long)all.size();
}

/* Boxes (6 ints each) of level lev; returns their number. */
int orc_amr_boxes(void *h, int lev, int *out, int cap) {
    AmrBase *a = (AmrBase *)h;
    if (lev < 0 || lev > a->finest()) return -1;
    const auto &b = a->boxes(lev);
    if ((int)b.size() > cap) return -1;
    for (size_t q = 0; q < b.size(); ++q)
        for (int d = 0; d < 3; ++d) {
            out[6 * q + d] = b[q].lo[d];
            out[6 * q + 3 + d] = b[q].hi[d];
        }
    return (int)b.size();
}

/* Level data in the boxes layout (valid cells, box-major, comp-major). */
int orc_amr_read(void *h, int lev, int which, double *out, double *t) {
    AmrBase *a = (AmrBase *)h;
    if (lev < 0 || lev > a->finest()) return -1;
    const MF *m = a->level(lev, which);
    size_t q = 0;
    for (const Fab &f : m->fabs) {
        auto ac = f.ca();
        for (int n = 0; n < m->nc; ++n)
            for_cells(f.vbox, [&](int i, int j, int k) { out[q++] = ac(i, j, k, n); });
    }
    if (t) *t = m->t;
    return 0;
}

int orc_amr_regrid_record(void *h, int q, int *lev, double *time, int *tagged, int cap_t,
                          int *n_tagged, unsigned char *mask, long long cap_m, long long *n_mask,
                          int *new_boxes, int cap_n, int *n_new) {
    AmrBase *a = (AmrBase *)h;
    if (q < 0 || q >= a->nregrids()) return -1;
    const auto &r = a->record(q);
    *lev = r.lev;
    *time = r.time;
    auto put = [](const std::vector<shamr::IBox> &v, int *out, int cap, int *n) {
        *n = (int)v.size();
        if (!out) return;
        for (size_t k = 0; k < v.size() && (int)k < cap; ++k)
            for (int d = 0; d < 3; ++d) {
                out[6 * k + d] = v[k].lo[d];
                out[6 * k + 3 + d] = v[k].hi[d];
            }
    };
    put(r.boxes_tagged_level, tagged, cap_t, n_tagged);
    put(r.new_boxes, new_boxes, cap_n, n_new);
    *n_mask = (long long)r.mask.size();
    if (mask && (long long)r.mask.size() <= cap_m) std::copy(r.mask.begin(), r.mask.end(), mask);
    return 0;
}

} /* extern "C" */

/* Projection::Compute over the levels 0..min(max_level, finest) of the
 * hierarchy (grid_new), orc::projection. */
extern "C" int orc_amr_projection(void *h, int fn, int comp, int mode, int max_level,
                                  double *data, int *nproj) {
    AmrBase *a = (AmrBase *)h;
    const int ml = std::min(max_level, a->finest());
    std::vector<const MF *> lv;
    for (int l = 0; l <= ml; ++l) lv.push_back(a->level(l, 0));
    std::vector<double> d;
    std::vector<int> n;
    orc::projection(lv, fn, comp, mode, d, n);
    std::copy(d.begin(), d.end(), data);
    std::copy(n.begin(), n.end(), nproj);
    return 0;
}
