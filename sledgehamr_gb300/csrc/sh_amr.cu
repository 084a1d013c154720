/* AMR hierarchy on the GPU (sh_amr_* of include/sledgehamr_gb300.h): the
 * host time stepper of sh_amr_driver.h over levels held by this library. */
#include <cfloat>
#include <cstring>
#include <memory>
#include <new>
#include <string>
#include <vector>

#include "sh_amr_driver.h"
#include "sh_checkpoint.h"
#include "sh_internal.h"
#include "sledgehamr_gb300.h"

namespace {

/* Level handle of the driver: the library level plus link bookkeeping, so
 * that a fine level's coarse-fine plan is rebuilt whenever either level was
 * re-created. */
struct GpuLevel {
    sh_level *L = nullptr;
    long long gen = 0;
    const GpuLevel *linked = nullptr;
    long long linked_gen = -1;
};

struct ShFail : std::runtime_error {
    int code;
    ShFail(int c, const std::string &m) : std::runtime_error(m), code(c) {}
};

struct GpuBackend {
    using Level = GpuLevel *;
    sh_ctx *ctx;
    sh_amr_config cfg;
    int ncomp = 0;
    long long next_gen = 1;

    void ok(int rc, const char *what) {
        if (rc != SH_OK)
            throw ShFail(rc, std::string(what) + ": " + sh_ctx_last_error(ctx));
    }

    Level create(int lev, const std::vector<shamr::IBox> &boxes, int N) {
        std::vector<sh_box> bx(boxes.size());
        for (size_t q = 0; q < boxes.size(); ++q)
            for (int d = 0; d < 3; ++d) {
                bx[q].lo[d] = boxes[q].lo[d];
                bx[q].hi[d] = boxes[q].hi[d];
            }
        const int lo[3] = {0, 0, 0}, hi[3] = {N - 1, N - 1, N - 1};
        GpuLevel *g = new GpuLevel();
        ok(sh_level_create_prec(ctx, cfg.project, cfg.with_gw, lo, hi, bx.data(),
                                (int)bx.size(), cfg.nghost, cfg.precision, &g->L),
           "sh_level_create");
        sh_level_set_index(g->L, lev);
        g->gen = next_gen++;
        return g;
    }
    void destroy(Level &l) {
        if (l) {
            sh_level_destroy(ctx, l->L);
            delete l;
        }
        l = nullptr;
    }
    double time(const Level &l, int which) {
        double t;
        sh_level_time(l->L, which, &t, nullptr);
        return t;
    }
    int istep(const Level &l, int which) {
        int s;
        sh_level_time(l->L, which, nullptr, &s);
        return s;
    }
    void set_time(Level &l, int which, double t, int s) { sh_level_set_time(l->L, which, t, s); }
    void link(Level f, const Level c) {
        if (!c) {
            if (f->linked) ok(sh_level_set_coarse(ctx, f->L, nullptr), "unlink");
            f->linked = nullptr;
            f->linked_gen = -1;
            return;
        }
        if (f->linked == c && f->linked_gen == c->gen) return;
        ok(sh_level_set_coarse(ctx, f->L, c->L), "sh_level_set_coarse");
        f->linked = c;
        f->linked_gen = c->gen;
    }
    void advance(int lev, Level &l, Level *coarse, double dt, double dx, bool no_swap) {
        link(l, coarse ? *coarse : nullptr);
        ok(sh_level_advance(ctx, l->L, cfg.integrator, nullptr, 0, dt, dx, cfg.params,
                            cfg.nparams, cfg.gw_params, cfg.ngw, 0, nullptr,
                            no_swap ? SH_ADVANCE_NO_SWAP : 0),
           "sh_level_advance");
    }
    void average_down(Level &f, int wf, Level &c, int wc) {
        ok(sh_average_down(ctx, f->L, wf, c->L, wc), "sh_average_down");
    }
    void average_down_te(Level &f, Level &c) {
        ok(sh_average_down_te(ctx, f->L, c->L), "sh_average_down_te");
    }
    std::vector<uint8_t> tag(Level &l, bool use_te, double time, int lev, double dt, double dx) {
        int nc = 0, nb = 0;
        long long nv = 0;
        sh_level_info(l->L, &nc, &nb, &nv);
        std::vector<uint8_t> mask((size_t)nv);
        ok(sh_tag(ctx, l->L, use_te ? 1 : 0, time, lev, dt, dx, cfg.te_crit, cfg.params_tag,
                  cfg.nparams_tag, cfg.params_mod, cfg.nparams_mod, mask.data(), nullptr,
                  nullptr, 0, nullptr),
           "sh_tag");
        return mask;
    }
    std::vector<uint8_t> tag_blocks(Level &l, bool use_te, double time, int lev, double dt,
                                    double dx, int block, int buffer, int nb) {
        std::vector<uint8_t> blk((size_t)nb * nb * nb);
        ok(sh_tag_blocks(ctx, l->L, use_te ? 1 : 0, time, lev, dt, dx, cfg.te_crit,
                         cfg.params_tag, cfg.nparams_tag, cfg.params_mod, cfg.nparams_mod, block,
                         buffer, blk.data(), nullptr),
           "sh_tag_blocks");
        return blk;
    }
    void fill_from_coarse(Level &f, Level &c, double time) {
        ok(sh_level_fill_from(ctx, f->L, SH_NEW, nullptr, SH_NEW, c->L, time), "fill from coarse");
    }
    void remake(Level &fresh, Level &old, Level &c, double time) {
        ok(sh_level_fill_from(ctx, fresh->L, SH_NEW, old->L, SH_NEW, c->L, time), "remake");
    }
    void extend(Level &fresh, Level &old, Level &c, double t_new, double t_old) {
        ok(sh_level_fill_from(ctx, fresh->L, SH_NEW, old->L, SH_NEW, c->L, t_new), "extend");
        ok(sh_level_fill_from(ctx, fresh->L, SH_OLD, old->L, SH_OLD, c->L, t_old), "extend");
    }
    void refresh_ghosts(Level &l, int which, Level *coarse) {
        link(l, coarse ? *coarse : nullptr);
        ok(sh_level_fill_patch(ctx, l->L, which), "sh_level_fill_patch");
    }
    void sync() { ok(sh_ctx_synchronize(ctx), "sh_ctx_synchronize"); }
    std::vector<double> read_valid(Level &l, int which) {
        int nc = 0, nb = 0;
        long long nv = 0;
        sh_level_info(l->L, &nc, &nb, &nv);
        std::vector<double> v((size_t)nv * nc);
        ok(sh_level_read(ctx, l->L, which, 1, v.data()), "sh_level_read");
        return v;
    }
    void write_valid(Level &l, int which, const std::vector<double> &v) {
        int nc = 0, nb = 0;
        long long nv = 0;
        sh_level_info(l->L, &nc, &nb, &nv);
        if ((long long)v.size() != nv * nc)
            throw ShFail(SH_ERR_ARG, "checkpoint data does not match the level's boxes");
        ok(sh_level_write(ctx, l->L, which, 1, v.data()), "sh_level_write");
    }
    /* params_mod = per-component max |value| of level 0's new data, once
     * per time */
    double maxima_time = -DBL_MAX;
    void params_mod_from_norm0(Level &l0, double time) {
        if (time == maxima_time) return;
        for (int c = 0; c < ncomp; ++c)
            ok(sh_level_reduce(ctx, l0->L, SH_NEW, SH_REDUCE_MAX_ABS, c, &cfg.params_mod[c]),
               "sh_level_reduce");
        cfg.nparams_mod = ncomp;
        maxima_time = time;
    }
};

} // namespace

struct sh_amr {
    GpuBackend backend;
    std::unique_ptr<shamr::Driver<GpuBackend>> driver;
    std::string err;
};

namespace {
shamr::Config driver_config(const sh_amr_config &c, int ncomp) {
    shamr::Config d;
    d.N0 = c.N0;
    d.L = c.L;
    d.cfl = c.cfl;
    d.t_start = c.t_start;
    d.nghost = c.nghost;
    d.max_level = c.max_level;
    d.blocking_factor = c.blocking_factor;
    d.max_grid_size = c.max_grid_size;
    d.n_error_buf = c.n_error_buf;
    d.regrid_dt = c.regrid_dt;
    d.string_width_threshold = c.string_width_threshold;
    d.string_lambda = c.string_lambda;
    d.te_crit.assign(c.te_crit, c.te_crit + ncomp);
    d.clustering = c.clustering;
    d.grid_eff = c.grid_eff;
    d.params_mod_norm0 = c.params_mod_norm0 != 0;
    d.max_local_regrids = c.max_local_regrids;
    d.volume_threshold_strong = c.volume_threshold_strong;
    d.volume_threshold_weak = c.volume_threshold_weak;
    return d;
}

template <class F>
int amr_guard(sh_ctx *ctx, F &&f) {
    try {
        f();
        return SH_OK;
    } catch (const ShFail &e) {
        sh::set_ctx_error(ctx, e.what());
        return e.code;
    } catch (const std::bad_alloc &) {
        sh::set_ctx_error(ctx, "host allocation failed");
        return SH_ERR_NOMEM;
    } catch (const std::exception &e) {
        sh::set_ctx_error(ctx, e.what());
        return SH_ERR_ARG;
    }
}
} // namespace

extern "C" {

int sh_amr_config_defaults(sh_amr_config *c) {
    if (!c) return SH_ERR_ARG;
    std::memset(c, 0, sizeof(*c));
    c->integrator = SH_INTEGRATOR_RKN4;
    c->nghost = 2;
    c->N0 = 64;
    c->max_level = 2;
    c->blocking_factor = 8;
    c->max_grid_size = 32;
    c->n_error_buf = 1;
    c->L = 16.;
    c->cfl = 0.25;
    c->t_start = 0.1;
    c->string_lambda = 1.;
    c->clustering = SH_CLUSTER_BR_WINDOWS;
    c->grid_eff = 0.7;
    for (int n = 0; n < 32; ++n) c->te_crit[n] = DBL_MAX;
    /* LocalRegrid's defaults (local_regrid.h:97-122) */
    c->max_local_regrids = 10;
    c->volume_threshold_strong = 1.05;
    c->volume_threshold_weak = 1.1;
    return SH_OK;
}

int sh_amr_create(sh_ctx *ctx, const sh_amr_config *cfg, const double *level0, sh_amr **out) {
    if (!ctx || !cfg || !out) return SH_ERR_ARG;
    *out = nullptr;
    int ncomp = 0;
    int rc = sh_project_ncomp(cfg->project, cfg->with_gw, &ncomp, nullptr);
    if (rc != SH_OK) return rc;
    if (cfg->nparams < 0 || cfg->nparams > 32 || cfg->ngw < 0 || cfg->ngw > 16)
        return SH_ERR_ARG;
    if (cfg->nparams_tag < 0 || cfg->nparams_tag > 32 || cfg->nparams_mod < 0 ||
        cfg->nparams_mod > 32)
        return SH_ERR_ARG;
    if ((cfg->clustering != SH_CLUSTER_BR && cfg->clustering != SH_CLUSTER_WINDOWS &&
         cfg->clustering != SH_CLUSTER_BR_WINDOWS) ||
        !(cfg->grid_eff > 0. && cfg->grid_eff <= 1.))
        return SH_ERR_ARG;
    sh_amr *a = new (std::nothrow) sh_amr();
    if (!a) return SH_ERR_NOMEM;
    a->backend.ctx = ctx;
    a->backend.cfg = *cfg;
    a->backend.ncomp = ncomp;
    rc = amr_guard(ctx, [&] {
        a->driver.reset(new shamr::Driver<GpuBackend>(a->backend, driver_config(*cfg, ncomp)));
        a->driver->record_regrids = cfg->record_regrids != 0;
        a->driver->init_coarse([&](GpuLevel *&l) {
            /* without level0 the new level keeps its zeroed buffers */
            if (level0)
                a->backend.ok(sh_level_write(ctx, l->L, SH_NEW, 0, level0), "sh_level_write");
        });
    });
    if (rc != SH_OK) {
        delete a;
        return rc;
    }
    *out = a;
    return SH_OK;
}

int sh_amr_set_tag_params(sh_amr *a, const double *params_tag, int nparams_tag,
                          const double *params_mod, int nparams_mod) {
    if (!a || nparams_tag < 0 || nparams_tag > 32 || nparams_mod < 0 || nparams_mod > 32 ||
        (nparams_tag > 0 && !params_tag) || (nparams_mod > 0 && !params_mod))
        return SH_ERR_ARG;
    sh_amr_config &c = a->backend.cfg;
    for (int q = 0; q < nparams_tag; ++q) c.params_tag[q] = params_tag[q];
    for (int q = 0; q < nparams_mod; ++q) c.params_mod[q] = params_mod[q];
    c.nparams_tag = nparams_tag;
    c.nparams_mod = nparams_mod;
    return SH_OK;
}

int sh_amr_destroy(sh_ctx *ctx, sh_amr *a) {
    if (!ctx || !a) return SH_ERR_ARG;
    delete a;
    return SH_OK;
}

int sh_amr_step(sh_ctx *ctx, sh_amr *a, int n) {
    if (!ctx || !a || n < 0) return SH_ERR_ARG;
    return amr_guard(ctx, [&] {
        for (int q = 0; q < n; ++q) {
            a->driver->step();
            if (!a->backend.cfg.check_finite) continue;
            for (int l = 0; l <= a->driver->finest; ++l) {
                long long bad = 0;
                const int rc = sh_level_check_finite(ctx, a->driver->levels[l]->L, SH_NEW, &bad);
                if (rc != SH_OK)
                    throw ShFail(rc, "level " + std::to_string(l) + ": " +
                                         sh_ctx_last_error(ctx));
            }
        }
    });
}

int sh_amr_info(const sh_amr *a, int *finest, long long *cell_updates, int *nregrids) {
    if (!a) return SH_ERR_ARG;
    if (finest) *finest = a->driver->finest;
    if (cell_updates) *cell_updates = a->driver->cell_updates;
    if (nregrids) *nregrids = (int)a->driver->regrids.size();
    return SH_OK;
}

int sh_amr_set_timer_sync(sh_amr *a, int on) {
    if (!a) return SH_ERR_ARG;
    a->driver->sync_timers = on != 0;
    return SH_OK;
}

int sh_amr_timer(const sh_amr *a, int q, const char **name, double *seconds, long long *calls) {
    if (!a || q < 0 || q >= shamr::Driver<GpuBackend>::kNTimers) return SH_ERR_ARG;
    const auto &t = a->driver->timers[q];
    if (name) *name = t.name;
    if (seconds) *seconds = t.sec;
    if (calls) *calls = t.calls;
    return SH_OK;
}

int sh_amr_checkpoint(sh_ctx *ctx, sh_amr *a, const char *folder) {
    if (!ctx || !a || !folder) return SH_ERR_ARG;
    return amr_guard(ctx, [&] {
        const shamr::Checkpoint k = a->driver->checkpoint();
        std::string err;
        if (!shamr::write_checkpoint(k, folder, &err)) throw ShFail(SH_ERR_ARG, err);
    });
}

int sh_amr_restart(sh_ctx *ctx, const sh_amr_config *cfg, const char *folder, sh_amr **out) {
    if (!ctx || !cfg || !folder || !out) return SH_ERR_ARG;
    *out = nullptr;
    shamr::Checkpoint k;
    std::string err;
    if (!shamr::read_checkpoint(folder, &k, &err)) {
        sh::set_ctx_error(ctx, err);
        return SH_ERR_ARG;
    }
    int ncomp = 0;
    int rc = sh_project_ncomp(cfg->project, cfg->with_gw, &ncomp, nullptr);
    if (rc != SH_OK) return rc;
    if (ncomp != k.ncomp) {
        sh::set_ctx_error(ctx, "checkpoint has " + std::to_string(k.ncomp) +
                                   " components, the project " + std::to_string(ncomp));
        return SH_ERR_ARG;
    }
    sh_amr *a = nullptr;
    rc = sh_amr_create(ctx, cfg, nullptr, &a);
    if (rc != SH_OK) return rc;
    rc = amr_guard(ctx, [&] { a->driver->restart(k); });
    if (rc != SH_OK) {
        delete a;
        return rc;
    }
    *out = a;
    return SH_OK;
}

int sh_amr_set_trace(sh_amr *a, int on) {
    if (!a) return SH_ERR_ARG;
    a->driver->record_trace = on != 0;
    return SH_OK;
}

int sh_amr_trace(const sh_amr *a, char *buf, long long cap, long long *len) {
    if (!a) return SH_ERR_ARG;
    std::string all;
    for (const std::string &e : a->driver->trace) all += e + "\n";
    if (len) *len = (long long)all.size();
    if (!buf) return SH_OK;
    if ((long long)all.size() + 1 > cap) return SH_ERR_ARG;
    std::memcpy(buf, all.c_str(), all.size() + 1);
    return SH_OK;
}

int sh_amr_level(const sh_amr *a, int lev, sh_level **level) {
    if (!a || !level || lev < 0 || lev > a->driver->finest) return SH_ERR_ARG;
    *level = a->driver->levels[lev]->L;
    return SH_OK;
}

int sh_amr_regrid_record(const sh_amr *a, int q, int *lev, double *time, sh_box *tagged_boxes,
                         int cap_tagged, int *n_tagged, uint8_t *mask, long long cap_mask,
                         long long *n_mask, sh_box *new_boxes, int cap_new, int *n_new) {
    if (!a || q < 0 || q >= (int)a->driver->regrids.size()) return SH_ERR_ARG;
    const shamr::RegridRecord &r = a->driver->regrids[q];
    if (lev) *lev = r.lev;
    if (time) *time = r.time;
    auto put = [](const std::vector<shamr::IBox> &src, sh_box *dst, int cap, int *n) {
        if (n) *n = (int)src.size();
        if (!dst) return true;
        if (cap < (int)src.size()) return false;
        for (size_t k = 0; k < src.size(); ++k)
            for (int d = 0; d < 3; ++d) {
                dst[k].lo[d] = src[k].lo[d];
                dst[k].hi[d] = src[k].hi[d];
            }
        return true;
    };
    if (!put(r.boxes_tagged_level, tagged_boxes, cap_tagged, n_tagged)) return SH_ERR_ARG;
    if (!put(r.new_boxes, new_boxes, cap_new, n_new)) return SH_ERR_ARG;
    if (n_mask) *n_mask = (long long)r.mask.size();
    if (mask) {
        if (cap_mask < (long long)r.mask.size()) return SH_ERR_ARG;
        std::memcpy(mask, r.mask.data(), r.mask.size());
    }
    return SH_OK;
}

} /* extern "C" */
