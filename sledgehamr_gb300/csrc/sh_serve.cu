/* Serving loop (sh_server_* of include/sledgehamr_gb300.h): requests for
 * first-order phase transition runs with GW spectra are admitted into one
 * pool (an ensemble whose members come and go) as soon as a free extent of
 * device memory holds them, every iteration advances all admitted runs by
 * one step of their own size in the same kernel launches, and a run that
 * reaches its end time has its GW spectrum computed and its memory
 * released.  Queued requests are scanned in arrival order and a request
 * that does not fit lets later, smaller ones pass, until the oldest has
 * waited kHeadPatience iterations; from then on nothing passes it.
 * There is no counterpart in the reference, which runs one simulation per
 * process; the per-run numerics are the FirstOrderPhaseTransition
 * equations of the ensemble path (leapfrog, 4th-order stencils, bubble
 * injection at t = 0, the GW spectrum of GravitationalWaves::
 * ComputeSpectrum).  Requests with refinement levels run as their own
 * AMR hierarchies (sh_amr with FirstOrderPhaseTransition + GW, the
 * leapfrog, truncation-error tags with the field maxima of level 0 as the
 * TruncationModifier parameters; FP32 + Kahan levels when the pool is FP32,
 * FP64 levels when it is FP64), each in a context of its own (its own
 * CUDA stream) stepped by a host thread of its own, so that their kernels
 * overlap with the pool's and with each other's; they are admitted while
 * the device has room for 16 times their level-0 state and fail (state 3)
 * if a later step runs out of memory. */
#include <atomic>
#include <cfloat>
#include <chrono>
#include <condition_variable>
#include <memory>
#include <mutex>
#include <thread>
#include <cmath>
#include <cstring>
#include <deque>
#include <map>
#include <new>
#include <stdexcept>
#include <string>
#include <vector>

#include <cuda_runtime.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "sledgehamr_gb300.h"

namespace {

constexpr int kHeadPatience = 64;

struct Req {
    sh_request spec;
    std::vector<double> xyz, profile;
    int state = 0; /* 0 queued, 1 running, 2 done, 3 failed */
    int slot = -1;
    long long steps_left = 0;
    double t_submit = 0, t_admit = 0, t_done = 0;
    std::vector<double> bins;
    std::vector<long long> ks;
    int rc = SH_OK;
    struct AmrJob *job = nullptr; /* AMR requests (owned by the server) */
    long long amr_cu = 0;         /* cell updates of the hierarchy counted so far */
};

/* An AMR request running in its own context and host thread. */
struct AmrJob {
    std::thread th;
    std::atomic<bool> done{false}, cancel{false};
    std::atomic<long long> cu{0}; /* cell updates so far */
    int rc = SH_OK;
    std::string err;
    std::vector<double> bins;
    std::vector<long long> ks;
    double t_done = 0;
};
constexpr int kAmrOmpThreads = 4; /* host threads of one hierarchy's regrids */

constexpr double kAmrMemoryFactor = 16.; /* admission: 16 x the level-0 state */
constexpr int kFoptComps = 14;           /* Phi, dPhi, 6 u, 6 du */

} // namespace

struct sh_server {
    sh_ctx *ctx = nullptr;
    int device = 0;
    std::vector<std::unique_ptr<AmrJob>> jobs;
    std::mutex mu;
    std::condition_variable cv; /* an AMR job finished */
    sh_ensemble *pool = nullptr;
    int precision = SH_PREC_FP64; /* of the pool; FP32 pools run FP32 + Kahan hierarchies */
    std::map<long long, Req> reqs;
    std::deque<long long> queue;
    std::vector<long long> running;
    long long next_id = 0, iterations = 0, cell_updates = 0;
    int head_waited = 0;
    std::chrono::steady_clock::time_point t0 = std::chrono::steady_clock::now();
    std::string err;
    double now() const {
        return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    }
};

namespace {

int finish(sh_server *S, long long id, Req &q) {
    const int P = q.spec.N * q.spec.zero_padding;
    const int cap = 3 * (P / 2 + 1) * (P / 2 + 1) + 16;
    q.bins.resize(cap);
    q.ks.resize(cap);
    int nb = 0;
    int rc;
    rc = sh_ensemble_gw_spectrum(S->pool, q.slot, q.spec.zero_padding,
                                 q.spec.projection_type, q.spec.unbinned, q.bins.data(),
                                 q.ks.data(), cap, &nb);
    if (rc == SH_OK) {
        q.bins.resize(nb);
        q.ks.resize(nb);
        q.state = 2;
    } else {
        q.state = 3;
        q.rc = rc;
        S->err = sh_ensemble_last_error(S->pool);
    }
    q.t_done = S->now();
    sh_ensemble_release(S->pool, q.slot);
    q.slot = -1;
    (void)id;
    return rc;
}

/* Steps an AMR request's hierarchy to its end time in its own context,
 * takes the spectrum of level 0 and frees everything (worker thread). */
void amr_worker(sh_server *S, AmrJob *job, sh_ctx *actx, sh_amr *amr, sh_request r,
                long long nsteps) {
#ifdef _OPENMP
    omp_set_num_threads(kAmrOmpThreads);
#endif
    int rc = SH_OK;
    for (long long s = 0; s < nsteps && rc == SH_OK && !job->cancel; ++s) {
        rc = sh_amr_step(actx, amr, 1);
        long long cu = 0;
        if (rc == SH_OK) rc = sh_amr_info(amr, nullptr, &cu, nullptr);
        if (rc == SH_OK) job->cu = cu;
    }
    if (rc == SH_OK && !job->cancel) {
        const int P = r.N * r.zero_padding;
        const int cap = 3 * (P / 2 + 1) * (P / 2 + 1) + 16;
        job->bins.resize(cap);
        job->ks.resize(cap);
        int nb = 0;
        sh_level *L0 = nullptr;
        rc = sh_amr_level(amr, 0, &L0);
        if (rc == SH_OK)
            rc = sh_gw_spectrum(actx, L0, nullptr, r.zero_padding, r.projection_type, r.unbinned,
                                job->bins.data(), job->ks.data(), cap, &nb);
        job->bins.resize(rc == SH_OK ? nb : 0);
        job->ks.resize(rc == SH_OK ? nb : 0);
    }
    if (rc != SH_OK) job->err = sh_ctx_last_error(actx);
    sh_amr_destroy(actx, amr);
    sh_ctx_destroy(actx);
    job->rc = job->cancel ? SH_ERR_ARG : rc;
    job->t_done = S->now();
    {
        std::lock_guard<std::mutex> lk(S->mu);
        job->done = true;
    }
    S->cv.notify_all();
}

/* An AMR request's hierarchy with its bubbles in a new context, handed to
 * a worker thread, if the device has room for kAmrMemoryFactor times its
 * level-0 state; SH_ERR_NOMEM otherwise. */
int admit_amr(sh_server *S, Req &q) {
    const sh_request &r = q.spec;
    size_t free_b = 0, total_b = 0;
    if (cudaSetDevice(S->device) != cudaSuccess ||
        cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) {
        S->err = "cudaMemGetInfo failed";
        return SH_ERR_CUDA;
    }
    const double need = kAmrMemoryFactor * (double)r.N * r.N * r.N * kFoptComps * sizeof(double);
    if ((double)free_b < need) return SH_ERR_NOMEM;
    int project = -1;
    int rc = sh_project_find("FirstOrderPhaseTransition", &project);
    if (rc != SH_OK) {
        S->err = "FirstOrderPhaseTransition is not compiled into the library";
        return rc;
    }
    sh_amr_config c;
    sh_amr_config_defaults(&c);
    c.project = project;
    c.with_gw = 1;
    c.integrator = 11; /* leapfrog */
    c.N0 = r.N;
    c.L = r.N * r.dx;
    c.cfl = r.dt / r.dx;
    c.t_start = 0.;
    c.nghost = 2;
    c.max_level = r.max_level;
    c.blocking_factor = r.blocking_factor > 0 ? r.blocking_factor : 8;
    c.max_grid_size = r.max_grid_size > 0 ? r.max_grid_size : 32;
    c.n_error_buf = 1;
    c.regrid_dt = r.regrid_dt;
    c.te_crit[0] = r.te_crit[0];
    c.te_crit[1] = r.te_crit[1];
    /* FirstOrderPhaseTransition params: [0] unused here, [1..3] q2 q3 q4 */
    c.params[0] = 0.;
    for (int k = 0; k < 3; ++k) c.params[1 + k] = r.params[k];
    for (int k = 4; k < 7; ++k) c.params[k] = 0.;
    c.nparams = 7;
    c.params_mod_norm0 = 1;
    /* the pool's precision form: FP32 (with or without compensation in the
     * pool) gives FP32 + Kahan levels */
    c.precision = S->precision == SH_PREC_FP64 ? SH_PREC_FP64 : SH_PREC_FP32_KAHAN;
    sh_ctx *actx = nullptr;
    rc = sh_ctx_create(S->device, &actx);
    if (rc != SH_OK) return rc;
    sh_amr *amr = nullptr;
    rc = sh_amr_create(actx, &c, nullptr, &amr);
    if (rc == SH_OK && r.nbubbles > 0) {
        sh_level *L0 = nullptr;
        rc = sh_amr_level(amr, 0, &L0);
        if (rc == SH_OK)
            rc = sh_level_add_bubbles(actx, L0, SH_NEW, 0, 1, r.nbubbles, q.xyz.data(),
                                      q.profile.data(), r.nbins, r.inv_dx, r.Lcut, r.dx);
    }
    if (rc != SH_OK) {
        S->err = sh_ctx_last_error(actx);
        if (amr) sh_amr_destroy(actx, amr);
        sh_ctx_destroy(actx);
        return rc;
    }
    S->jobs.emplace_back(new AmrJob());
    AmrJob *job = S->jobs.back().get();
    q.job = job;
    sh_request spec = r;
    spec.xyz = nullptr;
    spec.profile = nullptr;
    const long long nsteps = (long long)std::ceil(r.t_end / r.dt - 1e-9);
    job->th = std::thread(amr_worker, S, job, actx, amr, spec, nsteps);
    return SH_OK;
}

} // namespace

extern "C" {

int sh_server_create(sh_ctx *ctx, int precision, long long capacity_cells, sh_server **out) {
    if (!ctx || !out) return SH_ERR_ARG;
    *out = nullptr;
    sh_server *S = new (std::nothrow) sh_server();
    if (!S) return SH_ERR_NOMEM;
    S->ctx = ctx;
    S->precision = precision;
    int rc = sh_ensemble_create_pool(ctx, SH_FAMILY_FOPT_GW, precision, capacity_cells, &S->pool);
    if (rc != SH_OK) {
        delete S;
        return rc;
    }
    /* the pool's calls made the context's device current */
    if (cudaGetDevice(&S->device) != cudaSuccess) {
        sh_ensemble_destroy(S->pool);
        delete S;
        return SH_ERR_CUDA;
    }
    *out = S;
    return SH_OK;
}

int sh_server_destroy(sh_server *S) {
    if (!S) return SH_ERR_ARG;
    /* AMR requests still running stop after their current step */
    for (auto &j : S->jobs) j->cancel = true;
    for (auto &j : S->jobs)
        if (j->th.joinable()) j->th.join();
    S->jobs.clear();
    if (S->pool) sh_ensemble_destroy(S->pool);
    delete S;
    return SH_OK;
}

const char *sh_server_last_error(const sh_server *S) { return S ? S->err.c_str() : ""; }

int sh_server_submit(sh_server *S, const sh_request *r, long long *id) {
    if (!S || !r || !id) return SH_ERR_ARG;
    if (r->N < 8 || r->N > 4096 || !(r->dx > 0) || !(r->dt > 0) || !(r->t_end > 0) ||
        r->nbubbles < 0 || (r->nbubbles > 0 && (!r->xyz || !r->profile || r->nbins < 2)) ||
        r->zero_padding < 1 || r->projection_type < 1 || r->projection_type > 3 ||
        (r->N * r->zero_padding) % 2 != 0 || r->max_level < 0 || r->max_level > 8)
        return SH_ERR_ARG;
    long long pool_cap = 0;
    sh_ensemble_pool_info(S->pool, &pool_cap, nullptr, nullptr, nullptr);
    if (r->max_level == 0 && (long long)r->N * r->N * r->N > pool_cap) {
        S->err = "request larger than the pool";
        return SH_ERR_NOMEM;
    }
    Req q;
    q.spec = *r;
    if (r->nbubbles > 0) {
        q.xyz.assign(r->xyz, r->xyz + 3 * (size_t)r->nbubbles);
        q.profile.assign(r->profile, r->profile + 2 * (size_t)r->nbins);
    }
    q.spec.xyz = nullptr;
    q.spec.profile = nullptr;
    q.t_submit = S->now();
    *id = S->next_id++;
    S->reqs.emplace(*id, std::move(q));
    S->queue.push_back(*id);
    return SH_OK;
}

int sh_server_step(sh_server *S, int *running, int *queued, int *completed) {
    if (!S) return SH_ERR_ARG;
    int done_now = 0;
    /* admission */
    bool head_blocked = false;
    for (auto it = S->queue.begin(); it != S->queue.end();) {
        Req &q = S->reqs.at(*it);
        const bool is_head = it == S->queue.begin();
        if (!is_head && head_blocked && S->head_waited >= kHeadPatience) break;
        int slot = -1;
        int rc = q.spec.max_level > 0
                     ? admit_amr(S, q)
                     : sh_ensemble_admit(S->pool, q.spec.N, q.spec.dx, q.spec.params, q.spec.dt,
                                         &slot);
        if (rc == SH_ERR_NOMEM) {
            if (is_head) {
                head_blocked = true;
                S->head_waited++;
            }
            ++it;
            continue;
        }
        if (is_head) S->head_waited = 0;
        if (rc == SH_OK && q.spec.nbubbles > 0 && !q.job)
            rc = sh_ensemble_add_bubbles(S->pool, slot, q.spec.nbubbles, q.xyz.data(),
                                         q.profile.data(), q.spec.nbins, q.spec.inv_dx,
                                         q.spec.Lcut);
        if (rc != SH_OK) {
            /* admit_amr has set the message of an AMR request's failure */
            if (q.spec.max_level == 0) S->err = sh_ensemble_last_error(S->pool);
            q.state = 3;
            q.rc = rc;
            q.t_done = S->now();
            if (slot >= 0) sh_ensemble_release(S->pool, slot);
            it = S->queue.erase(it);
            continue;
        }
        q.state = 1;
        q.slot = slot;
        q.t_admit = S->now();
        q.steps_left = (long long)std::ceil(q.spec.t_end / q.spec.dt - 1e-9);
        S->running.push_back(*it);
        it = S->queue.erase(it);
    }
    /* one step of every running pool member, each with its own dt, in shared
     * launches; AMR hierarchies advance in their own threads and are
     * collected here when they finish */
    if (!S->running.empty()) {
        bool pool_members = false;
        for (long long id : S->running) pool_members = pool_members || !S->reqs.at(id).job;
        if (pool_members) {
            int rc = sh_ensemble_step(S->pool, 0., 1);
            if (rc != SH_OK) {
                S->err = sh_ensemble_last_error(S->pool);
                return rc;
            }
        } else {
            /* only AMR requests run: wait (bounded) for one to finish
             * instead of returning at once */
            std::unique_lock<std::mutex> lk(S->mu);
            S->cv.wait_for(lk, std::chrono::milliseconds(5), [&] {
                for (long long id : S->running)
                    if (S->reqs.at(id).job->done) return true;
                return false;
            });
        }
        S->iterations++;
        std::vector<long long> still;
        for (long long id : S->running) {
            Req &q = S->reqs.at(id);
            if (q.job) {
                AmrJob *job = q.job;
                const long long cu = job->cu;
                S->cell_updates += cu - q.amr_cu;
                q.amr_cu = cu;
                if (!job->done) {
                    still.push_back(id);
                    continue;
                }
                job->th.join();
                if (job->rc == SH_OK) {
                    q.bins.swap(job->bins);
                    q.ks.swap(job->ks);
                    q.state = 2;
                } else {
                    q.state = 3;
                    q.rc = job->rc;
                    S->err = job->err;
                }
                q.t_done = job->t_done;
                q.job = nullptr;
                for (auto it = S->jobs.begin(); it != S->jobs.end(); ++it)
                    if (it->get() == job) {
                        S->jobs.erase(it);
                        break;
                    }
                ++done_now;
                continue;
            }
            S->cell_updates += (long long)q.spec.N * q.spec.N * q.spec.N;
            if (--q.steps_left <= 0) {
                finish(S, id, q);
                ++done_now;
            } else {
                still.push_back(id);
            }
        }
        S->running.swap(still);
    }
    if (running) *running = (int)S->running.size();
    if (queued) *queued = (int)S->queue.size();
    if (completed) *completed = done_now;
    return SH_OK;
}

int sh_server_status(const sh_server *S, long long id, int *state, double *times) {
    if (!S || !state) return SH_ERR_ARG;
    auto it = S->reqs.find(id);
    if (it == S->reqs.end()) return SH_ERR_ARG;
    *state = it->second.state;
    if (times) {
        times[0] = it->second.t_submit;
        times[1] = it->second.t_admit;
        times[2] = it->second.t_done;
    }
    return SH_OK;
}

int sh_server_result(const sh_server *S, long long id, double *bins, long long *ks, int cap,
                     int *nbins) {
    if (!S || !nbins) return SH_ERR_ARG;
    auto it = S->reqs.find(id);
    if (it == S->reqs.end()) return SH_ERR_ARG;
    const Req &q = it->second;
    if (q.state == 3) return q.rc;
    if (q.state != 2) return SH_ERR_ARG;
    *nbins = (int)q.bins.size();
    if (bins) {
        if (cap < *nbins) return SH_ERR_ARG;
        std::memcpy(bins, q.bins.data(), q.bins.size() * sizeof(double));
        if (ks) std::memcpy(ks, q.ks.data(), q.ks.size() * sizeof(long long));
    }
    return SH_OK;
}

int sh_server_info(const sh_server *S, int *running, int *queued, long long *cell_updates,
                   long long *iterations, long long *free_cells) {
    if (!S) return SH_ERR_ARG;
    if (running) *running = (int)S->running.size();
    if (queued) *queued = (int)S->queue.size();
    if (cell_updates) *cell_updates = S->cell_updates;
    if (iterations) *iterations = S->iterations;
    if (free_cells) sh_ensemble_pool_info(S->pool, nullptr, free_cells, nullptr, nullptr);
    return SH_OK;
}

} /* extern "C" */
