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
 * ComputeSpectrum). */
#include <chrono>
#include <cmath>
#include <cstring>
#include <deque>
#include <map>
#include <new>
#include <stdexcept>
#include <string>
#include <vector>

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
};

} // namespace

struct sh_server {
    sh_ctx *ctx = nullptr;
    sh_ensemble *pool = nullptr;
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
    int rc = sh_ensemble_gw_spectrum(S->pool, q.slot, q.spec.zero_padding,
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

} // namespace

extern "C" {

int sh_server_create(sh_ctx *ctx, int precision, long long capacity_cells, sh_server **out) {
    if (!ctx || !out) return SH_ERR_ARG;
    *out = nullptr;
    sh_server *S = new (std::nothrow) sh_server();
    if (!S) return SH_ERR_NOMEM;
    S->ctx = ctx;
    int rc = sh_ensemble_create_pool(ctx, SH_FAMILY_FOPT_GW, precision, capacity_cells, &S->pool);
    if (rc != SH_OK) {
        delete S;
        return rc;
    }
    *out = S;
    return SH_OK;
}

int sh_server_destroy(sh_server *S) {
    if (!S) return SH_ERR_ARG;
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
        (r->N * r->zero_padding) % 2 != 0)
        return SH_ERR_ARG;
    long long pool_cap = 0;
    sh_ensemble_pool_info(S->pool, &pool_cap, nullptr, nullptr, nullptr);
    if ((long long)r->N * r->N * r->N > pool_cap) {
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
        int rc = sh_ensemble_admit(S->pool, q.spec.N, q.spec.dx, q.spec.params, q.spec.dt, &slot);
        if (rc == SH_ERR_NOMEM) {
            if (is_head) {
                head_blocked = true;
                S->head_waited++;
            }
            ++it;
            continue;
        }
        if (is_head) S->head_waited = 0;
        if (rc == SH_OK && q.spec.nbubbles > 0)
            rc = sh_ensemble_add_bubbles(S->pool, slot, q.spec.nbubbles, q.xyz.data(),
                                         q.profile.data(), q.spec.nbins, q.spec.inv_dx,
                                         q.spec.Lcut);
        if (rc != SH_OK) {
            S->err = sh_ensemble_last_error(S->pool);
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
    /* one step of every running request, each with its own dt */
    if (!S->running.empty()) {
        int rc = sh_ensemble_step(S->pool, 0., 1);
        if (rc != SH_OK) {
            S->err = sh_ensemble_last_error(S->pool);
            return rc;
        }
        S->iterations++;
        std::vector<long long> still;
        for (long long id : S->running) {
            Req &q = S->reqs.at(id);
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
