/* ORACLE (test infrastructure only).
 *
 * extern "C" entry points of the oracle, shared by liboracle.so (the CPU
 * restatement, oracle_capi.cpp) and oracle/_ref/libshref.so (the same
 * drivers around the reference's own per-cell headers, ref_harness.cpp).
 * The including file defines ORC_PROJECTS(X) as a list X(id, Policy) and
 * the symbol prefix ORC_API(name).
 *
 * Host array layout ("canonical layout") used by every entry point: for a
 * cubic periodic level of N^3 cells, component-major, then z, y, x with x
 * fastest: a[((n*N + k)*N + j)*N + i].
 *
 * Return codes: 0 ok, -1 bad argument, -2 project not available, -3
 * internal error.
 */
#ifndef SH_ORACLE_CAPI_BODY_H_
#define SH_ORACLE_CAPI_BODY_H_

#include "oracle_core.h"

#include <memory>

namespace orc {
namespace capi {

template <class T>
struct TypeTag {
    using type = T;
};

template <class F>
inline int with_project(int id, F &&f) {
#define ORC_CASE(ID, P)                                                        \
    case ID:                                                                   \
        f(TypeTag<P>());                                                       \
        return 0;
    switch (id) {
        ORC_PROJECTS(ORC_CASE)
    default:
        return -2;
    }
#undef ORC_CASE
}

/* Boxes of size max_grid tiling [0,N)^3 (max_grid <= 0: one box). */
inline std::vector<Box> chop(int N, int max_grid) {
    if (max_grid <= 0 || max_grid >= N) return {Box{{0, 0, 0}, {N - 1, N - 1, N - 1}}};
    std::vector<Box> r;
    for (int z = 0; z < N; z += max_grid)
        for (int y = 0; y < N; y += max_grid)
            for (int x = 0; x < N; x += max_grid)
                r.push_back(Box{{x, y, z},
                                {std::min(x + max_grid, N) - 1, std::min(y + max_grid, N) - 1,
                                 std::min(z + max_grid, N) - 1}});
    return r;
}

inline void scatter(MF &mf, const double *host, int N, int ncomp) {
    for (Fab &f : mf.fabs) {
        auto a = f.a();
        for (int n = 0; n < ncomp; ++n)
            for_cells(f.vbox, [&](int i, int j, int k) {
                a(i, j, k, n) = host[(((size_t)n * N + k) * N + j) * N + i];
            });
    }
}
inline void gather(const MF &mf, double *host, int N, int ncomp) {
    for (const Fab &f : mf.fabs) {
        auto a = f.ca();
        for (int n = 0; n < ncomp; ++n)
            for_cells(f.vbox, [&](int i, int j, int k) {
                host[(((size_t)n * N + k) * N + j) * N + i] = a(i, j, k, n);
            });
    }
}

inline RknTableau tableau_from_flat(const double *flat, int s) {
    /* flat = nodes[s], bbar[s], b[s], lower triangle incl. diagonal */
    RknTableau t;
    t.nodes.assign(flat, flat + s);
    t.bbar.assign(flat + s, flat + 2 * s);
    t.b.assign(flat + 2 * s, flat + 3 * s);
    const double *tri = flat + 3 * s;
    for (int i = 0; i < s; ++i) {
        std::vector<double> row(tri, tri + i + 1);
        tri += i + 1;
        t.a.push_back(row);
    }
    return t;
}

} // namespace capi
} // namespace orc

extern "C" {

/* Evolves a cubic periodic single level of N^3 cells, split into boxes of
 * max_grid cells per side with nghost ghost cells, by nsteps steps of the
 * integrator `integrator` (10 SSPRK3, 11 leapfrog, 20 user RKN tableau,
 * 21 RKN4, 22 RKN5).  `init_new` (may be NULL) is the content of the second
 * time level before the first step, which the leapfrog's second force
 * evaluation reads as momenta. */
int ORC_API(evolve_periodic)(int project, int integrator, const double *tableau_flat,
                             int nstages, int N, int max_grid, int nghost, int ncomp,
                             int with_gw, const double *state_in, const double *init_new,
                             double *state_out, double t0, double dt, double dx, int nsteps,
                             const double *params, int nparams, const double *gw_params,
                             int ngw, int ko_order, const double *ko_strength) {
    using namespace orc;
    if (N <= 0 || ncomp <= 0 || nghost < 0 || nsteps < 0 || !state_in || !state_out) return -1;
    try {
        return capi::with_project(project, [&](auto tag) {
            using P = typename decltype(tag)::type;
            IntegratorSpec spec;
            spec.type = integrator;
            if (integrator == RknButcherTableau) spec.user = capi::tableau_from_flat(tableau_flat, nstages);
            Box dom{{0, 0, 0}, {N - 1, N - 1, N - 1}};
            auto boxes = capi::chop(N, max_grid);
            MF grid_new, grid_old;
            grid_new.define(dom, boxes, ncomp, nghost, t0);
            grid_old.define(dom, boxes, ncomp, nghost);
            capi::scatter(grid_new, state_in, N, ncomp);
            if (init_new) capi::scatter(grid_old, init_new, N, ncomp);
            std::vector<double> ko(ncomp, 0.0);
            if (ko_strength) ko.assign(ko_strength, ko_strength + ncomp);
            RhsConfig c;
            c.lev = 0; c.dt = dt; c.dx = dx; c.params = params; c.gw_params = gw_params;
            c.with_gw = with_gw != 0; c.ko_order = ko_order; c.ko_strength = ko.data();
            for (int s = 0; s < nsteps; ++s)
                advance_single_level<P>(spec, grid_old, grid_new, dt, c, with_gw != 0,
                                        ncomp - (with_gw ? 12 : 0));
            capi::gather(grid_new, state_out, N, ncomp);
        });
    } catch (...) {
        return -3;
    }
}

/* rhs = f(state) on a periodic N^3 level (ghosts filled periodically). */
int ORC_API(fill_rhs)(int project, int N, int nghost, int ncomp, int with_gw,
                      const double *state_in, double *rhs_out, double time, int lev, double dt,
                      double dx, const double *params, const double *gw_params, int ko_order,
                      const double *ko_strength) {
    using namespace orc;
    if (N <= 0 || ncomp <= 0 || !state_in || !rhs_out) return -1;
    try {
        return capi::with_project(project, [&](auto tag) {
            using P = typename decltype(tag)::type;
            Box dom{{0, 0, 0}, {N - 1, N - 1, N - 1}};
            auto boxes = capi::chop(N, 0);
            MF st, rhs;
            st.define(dom, boxes, ncomp, nghost);
            rhs.define(dom, boxes, ncomp, nghost);
            capi::scatter(st, state_in, N, ncomp);
            capi::scatter(rhs, rhs_out, N, ncomp); /* FillRhs leaves unwritten comps */
            fill_boundary_periodic(st);
            std::vector<double> ko(ncomp, 0.0);
            if (ko_strength) ko.assign(ko_strength, ko_strength + ncomp);
            RhsConfig c;
            c.lev = lev; c.dt = dt; c.dx = dx; c.params = params; c.gw_params = gw_params;
            c.with_gw = with_gw != 0; c.ko_order = ko_order; c.ko_strength = ko.data();
            fill_rhs<P>(rhs, st, time, c);
            capi::gather(rhs, rhs_out, N, ncomp);
        });
    } catch (...) {
        return -3;
    }
}

/* Average-down with truncation error on a periodic level pair: fine is
 * (2Nc)^3, crse Nc^3 (in/out); te (2Nc)^3 receives |crse - avg| at even
 * fine cells, other cells keep their input values. */
int ORC_API(avgdown_te)(int ncomp, int Nc, const double *fine, double *crse, double *te) {
    using namespace orc;
    if (Nc <= 0 || ncomp <= 0 || !fine || !crse || !te) return -1;
    const int Nf = 2 * Nc;
    MF F, C, T;
    F.define(Box{{0, 0, 0}, {Nf - 1, Nf - 1, Nf - 1}}, capi::chop(Nf, 0), ncomp, 0);
    T.define(F.domain, F.boxes(), ncomp, 0);
    C.define(Box{{0, 0, 0}, {Nc - 1, Nc - 1, Nc - 1}}, capi::chop(Nc, 0), ncomp, 0);
    capi::scatter(F, fine, Nf, ncomp);
    capi::scatter(C, crse, Nc, ncomp);
    capi::scatter(T, te, Nf, ncomp);
    average_down_with_te(F, C, T, ncomp);
    capi::gather(C, crse, Nc, ncomp);
    capi::gather(T, te, Nf, ncomp);
    return 0;
}

/* Plain 2x2x2 average-down, fine (2Nc)^3 -> crse Nc^3. */
int ORC_API(average_down)(int ncomp, int Nc, const double *fine, double *crse) {
    using namespace orc;
    if (Nc <= 0 || ncomp <= 0 || !fine || !crse) return -1;
    const int Nf = 2 * Nc;
    MF F, C;
    F.define(Box{{0, 0, 0}, {Nf - 1, Nf - 1, Nf - 1}}, capi::chop(Nf, 0), ncomp, 0);
    C.define(Box{{0, 0, 0}, {Nc - 1, Nc - 1, Nc - 1}}, capi::chop(Nc, 0), ncomp, 0);
    capi::scatter(F, fine, Nf, ncomp);
    average_down(F, C, ncomp);
    capi::gather(C, crse, Nc, ncomp);
    return 0;
}

/* Tag mask (CPU semantics) of a periodic N^3 level split into boxes of
 * max_grid.  te may be NULL (no truncation-error tags).  mask_out holds N^3
 * bytes in canonical layout; counts_out[0] = total, [1] = user, [2..] per
 * component truncation-error tags (ncomp entries). */
int ORC_API(tag)(int project, int N, int max_grid, int ncomp, const double *state,
                 const double *te, double time, int lev, double dt, double dx,
                 const double *te_crit, const double *params_tag, const double *params_mod,
                 unsigned char *mask_out, long *counts_out) {
    using namespace orc;
    if (N <= 0 || ncomp <= 0 || !state || !mask_out) return -1;
    try {
        return capi::with_project(project, [&](auto tag) {
            using P = typename decltype(tag)::type;
            Box dom{{0, 0, 0}, {N - 1, N - 1, N - 1}};
            auto boxes = capi::chop(N, max_grid);
            MF st, T;
            st.define(dom, boxes, ncomp, 1);
            capi::scatter(st, state, N, ncomp);
            fill_boundary_periodic(st);
            if (te) {
                T.define(dom, boxes, ncomp, 1);
                capi::scatter(T, te, N, ncomp);
            }
            std::vector<std::vector<uint8_t>> mask;
            long tot = 0, usr = 0;
            std::vector<long> trunc(ncomp, 0);
            tag_cpu_literal<P>(st, te ? &T : nullptr, time, lev, dt, dx, te_crit, ncomp, params_tag,
                               params_mod, mask, &tot, &usr, trunc.data());
            for (size_t b = 0; b < boxes.size(); ++b) {
                const Box &vb = boxes[b];
                size_t q = 0;
                for_cells(vb, [&](int i, int j, int k) {
                    mask_out[((size_t)k * N + j) * N + i] = mask[b][q++];
                });
            }
            if (counts_out) {
                counts_out[0] = tot;
                counts_out[1] = usr;
                for (int n = 0; n < ncomp; ++n) counts_out[2 + n] = trunc[n];
            }
        });
    } catch (...) {
        return -3;
    }
}

/* GW spectrum of six N^3 components (comps: 6 consecutive canonical
 * arrays).  bins_out needs room for max_bins; *nbins receives the count and
 * ks_out (may be NULL) the k^2 of every bin. */
int ORC_API(gw_spectrum)(const double *comps, int N, int zero_padding, int projection_type,
                         int unbinned, double *bins_out, long long *ks_out, int max_bins,
                         int *nbins) {
    using namespace orc;
    if (N <= 0 || zero_padding <= 0 || !comps || !bins_out || !nbins) return -1;
    std::vector<const double *> c6(6);
    for (int q = 0; q < 6; ++q) c6[q] = comps + (size_t)q * N * N * N;
    std::vector<long long> ks;
    std::vector<double> s = gw_spectrum(c6, N, zero_padding, projection_type, unbinned != 0, ks);
    *nbins = (int)s.size();
    if ((int)s.size() > max_bins) return -1;
    std::copy(s.begin(), s.end(), bins_out);
    if (ks_out) std::copy(ks.begin(), ks.end(), ks_out);
    return 0;
}

int ORC_API(unique_k2)(int dim, long long *out, int max_n, int *n) {
    auto v = orc::unique_k2(dim);
    *n = (int)v.size();
    if ((int)v.size() > max_n) return -1;
    std::copy(v.begin(), v.end(), out);
    return 0;
}

int ORC_API(index_to_k)(int N, int projection_type, double *out) {
    auto v = orc::index_to_k(N, projection_type);
    std::copy(v.begin(), v.end(), out);
    return 0;
}

/* The TT projector contraction weights Lambda_ijlm of every k-cell of a
 * P^3 R2C grid ((P/2+1) x P x P cells, a fastest), 81 per cell in (i, j, l,
 * m) order, with the k-map of projection_type (the oracle's gw_lambda). */
int ORC_API(gw_lambda_table)(int P, int projection_type, double *out) {
    auto itk = orc::index_to_k(P, projection_type);
    const int H = P / 2 + 1;
    size_t q = 0;
    for (int c = 0; c < P; ++c)
        for (int b = 0; b < P; ++b)
            for (int a = 0; a < H; ++a) {
                int abc[3] = {a, b, c};
                for (int i = 0; i < 3; ++i)
                    for (int j = 0; j < 3; ++j)
                        for (int l = 0; l < 3; ++l)
                            for (int m = 0; m < 3; ++m)
                                out[q++] = orc::gw_lambda(i, j, l, m, abc, itk.data());
            }
    return 0;
}

} /* extern "C" */

#endif // SH_ORACLE_CAPI_BODY_H_
