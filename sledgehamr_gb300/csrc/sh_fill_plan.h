/* Host-side planning of the ghost fills and level copies of
 * libsledgehamr_gb300.so, free of CUDA so that it can be compiled and
 * tested on its own: the owner map of a level (which box holds each block
 * of owner_res cells) and the fill plan of one level's ghost-grown boxes
 * from the valid cells of a source level (same-level ghost exchange with
 * periodic images, or level-to-level copies) and from a coarse level
 * (coarse-fine interpolation), as rectangles per destination box.
 *
 * Reference: LevelSynchronizer::FillPatch / FillIntermediatePatch /
 * FillCoarsePatch (source/level_synchronizer.cpp:56-214), whose AMReX
 * FillPatchSingleLevel / FillPatchTwoLevels / InterpFromCoarseLevel decide
 * the same split between copied and interpolated cells.
 */
#ifndef SH_FILL_PLAN_H_
#define SH_FILL_PLAN_H_

#include <algorithm>
#include <climits>
#include <stdexcept>
#include <string>
#include <vector>

#include "sledgehamr_gb300.h"

#ifdef _OPENMP
#include <omp.h>
#endif

namespace sh {

/* One rectangle of ghost cells copied from a valid region of a source level
 * (possibly through a periodic image): dst cells [lo, hi] of box dbox take
 * the values of cells [lo - shift, hi - shift] of box sbox. */
struct GhostCopyDev {
    int dbox, sbox;
    int lo[3], hi[3];
    int shift[3];
    long long first; /* running cell count (prefix sum) */
};

/* A rectangle [lo, hi] of cells of box dbox (ghost-grown) filled by
 * quadratic interpolation from the coarse level. */
struct CfRect {
    int dbox;
    int lo[3], hi[3];
    long long first; /* running cell count */
};

/* Fill plan of dst's ghost-grown boxes, built on the block grid of src:
 * every block region of a dst box takes the valid cells of its owner box in
 * src (periodic images included) and regions no src box owns are
 * interpolated from the coarse level (FillPatchTwoLevels /
 * InterpFromCoarseLevel).  With ghosts_only (src == dst: ghost fill) the
 * valid region of every dst box is skipped. */
struct FillPlan {
    std::vector<GhostCopyDev> rects;
    long long rect_cells = 0;
    std::vector<CfRect> cf;
    long long cf_cells = 0;
};

/* Invalid levels or layouts (overlapping boxes, a coarse level that does not
 * cover the cells to interpolate, mismatched domains). */
struct PlanError : std::runtime_error {
    using std::runtime_error::runtime_error;
};

inline void plan_require(bool c, const char *msg) {
    if (!c) throw PlanError(msg);
}

inline int floordiv(int a, int b) { return a >= 0 ? a / b : -((-a + b - 1) / b); }

/* Which box of a level holds each aligned block of res cells (-1: none);
 * res is the largest block size every box boundary and the domain are
 * aligned to. */
struct OwnerMap {
    std::vector<int> owner;
    int res = 1;
    int nb[3] = {1, 1, 1};
};

inline void build_owner_map(const int dlo[3], const int dhi[3], const sh_box *boxes, int nbox,
                            OwnerMap &m) {
    auto gcd = [](int a, int b) {
        a = a < 0 ? -a : a;
        b = b < 0 ? -b : b;
        while (b) {
            int r = a % b;
            a = b;
            b = r;
        }
        return a;
    };
    int res = 0;
    for (int d = 0; d < 3; ++d) res = gcd(res, dhi[d] - dlo[d] + 1);
    for (int q = 0; q < nbox; ++q)
        for (int d = 0; d < 3; ++d) {
            res = gcd(res, boxes[q].lo[d] - dlo[d]);
            res = gcd(res, boxes[q].hi[d] + 1 - dlo[d]);
        }
    if (res <= 0) res = 1;
    m.res = res;
    for (int d = 0; d < 3; ++d) m.nb[d] = (dhi[d] - dlo[d] + 1) / res;
    const long long nmap = (long long)m.nb[0] * m.nb[1] * m.nb[2];
    m.owner.resize((size_t)nmap);
    int *own = m.owner.data();
#pragma omp parallel for schedule(static)
    for (long long q = 0; q < nmap; ++q) own[q] = -1;
    /* boxes in parallel; overlapping boxes would leave fewer owned blocks
     * than the boxes hold, which the count below detects */
    long long want = 0;
#pragma omp parallel for schedule(dynamic, 64) reduction(+ : want)
    for (long long q = 0; q < nbox; ++q) {
        const sh_box &b = boxes[q];
        for (int z = (b.lo[2] - dlo[2]) / res; z <= (b.hi[2] - dlo[2]) / res; ++z)
            for (int y = (b.lo[1] - dlo[1]) / res; y <= (b.hi[1] - dlo[1]) / res; ++y)
                for (int x = (b.lo[0] - dlo[0]) / res; x <= (b.hi[0] - dlo[0]) / res; ++x) {
                    own[((size_t)z * m.nb[1] + y) * m.nb[0] + x] = (int)q;
                    ++want;
                }
    }
    long long have = 0;
#pragma omp parallel for schedule(static) reduction(+ : have)
    for (long long q = 0; q < nmap; ++q) have += own[q] >= 0;
    if (have != want) throw PlanError("boxes of a level overlap");
}

/* What a fill plan needs of a level. */
struct PlanLevel {
    int dlo[3], dhi[3];
    const sh_box *boxes;
    int nbox;
    int nghost;
    int ncomp;
    const int *owner;
    int owner_res;
    int owner_nb[3];
};

inline FillPlan build_fill_plan(const PlanLevel &D, const PlanLevel *S, const PlanLevel *C,
                                bool ghosts_only, bool want_copies = true) {
    FillPlan P;
    const int ext[3] = {D.dhi[0] - D.dlo[0] + 1, D.dhi[1] - D.dlo[1] + 1,
                        D.dhi[2] - D.dlo[2] + 1};
    if (S)
        for (int d = 0; d < 3; ++d)
            plan_require(S->dlo[d] == D.dlo[d] && S->dhi[d] == D.dhi[d],
                    "fill source has a different domain");
    if (C) {
        plan_require(C->ncomp == D.ncomp, "coarse level differs in components");
        plan_require(C->nghost >= 1, "coarse level needs at least one ghost cell");
        for (int d = 0; d < 3; ++d)
            plan_require(2 * (C->dhi[d] - C->dlo[d] + 1) == ext[d] && 2 * C->dlo[d] == D.dlo[d],
                    "coarse domain is not the fine domain coarsened by 2");
    }
    /* blocks: those of src, or (no src) those of dst */
    const PlanLevel &G = S ? *S : D;
    const int R = G.owner_res;
    const int g = D.nghost;
    /* per destination box: the blocks of its ghost-grown region, each with a
     * source (owner box and periodic shift), "interpolate" or "skip", then
     * runs of equal source along x merged along y and z */
    struct Blk {
        int kind; /* 0 skip, 1 copy, 2 interpolate */
        int own;
    };
    struct Run {
        int kind, own, sh[3], lo[3], hi[3];
    };
    const long long nbox = (long long)D.nbox;
    /* boxes are independent: host threads share them and append their
     * rectangles to buffers of their own; where each box's rectangles went
     * (thread, first, count) puts them back in box order afterwards, so the
     * plan is deterministic */
    struct Where {
        int thread;
        int nrect, ncf;
        size_t rect0, cf0;
    };
    std::vector<Where> where((size_t)nbox);
    std::vector<std::vector<GhostCopyDev>> thr_rects;
    std::vector<std::vector<CfRect>> thr_cf;
    bool uncovered = false;
#pragma omp parallel
    {
#ifdef _OPENMP
    const int tid = omp_get_thread_num();
#pragma omp single
    {
        thr_rects.resize(omp_get_num_threads());
        thr_cf.resize(omp_get_num_threads());
    }
#else
    const int tid = 0;
    thr_rects.resize(1);
    thr_cf.resize(1);
#endif
    std::vector<GhostCopyDev> &my_rects = thr_rects[tid];
    std::vector<CfRect> &my_cf = thr_cf[tid];
    std::vector<Blk> blk;
    std::vector<Run> runs, merged;
    std::vector<int> open_prev, open_cur; /* merged rectangle ending at the
                                             previous row / plane, by start */
    struct Axis {
        int lo, hi, wb, sh;
        bool inside;
    };
    std::vector<Axis> ax[3];
#pragma omp for schedule(dynamic, 16)
    for (long long b = 0; b < nbox; ++b) {
        int glo[3], ghi[3], blo[3], nbk[3];
        for (int d = 0; d < 3; ++d) {
            glo[d] = D.boxes[b].lo[d] - g;
            ghi[d] = D.boxes[b].hi[d] + g;
            blo[d] = floordiv(glo[d] - D.dlo[d], R);
            nbk[d] = floordiv(ghi[d] - D.dlo[d], R) - blo[d] + 1;
        }
        blk.assign((size_t)nbk[0] * nbk[1] * nbk[2], Blk{});
        /* per axis and block column: the cells it covers, its periodic
         * image in the source's block grid and whether it lies inside the
         * box's valid region (the block loop below only combines these) */
        for (int d = 0; d < 3; ++d) {
            ax[d].resize(nbk[d]);
            const int nbd = G.owner_nb[d];
            for (int t = 0; t < nbk[d]; ++t) {
                Axis &a = ax[d][t];
                const int bb = blo[d] + t;
                a.lo = std::max(glo[d], D.dlo[d] + bb * R);
                a.hi = std::min(ghi[d], D.dlo[d] + (bb + 1) * R - 1);
                a.wb = ((bb % nbd) + nbd) % nbd;
                a.sh = (bb - a.wb) * R; /* periodic image offset */
                a.inside = a.lo >= D.boxes[b].lo[d] && a.hi <= D.boxes[b].hi[d];
            }
        }
        /* the blocks, row by row: kind and source box (the periodic shift
         * of a block is that of its axis columns) */
        for (int z = 0; z < nbk[2]; ++z)
            for (int y = 0; y < nbk[1]; ++y) {
                const Axis &ay = ax[1][y], &az = ax[2][z];
                const bool inside_yz = ay.inside && az.inside;
                const bool unshifted_yz = ay.sh == 0 && az.sh == 0;
                const int *own_row =
                    S ? S->owner + ((size_t)az.wb * G.owner_nb[1] + ay.wb) * G.owner_nb[0]
                      : nullptr;
                Blk *row = blk.data() + ((size_t)z * nbk[1] + y) * nbk[0];
                for (int x = 0; x < nbk[0]; ++x) {
                    const Axis &axx = ax[0][x];
                    Blk &k = row[x];
                    k.kind = 0;
                    k.own = -1;
                    if (ghosts_only && inside_yz && axx.inside) continue;
                    const int own = own_row ? own_row[axx.wb] : -1;
                    if (own >= 0) {
                        if (S == &D && own == (int)b && unshifted_yz && axx.sh == 0) continue;
                        k.kind = 1;
                        k.own = own;
                        continue;
                    }
                    if (!C) continue; /* nothing to fill from: left as is */
                    k.kind = 2; /* parents checked per merged rectangle below */
                }
            }
        /* x-runs of equal kind / source */
        runs.clear();
        for (int z = 0; z < nbk[2]; ++z)
            for (int y = 0; y < nbk[1]; ++y) {
                const Axis &ay = ax[1][y], &az = ax[2][z];
                const Blk *row = blk.data() + ((size_t)z * nbk[1] + y) * nbk[0];
                int x = 0;
                while (x < nbk[0]) {
                    const Blk &k = row[x];
                    if (k.kind == 0) {
                        ++x;
                        continue;
                    }
                    int x1 = x;
                    while (x1 + 1 < nbk[0] && row[x1 + 1].kind == k.kind &&
                           row[x1 + 1].own == k.own && ax[0][x1 + 1].sh == ax[0][x].sh)
                        ++x1;
                    Run r{k.kind, k.own, {ax[0][x].sh, ay.sh, az.sh},
                          {ax[0][x].lo, ay.lo, az.lo}, {ax[0][x1].hi, ay.hi, az.hi}};
                    runs.push_back(r);
                    x = x1 + 1;
                }
            }
        /* merge along y, then along z (same kind and source, the same
         * extent along the other axes, adjacent along the merged one).  Runs
         * come in (z, y, x) order; a run can only join the rectangle that
         * starts at its first block and ends on the row (plane) before it -
         * two such rectangles would overlap - which open_prev holds by
         * start block; rectangles keep the order of their first run. */
        auto same_source = [](const Run &m, const Run &r) {
            return m.kind == r.kind && m.own == r.own && m.sh[0] == r.sh[0] &&
                   m.sh[1] == r.sh[1] && m.sh[2] == r.sh[2];
        };
        const int nx = nbk[0], nxy = nbk[0] * nbk[1];
        /* the block column of axis d that starts at cell lo */
        auto start_block = [&](int d, int lo) {
            return (int)(std::lower_bound(ax[d].begin(), ax[d].end(), lo,
                                          [](const Axis &a, int v) { return a.lo < v; }) -
                         ax[d].begin());
        };
        /* along y: rows of one plane */
        merged.clear();
        open_prev.assign(nx, -1);
        open_cur.assign(nx, -1);
        {
            int row_y = INT_MIN, row_z = INT_MIN;
            for (const Run &r : runs) {
                if (r.lo[2] != row_z) { /* a new plane: nothing open */
                    std::fill(open_prev.begin(), open_prev.end(), -1);
                    std::fill(open_cur.begin(), open_cur.end(), -1);
                    row_z = r.lo[2];
                    row_y = r.lo[1];
                } else if (r.lo[1] != row_y) { /* the next row */
                    open_prev.swap(open_cur);
                    std::fill(open_cur.begin(), open_cur.end(), -1);
                    row_y = r.lo[1];
                }
                const int x0 = start_block(0, r.lo[0]);
                const int c = open_prev[x0];
                if (c >= 0) {
                    Run &m = merged[c];
                    if (same_source(m, r) && m.hi[1] + 1 == r.lo[1] && m.hi[0] == r.hi[0]) {
                        m.hi[1] = r.hi[1];
                        open_cur[x0] = c;
                        continue;
                    }
                }
                open_cur[x0] = (int)merged.size();
                merged.push_back(r);
            }
        }
        runs.swap(merged);
        /* along z: rectangles in the order of their first plane */
        merged.clear();
        open_prev.assign(nxy, -1);
        open_cur.assign(nxy, -1);
        {
            int plane = INT_MIN;
            for (const Run &r : runs) {
                if (r.lo[2] != plane) {
                    open_prev.swap(open_cur);
                    std::fill(open_cur.begin(), open_cur.end(), -1);
                    plane = r.lo[2];
                }
                const int key = start_block(0, r.lo[0]) + nx * start_block(1, r.lo[1]);
                const int c = open_prev[key];
                if (c >= 0) {
                    Run &m = merged[c];
                    if (same_source(m, r) && m.hi[2] + 1 == r.lo[2] && m.hi[0] == r.hi[0] &&
                        m.lo[1] == r.lo[1] && m.hi[1] == r.hi[1]) {
                        m.hi[2] = r.hi[2];
                        open_cur[key] = c;
                        continue;
                    }
                }
                open_cur[key] = (int)merged.size();
                merged.push_back(r);
            }
        }
        runs.swap(merged);
        Where &w = where[(size_t)b];
        w.thread = tid;
        w.rect0 = my_rects.size();
        w.cf0 = my_cf.size();
        for (const Run &r : runs) {
            if (r.kind == 1) {
                if (!want_copies) continue;
                GhostCopyDev c;
                c.dbox = (int)b;
                c.sbox = r.own;
                for (int d = 0; d < 3; ++d) {
                    c.lo[d] = r.lo[d];
                    c.hi[d] = r.hi[d];
                    c.shift[d] = r.sh[d];
                }
                my_rects.push_back(c);
            } else {
                /* the parents of the region must lie on the coarse level
                 * (checked per coarse block) */
                const int Rc = C->owner_res;
                int pb0[3], pb1[3];
                for (int d = 0; d < 3; ++d) {
                    pb0[d] = floordiv(floordiv(r.lo[d], 2) - C->dlo[d], Rc);
                    pb1[d] = floordiv(floordiv(r.hi[d], 2) - C->dlo[d], Rc);
                }
                for (int pz = pb0[2]; pz <= pb1[2]; ++pz)
                    for (int py = pb0[1]; py <= pb1[1]; ++py)
                        for (int px = pb0[0]; px <= pb1[0]; ++px) {
                            const int p3[3] = {px, py, pz};
                            int cb[3];
                            for (int d = 0; d < 3; ++d) {
                                const int n = C->owner_nb[d];
                                cb[d] = ((p3[d] % n) + n) % n;
                            }
                            if (C->owner[((size_t)cb[2] * C->owner_nb[1] + cb[1]) *
                                             C->owner_nb[0] +
                                         cb[0]] < 0) {
#pragma omp atomic write
                                uncovered = true;
                            }
                        }
                CfRect c;
                c.dbox = (int)b;
                for (int d = 0; d < 3; ++d) {
                    c.lo[d] = r.lo[d];
                    c.hi[d] = r.hi[d];
                }
                my_cf.push_back(c);
            }
        }
        w.nrect = (int)(my_rects.size() - w.rect0);
        w.ncf = (int)(my_cf.size() - w.cf0);
    }
    } /* omp parallel */
    if (uncovered)
        throw PlanError("coarse level does not cover the cells to interpolate (levels "
                                  "are not properly nested)");
    auto cells = [](const int lo[3], const int hi[3]) {
        return (long long)(hi[0] - lo[0] + 1) * (hi[1] - lo[1] + 1) * (hi[2] - lo[2] + 1);
    };
    size_t nr = 0, nc = 0;
    for (const Where &w : where) {
        nr += w.nrect;
        nc += w.ncf;
    }
    P.rects.resize(nr);
    P.cf.resize(nc);
    nr = nc = 0;
    for (const Where &w : where) {
        std::copy_n(thr_rects[w.thread].begin() + w.rect0, w.nrect, P.rects.begin() + nr);
        std::copy_n(thr_cf[w.thread].begin() + w.cf0, w.ncf, P.cf.begin() + nc);
        nr += w.nrect;
        nc += w.ncf;
    }
    for (GhostCopyDev &c : P.rects) {
        c.first = P.rect_cells;
        P.rect_cells += cells(c.lo, c.hi);
    }
    for (CfRect &c : P.cf) {
        c.first = P.cf_cells;
        P.cf_cells += cells(c.lo, c.hi);
    }
    return P;
}

} // namespace sh

#endif // SH_FILL_PLAN_H_
