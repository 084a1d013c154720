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
#include <stdexcept>
#include <string>
#include <vector>

#include "sledgehamr_gb300.h"

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
        int sh[3];
        int lo[3], hi[3];
    };
    struct Run {
        int kind, own, sh[3], lo[3], hi[3];
    };
    const long long nbox = (long long)D.nbox;
    std::vector<std::vector<GhostCopyDev>> box_rects(nbox);
    std::vector<std::vector<CfRect>> box_cf(nbox);
    bool uncovered = false;
    /* boxes are independent: host threads share them, results are
     * concatenated in box order afterwards (the plan is deterministic) */
#pragma omp parallel
    {
    std::vector<Blk> blk;
    std::vector<Run> runs, merged;
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
        for (int z = 0; z < nbk[2]; ++z)
            for (int y = 0; y < nbk[1]; ++y)
                for (int x = 0; x < nbk[0]; ++x) {
                    Blk &k = blk[((size_t)z * nbk[1] + y) * nbk[0] + x];
                    const Axis *axk[3] = {&ax[0][x], &ax[1][y], &ax[2][z]};
                    int wb[3];
                    bool inside_valid = true;
                    for (int d = 0; d < 3; ++d) {
                        k.lo[d] = axk[d]->lo;
                        k.hi[d] = axk[d]->hi;
                        wb[d] = axk[d]->wb;
                        k.sh[d] = axk[d]->sh;
                        inside_valid = inside_valid && axk[d]->inside;
                    }
                    k.kind = 0;
                    k.own = -1;
                    if (ghosts_only && inside_valid) continue;
                    const int own = S ? S->owner[((size_t)wb[2] * G.owner_nb[1] + wb[1]) *
                                                     G.owner_nb[0] +
                                                 wb[0]]
                                      : -1;
                    if (own >= 0) {
                        if (S == &D && own == (int)b && k.sh[0] == 0 && k.sh[1] == 0 &&
                            k.sh[2] == 0)
                            continue;
                        k.kind = 1;
                        k.own = own;
                        continue;
                    }
                    if (!C) continue; /* nothing to fill from: left as is */
                    k.kind = 2; /* parents checked per merged rectangle below */
                }
        /* x-runs of equal kind / source */
        runs.clear();
        for (int z = 0; z < nbk[2]; ++z)
            for (int y = 0; y < nbk[1]; ++y) {
                int x = 0;
                while (x < nbk[0]) {
                    const Blk &k = blk[((size_t)z * nbk[1] + y) * nbk[0] + x];
                    if (k.kind == 0) {
                        ++x;
                        continue;
                    }
                    int x1 = x;
                    while (x1 + 1 < nbk[0]) {
                        const Blk &n = blk[((size_t)z * nbk[1] + y) * nbk[0] + x1 + 1];
                        if (n.kind != k.kind || n.own != k.own || n.sh[0] != k.sh[0] ||
                            n.sh[1] != k.sh[1] || n.sh[2] != k.sh[2])
                            break;
                        ++x1;
                    }
                    const Blk &e = blk[((size_t)z * nbk[1] + y) * nbk[0] + x1];
                    Run r{k.kind, k.own, {k.sh[0], k.sh[1], k.sh[2]},
                          {k.lo[0], k.lo[1], k.lo[2]}, {e.hi[0], k.hi[1], k.hi[2]}};
                    runs.push_back(r);
                    x = x1 + 1;
                }
            }
        /* merge along y, then along z (same kind, source and x extent) */
        for (int d = 1; d <= 2; ++d) {
            merged.clear();
            for (const Run &r : runs) {
                bool done = false;
                for (size_t q = merged.size(); q-- > 0;) {
                    Run &m = merged[q];
                    /* runs are ordered by z: along y only the same plane */
                    if (d == 1 && m.lo[2] != r.lo[2]) break;
                    bool same = m.kind == r.kind && m.own == r.own && m.sh[0] == r.sh[0] &&
                                m.sh[1] == r.sh[1] && m.sh[2] == r.sh[2] &&
                                m.hi[d] + 1 == r.lo[d];
                    for (int e = 0; e < 3 && same; ++e)
                        if (e != d) same = m.lo[e] == r.lo[e] && m.hi[e] == r.hi[e];
                    if (same) {
                        m.hi[d] = r.hi[d];
                        done = true;
                        break;
                    }
                }
                if (!done) merged.push_back(r);
            }
            runs.swap(merged);
        }
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
                box_rects[b].push_back(c);
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
                box_cf[b].push_back(c);
            }
        }
    }
    } /* omp parallel */
    if (uncovered)
        throw PlanError("coarse level does not cover the cells to interpolate (levels "
                                  "are not properly nested)");
    auto cells = [](const int lo[3], const int hi[3]) {
        return (long long)(hi[0] - lo[0] + 1) * (hi[1] - lo[1] + 1) * (hi[2] - lo[2] + 1);
    };
    for (long long b = 0; b < nbox; ++b) {
        for (GhostCopyDev &c : box_rects[b]) {
            c.first = P.rect_cells;
            P.rect_cells += cells(c.lo, c.hi);
            P.rects.push_back(c);
        }
        for (CfRect &c : box_cf[b]) {
            c.first = P.cf_cells;
            P.cf_cells += cells(c.lo, c.hi);
            P.cf.push_back(c);
        }
    }
    return P;
}

} // namespace sh

#endif // SH_FILL_PLAN_H_
