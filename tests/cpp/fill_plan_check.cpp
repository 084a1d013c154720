/* Host check of the fill planning of sledgehamr_gb300/csrc/sh_fill_plan.h:
 * on periodic layouts, every cell a plan is responsible for (the ghost
 * shell of every box for a ghost fill, the whole ghost-grown box for a
 * level-to-level fill) is written by exactly one rectangle; copied cells
 * come from the valid region of the source box named (through the periodic
 * shift); interpolated cells are owned by no source box and their parents
 * lie on the coarse level; overlapping boxes are rejected.  With an
 * argument, also prints the time of the plans of a large layout built by the
 * AMR driver's clustering (the level-2 size of the AMR benchmark). */
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <random>
#include <vector>

#include "sh_amr_driver.h"
#include "sh_fill_plan.h"

using namespace sh;

namespace {

struct Lvl {
    int dlo[3] = {0, 0, 0}, dhi[3];
    std::vector<sh_box> boxes;
    OwnerMap om;
    int nghost = 2;
    PlanLevel view() const {
        PlanLevel p;
        for (int d = 0; d < 3; ++d) {
            p.dlo[d] = dlo[d];
            p.dhi[d] = dhi[d];
            p.owner_nb[d] = om.nb[d];
        }
        p.boxes = boxes.data();
        p.nbox = (int)boxes.size();
        p.nghost = nghost;
        p.ncomp = 4;
        p.owner = om.owner.data();
        p.owner_res = om.res;
        return p;
    }
};

Lvl make_level(int N, const std::vector<sh_box> &boxes, int nghost) {
    Lvl L;
    for (int d = 0; d < 3; ++d) L.dhi[d] = N - 1;
    L.boxes = boxes;
    L.nghost = nghost;
    build_owner_map(L.dlo, L.dhi, L.boxes.data(), (int)L.boxes.size(), L.om);
    return L;
}

std::vector<sh_box> chop(int N, int m) {
    std::vector<sh_box> out;
    for (int z = 0; z < N; z += m)
        for (int y = 0; y < N; y += m)
            for (int x = 0; x < N; x += m)
                out.push_back(sh_box{{x, y, z}, {x + m - 1, y + m - 1, z + m - 1}});
    return out;
}

/* owner box of cell c (periodic) or -1 */
int owner_of(const Lvl &L, const int c[3]) {
    int w[3];
    for (int d = 0; d < 3; ++d) {
        const int n = L.dhi[d] + 1;
        w[d] = ((c[d] % n) + n) % n;
    }
    for (size_t q = 0; q < L.boxes.size(); ++q) {
        bool in = true;
        for (int d = 0; d < 3; ++d) in = in && w[d] >= L.boxes[q].lo[d] && w[d] <= L.boxes[q].hi[d];
        if (in) return (int)q;
    }
    return -1;
}

bool inside(const sh_box &b, const int c[3]) {
    for (int d = 0; d < 3; ++d)
        if (c[d] < b.lo[d] || c[d] > b.hi[d]) return false;
    return true;
}

int fails = 0;
#define CHECK(c, ...)                                                                         \
    do {                                                                                      \
        if (!(c)) {                                                                           \
            if (fails++ < 10) std::printf(__VA_ARGS__);                                        \
        }                                                                                     \
    } while (0)

/* Every cell of box b's ghost-grown region that the plan must write
 * (ghosts only, or all) written exactly once, with the source rules. */
void check_plan(const Lvl &D, const Lvl *S, const Lvl *C, bool ghosts_only, const FillPlan &P) {
    const int g = D.nghost;
    long long rect_cells = 0, cf_cells = 0;
    for (const auto &r : P.rects) {
        CHECK(r.first == rect_cells, "rect prefix wrong\n");
        rect_cells += (long long)(r.hi[0] - r.lo[0] + 1) * (r.hi[1] - r.lo[1] + 1) * (r.hi[2] - r.lo[2] + 1);
    }
    for (const auto &r : P.cf) {
        CHECK(r.first == cf_cells, "cf prefix wrong\n");
        cf_cells += (long long)(r.hi[0] - r.lo[0] + 1) * (r.hi[1] - r.lo[1] + 1) * (r.hi[2] - r.lo[2] + 1);
    }
    CHECK(rect_cells == P.rect_cells && cf_cells == P.cf_cells, "cell totals wrong\n");
    for (size_t b = 0; b < D.boxes.size(); ++b) {
        const sh_box &bx = D.boxes[b];
        const int n[3] = {bx.hi[0] - bx.lo[0] + 1 + 2 * g, bx.hi[1] - bx.lo[1] + 1 + 2 * g,
                          bx.hi[2] - bx.lo[2] + 1 + 2 * g};
        std::vector<int> hits((size_t)n[0] * n[1] * n[2], 0);
        auto idx = [&](int i, int j, int k) {
            return ((size_t)(k - bx.lo[2] + g) * n[1] + (j - bx.lo[1] + g)) * n[0] + (i - bx.lo[0] + g);
        };
        for (const auto &r : P.rects) {
            if (r.dbox != (int)b) continue;
            for (int k = r.lo[2]; k <= r.hi[2]; ++k)
                for (int j = r.lo[1]; j <= r.hi[1]; ++j)
                    for (int i = r.lo[0]; i <= r.hi[0]; ++i) {
                        ++hits[idx(i, j, k)];
                        const int src[3] = {i - r.shift[0], j - r.shift[1], k - r.shift[2]};
                        CHECK(S && inside(S->boxes[r.sbox], src), "copy source outside its box\n");
                    }
        }
        for (const auto &r : P.cf) {
            if (r.dbox != (int)b) continue;
            for (int k = r.lo[2]; k <= r.hi[2]; ++k)
                for (int j = r.lo[1]; j <= r.hi[1]; ++j)
                    for (int i = r.lo[0]; i <= r.hi[0]; ++i) {
                        ++hits[idx(i, j, k)];
                        const int c[3] = {i, j, k};
                        CHECK(!S || owner_of(*S, c) < 0, "interpolated cell owned by a source box\n");
                        const int p[3] = {floordiv(i, 2), floordiv(j, 2), floordiv(k, 2)};
                        CHECK(C && owner_of(*C, p) >= 0, "parent not on the coarse level\n");
                    }
        }
        for (int k = bx.lo[2] - g; k <= bx.hi[2] + g; ++k)
            for (int j = bx.lo[1] - g; j <= bx.hi[1] + g; ++j)
                for (int i = bx.lo[0] - g; i <= bx.hi[0] + g; ++i) {
                    const int c[3] = {i, j, k};
                    const bool valid = inside(bx, c);
                    const int h = hits[idx(i, j, k)];
                    if (ghosts_only && valid) {
                        CHECK(h == 0, "valid cell written by a ghost fill\n");
                        continue;
                    }
                    const bool fillable = (S && owner_of(*S, c) >= 0) || C;
                    CHECK(h == (fillable ? 1 : 0), "cell (%d %d %d) of box %zu written %d times\n", i,
                          j, k, b, h);
                }
    }
}

/* Non-overlapping boxes of 8..16 cells on an 8-cell block grid of an N^3
 * domain: random blocks merged along x. */
std::vector<sh_box> random_boxes(int N, double frac, std::mt19937 &g) {
    const int nb = N / 8;
    std::vector<sh_box> out;
    std::uniform_real_distribution<double> u(0., 1.);
    for (int z = 0; z < nb; ++z)
        for (int y = 0; y < nb; ++y)
            for (int x = 0; x < nb; ++x) {
                if (u(g) >= frac) continue;
                if (!out.empty() && out.back().hi[0] == 8 * x - 1 && out.back().lo[1] == 8 * y &&
                    out.back().lo[2] == 8 * z && out.back().hi[0] - out.back().lo[0] < 15) {
                    out.back().hi[0] += 8;
                    continue;
                }
                out.push_back(sh_box{{8 * x, 8 * y, 8 * z}, {8 * x + 7, 8 * y + 7, 8 * z + 7}});
            }
    return out;
}

} // namespace

int main(int argc, char **argv) {
    std::mt19937 g(7);
    /* A: periodic single level, ghost fill */
    {
        const Lvl L = make_level(48, chop(48, 16), 2);
        const PlanLevel v = L.view();
        const FillPlan P = build_fill_plan(v, &v, nullptr, true);
        CHECK(P.cf.empty(), "periodic level has interpolated cells\n");
        check_plan(L, &L, nullptr, true, P);
    }
    /* B, C: two levels; ghost fill with coarse-fine cells, then a remake
     * from an older layout */
    for (int it = 0; it < 4; ++it) {
        const Lvl Cl = make_level(32, chop(32, 16), 2);
        const Lvl F1 = make_level(64, random_boxes(64, 0.35, g), 2);
        const Lvl F2 = make_level(64, random_boxes(64, 0.35, g), 2);
        const PlanLevel c = Cl.view(), f1 = F1.view(), f2 = F2.view();
        const FillPlan G = build_fill_plan(f1, &f1, &c, true);
        check_plan(F1, &F1, &Cl, true, G);
        const FillPlan R = build_fill_plan(f2, &f1, &c, false);
        check_plan(F2, &F1, &Cl, false, R);
        const FillPlan Z = build_fill_plan(f2, nullptr, &c, false);
        check_plan(F2, nullptr, &Cl, false, Z);
    }
    /* overlapping boxes */
    {
        bool thrown = false;
        try {
            make_level(32, {sh_box{{0, 0, 0}, {15, 15, 15}}, sh_box{{8, 8, 8}, {23, 23, 23}}}, 2);
        } catch (const PlanError &) {
            thrown = true;
        }
        CHECK(thrown, "overlap not detected\n");
    }
    /* an uncovered coarse-fine region */
    {
        const Lvl Cl = make_level(16, {sh_box{{0, 0, 0}, {7, 7, 7}}}, 1);
        const Lvl F = make_level(32, {sh_box{{16, 16, 16}, {23, 23, 23}}}, 1);
        const PlanLevel c = Cl.view(), f = F.view();
        bool thrown = false;
        try {
            build_fill_plan(f, &f, &c, true);
        } catch (const PlanError &) {
            thrown = true;
        }
        CHECK(thrown, "uncovered coarse-fine cells not detected\n");
    }
    if (argc > 1) {
        /* timing: a level of ~1024^3 refined along tubes (clustered as the
         * AMR driver does), its ghost plan, coarse link and a remake */
        const int nb = 128, w = 4;
        std::vector<uint8_t> tags((size_t)nb * nb * nb, 0), allowed(tags.size(), 1);
        std::mt19937 r(1);
        std::uniform_real_distribution<double> u(0., 1.);
        for (int q = 0; q < 60; ++q) {
            const double cx = u(r) * nb, cy = u(r) * nb, cz = u(r) * nb, R = 5 + u(r) * nb / 4;
            for (int t = 0; t < 4000; ++t) {
                const double a = 6.283185307 * t / 4000;
                for (int dz = -1; dz <= 1; ++dz)
                    for (int dy = -1; dy <= 1; ++dy)
                        for (int dx = -1; dx <= 1; ++dx) {
                            const int x = ((int)(cx + R * std::cos(a)) + dx + nb) % nb;
                            const int y = ((int)(cy + R * std::sin(a)) + dy + nb) % nb;
                            const int z = ((int)cz + dz + nb) % nb;
                            tags[((size_t)z * nb + y) * nb + x] = 1;
                        }
            }
        }
        auto bb = shamr::make_boxes(tags, allowed, nb, 2, 0.7, w);
        std::vector<sh_box> fine;
        for (auto &b : bb) fine.push_back(sh_box{{b.lo[0] * 8, b.lo[1] * 8, b.lo[2] * 8},
                                                 {b.hi[0] * 8 + 7, b.hi[1] * 8 + 7, b.hi[2] * 8 + 7}});
        const Lvl Cl = make_level(512, chop(512, 32), 2);
        auto ms = [](auto a, auto b) { return std::chrono::duration<double>(b - a).count() * 1e3; };
        for (int rep = 0; rep < 3; ++rep) {
            auto t0 = std::chrono::steady_clock::now();
            const Lvl F = make_level(1024, fine, 2);
            auto t1 = std::chrono::steady_clock::now();
            const PlanLevel c = Cl.view(), f = F.view();
            const FillPlan G = build_fill_plan(f, &f, nullptr, true);
            auto t2 = std::chrono::steady_clock::now();
            const FillPlan L = build_fill_plan(f, &f, &c, true, false);
            auto t3 = std::chrono::steady_clock::now();
            const FillPlan R = build_fill_plan(f, &f, &c, false);
            auto t4 = std::chrono::steady_clock::now();
            if (rep == 2)
                std::printf("boxes %zu: owner map %.2f ms, ghost plan %.2f ms (%zu rects), coarse "
                            "link %.2f ms (%zu cf), full fill %.2f ms (%zu rects)\n",
                            fine.size(), ms(t0, t1), ms(t1, t2), G.rects.size(), ms(t2, t3),
                            L.cf.size(), ms(t3, t4), R.rects.size());
        }
    }
    std::printf(fails ? "FAILED %d\n" : "ok\n", fails);
    return fails ? 1 : 0;
}
