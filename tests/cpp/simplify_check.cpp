/* Host check of shamr::simplify (csrc/sh_amr_driver.h): on random sets of
 * disjoint boxes its result equals that of a plain implementation of the
 * same merging rule written here (full passes over the three directions,
 * each ordering the boxes with a comparator and merging neighbours that
 * share a whole face, until a pass merges nothing), and covers the same
 * cells. */
#include <algorithm>
#include <cstdio>
#include <random>
#include <tuple>
#include <vector>

#include "sh_amr_driver.h"

using shamr::IBox;

namespace {

void plain_simplify(std::vector<IBox> &v) {
    bool any = true;
    while (any) {
        any = false;
        for (int d = 0; d < 3; ++d) {
            const int e = (d + 1) % 3, f = (d + 2) % 3;
            std::sort(v.begin(), v.end(), [&](const IBox &a, const IBox &b) {
                return std::make_tuple(a.lo[e], a.hi[e], a.lo[f], a.hi[f], a.lo[d]) <
                       std::make_tuple(b.lo[e], b.hi[e], b.lo[f], b.hi[f], b.lo[d]);
            });
            std::vector<IBox> res;
            for (const IBox &x : v) {
                if (!res.empty()) {
                    IBox &p = res.back();
                    if (p.lo[e] == x.lo[e] && p.hi[e] == x.hi[e] && p.lo[f] == x.lo[f] &&
                        p.hi[f] == x.hi[f] && p.hi[d] + 1 == x.lo[d]) {
                        p.hi[d] = x.hi[d];
                        any = true;
                        continue;
                    }
                }
                res.push_back(x);
            }
            v.swap(res);
        }
    }
}

std::vector<std::tuple<int, int, int, int, int, int>> canon(const std::vector<IBox> &v) {
    std::vector<std::tuple<int, int, int, int, int, int>> out;
    for (const IBox &b : v) out.emplace_back(b.lo[0], b.lo[1], b.lo[2], b.hi[0], b.hi[1], b.hi[2]);
    std::sort(out.begin(), out.end());
    return out;
}

long long cells(const std::vector<IBox> &v) {
    long long n = 0;
    for (const IBox &b : v) n += b.volume();
    return n;
}

} // namespace

int main() {
    std::mt19937 g(11);
    int bad = 0;
    for (int it = 0; it < 400; ++it) {
        const int n = 4 + (int)(g() % 28);
        const double p = (g() % 1000) / 1000.0;
        std::vector<IBox> v;
        /* unit boxes, or 2-wide slabs, of a random set of cells */
        const int wx = 1 + (int)(g() % 2);
        for (int z = 0; z < n; ++z)
            for (int y = 0; y < n; ++y)
                for (int x = 0; x + wx <= n; x += wx)
                    if ((g() % 1000) / 1000.0 < p) v.push_back(IBox{{x, y, z}, {x + wx - 1, y, z}});
        std::shuffle(v.begin(), v.end(), g);
        std::vector<IBox> a = v, b = v;
        shamr::simplify(a);
        plain_simplify(b);
        if (canon(a) != canon(b) || cells(a) != cells(v)) ++bad;
    }
    std::printf(bad ? "FAILED %d\n" : "ok\n", bad);
    return bad ? 1 : 0;
}
