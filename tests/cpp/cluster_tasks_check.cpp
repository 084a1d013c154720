/* Host check of shamr::cluster_parallel (csrc/sh_amr_driver.h): with the
 * large halves clustered as OpenMP tasks, the Berger-Rigoutsos clusters and
 * their order equal those of the serial recursion, on thin random-walk tags,
 * sparse and dense random tags, and a full and an empty set. */
#include <cmath>
#include <cstdio>
#include <random>
#include <vector>

#include "sh_amr_driver.h"

using shamr::BlockSet;
using shamr::IBox;

namespace {

std::vector<uint8_t> tag_set(int nb, unsigned seed, int kind) {
    std::mt19937 rng(seed);
    std::vector<uint8_t> tags((size_t)nb * nb * nb, 0);
    if (kind == 0) { /* string-like random walks */
        std::normal_distribution<double> g(0., 1.);
        for (int s = 0; s < nb / 4 + 1; ++s) {
            double p[3] = {double(rng() % nb), double(rng() % nb), double(rng() % nb)};
            for (int step = 0; step < nb * 4; ++step) {
                int i[3];
                for (int d = 0; d < 3; ++d) {
                    p[d] += g(rng);
                    i[d] = (((int)std::floor(p[d])) % nb + nb) % nb;
                }
                tags[((size_t)i[2] * nb + i[1]) * nb + i[0]] = 1;
            }
        }
    } else if (kind == 1 || kind == 2) {
        std::uniform_real_distribution<double> u(0., 1.);
        const double f = kind == 1 ? 0.01 : 0.3;
        for (auto &t : tags) t = u(rng) < f;
    } else if (kind == 3) {
        for (auto &t : tags) t = 1;
    }
    return tags;
}

} // namespace

int main() {
    int bad = 0, cases = 0;
    for (int nb : {8, 33, 64, 96})
        for (int kind = 0; kind < 5; ++kind)
            for (unsigned seed = 0; seed < 2; ++seed)
                for (double eff : {0.5, 0.7, 0.9}) {
                    const std::vector<uint8_t> tags = tag_set(nb, seed, kind);
                    const BlockSet t{tags, nb};
                    const IBox all{{0, 0, 0}, {nb - 1, nb - 1, nb - 1}};
                    std::vector<IBox> a, b;
                    shamr::cluster(t, all, eff, a);
                    shamr::cluster_parallel(t, all, eff, b, 8);
                    bool same = a.size() == b.size();
                    for (size_t q = 0; same && q < a.size(); ++q)
                        for (int d = 0; d < 3; ++d)
                            same = same && a[q].lo[d] == b[q].lo[d] && a[q].hi[d] == b[q].hi[d];
                    ++cases;
                    if (!same) {
                        ++bad;
                        std::printf("differ: nb %d kind %d seed %u eff %.1f (%zu vs %zu)\n", nb,
                                    kind, seed, eff, a.size(), b.size());
                    }
                }
    if (bad) return 1;
    std::printf("%d cases\nok\n", cases);
    return 0;
}
