/* Host-side AMR time stepper: sledgehamr's recursive subcycling with shadow
 * level, truncation-error scheduling and regrids, over a backend that owns
 * the level data and runs the numerical operations.
 *
 * Reference (order of operations restated here):
 *   TimeStepper::Advance ........... source/time_stepper.cpp:90-133
 *   TimeStepper::SynchronizeLevels . time_stepper.cpp:140-162
 *   TimeStepper::SynchronizeTimes .. time_stepper.cpp:168-171
 *   TimeStepper::ScheduleRegrid .... time_stepper.cpp:221-295
 *   TimeStepper::DoRegridIfScheduled / NoShadowRegrid / DoRegrid
 *                                    time_stepper.cpp:301-397
 *   RegridScheduler ................ source/regrid_scheduler.{h,cpp}
 *   Integrator::Advance ............ source/integrators/integrator.cpp:11-31
 *   Sledgehamr::CreateShadowLevel .. source/sledgehamr.cpp:234-251
 *   Sledgehamr::ErrorEst ........... sledgehamr.cpp:207-229
 *   MakeNewLevelFromCoarse / RemakeLevel / ClearLevel
 *                                    sledgehamr.cpp:149-198
 *   AxionStrings CreateLevelIf ..... projects/AxionStrings/cosmology.h:25-27,
 *                                    :46-48 (string width <= threshold)
 *
 * New grids (the part sledgehamr delegates to AMReX's clustering or its
 * local regrid): the tags of level l are buffered by n_error_buf cells,
 * coarsened to blocks of blocking_factor cells of level l+1, restricted to
 * blocks whose surroundings (ceil(nghost/2)+1 cells of level l) lie inside
 * level l.  The blocks are then turned into boxes in one of two ways:
 *   clustering 0 (default): Berger-Rigoutsos clustering (Berger & Rigoutsos,
 *     IEEE Trans. SMC 21 (1991) 1278) of the tagged blocks until every
 *     cluster is at least grid_eff tagged: a cluster is shrunk to the bounding
 *     box of its tags and, if too sparse, cut at the hole of its tag
 *     signatures nearest its middle, else at the strongest zero crossing of
 *     the signatures' second difference, else in half along its longest
 *     side; the clusters are intersected with the nesting region, boxes
 *     sharing a whole face are merged, and boxes longer than max_grid_size
 *     are chopped into near-equal pieces - the sequence of AMReX's
 *     MakeNewGrids (cluster, intersect, simplify, maxSize), restated;
 *   clustering 1: tagged blocks merged inside aligned windows of
 *     max_grid_size cells by x-runs, then equal runs along y, then along z
 *     (every box fully tagged).
 * At most one new level is added per regrid, as in AMReX.
 *
 * The backend B provides (Level is a handle it owns):
 *   Level create(int lev, const std::vector<IBox>&, int N);   // lev -1: shadow
 *   void destroy(Level&);
 *   void set_time(Level&, int which, double t, int istep);
 *   double time(const Level&, int which); int istep(const Level&, int which);
 *   void advance(int lev, Level&, Level *coarse, double dt, double dx, bool no_swap);
 *   void average_down(Level &fine, int which_f, Level &crse, int which_c);
 *   void average_down_te(Level &fine, Level &crse);
 *   std::vector<uint8_t> tag(Level&, bool use_te, double time, int lev,
 *                            double dt, double dx);          // boxes layout
 *   std::vector<uint8_t> tag_blocks(Level&, bool use_te, double time, int lev,
 *                            double dt, double dx, int block, int buffer, int nb);
 *                            // as mask_to_blocks(tag(...), ...)
 *   void fill_from_coarse(Level &fine, Level &crse, double time);
 *   void remake(Level &fresh, Level &old, Level &crse, double time);
 *   void refresh_ghosts(Level&, int which, Level *coarse);
 *   void sync();   // wait for queued device work (timers with sync_timers)
 *   std::vector<double> read_valid(Level&, int which);   // boxes layout
 *   void write_valid(Level&, int which, const std::vector<double>&);
 *   void extend(Level &fresh, Level &old, Level &crse, double t_new, double t_old);
 *        // both time levels of fresh from old where old has cells, else
 *        // from the coarse level at t_new / t_old (LocalRegrid::AddBoxes)
 */
#ifndef SH_AMR_DRIVER_H_
#define SH_AMR_DRIVER_H_

#include <algorithm>
#include <atomic>
#include <cfloat>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <functional>
#include <stdexcept>
#include <string>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace shamr {

constexpr int kNew = 0, kOld = 1;

struct IBox {
    int lo[3];
    int hi[3];
    long long volume() const {
        return (long long)(hi[0] - lo[0] + 1) * (hi[1] - lo[1] + 1) * (hi[2] - lo[2] + 1);
    }
};

struct Config {
    int N0 = 64;                /* coarse cells per side */
    double L = 16.;             /* box length */
    double cfl = 0.25;          /* dt = cfl dx */
    double t_start = 0.1;
    int nghost = 2;
    int max_level = 2;
    int blocking_factor = 8;    /* cells of the created level */
    int max_grid_size = 32;     /* cells of the created level */
    int n_error_buf = 1;        /* cells of the tagged level */
    double regrid_dt = 0.;      /* coarse-level regrid interval */
    std::vector<double> te_crit; /* per component; DBL_MAX: off */
    double string_width_threshold = 0.; /* > 0: AxionStrings CreateLevelIf */
    double string_lambda = 1.;  /* lambda of cosmology.h */
    int clustering = 0;         /* 0 Berger-Rigoutsos, 1 aligned windows */
    double grid_eff = 0.7;      /* minimum tagged fraction of a cluster */
    bool params_mod_norm0 = false; /* TruncationModifier params from level 0 */
    /* LocalRegrid (source/local_regrid/local_regrid.h:97-122): attempts
     * before a global regrid is forced, and the volume thresholds */
    int max_local_regrids = 0;
    double volume_threshold_strong = 1.05; /* amr.volume_threshold_strong */
    double volume_threshold_weak = 1.1;    /* amr.volume_threshold_weak */
};

/* The whole state of a hierarchy between two coarse steps: what the
 * reference's Checkpoint::Write saves (source/output_types/checkpoint.cpp:
 * 18-98: level-0 time, finest level, box arrays, isteps, grid_new of every
 * level) plus what this time stepper needs to continue exactly as if it
 * had not stopped (both time levels with their times and steps, the regrid
 * schedule, the last regrid times, which levels hold truncation errors). */
struct LevelState {
    std::vector<IBox> boxes;
    double t_new = 0., t_old = 0.;
    int s_new = 0, s_old = 0;
    std::vector<double> data_new, data_old; /* valid cells, box after box, comp-major */
};
struct Checkpoint {
    int finest = 0, ncomp = 0, N0 = 0, nghost = 0, max_level = 0, blocking_factor = 0;
    std::vector<LevelState> levels;
    std::vector<double> last_regrid_time;
    std::vector<std::pair<int, double>> schedule; /* (lowest level, time) */
    std::vector<uint8_t> te_valid;
    long long cell_updates = 0;
    /* LocalRegrid state: attempts since the last global regrid, per level
     * the no-local / global-requested flags and the cells at the last
     * global regrid */
    int lr_nregrids = 0;
    std::vector<uint8_t> lr_no_local, lr_do_global;
    std::vector<long long> lr_last_numpts;
};

struct RegridRecord {
    int lev;          /* level whose tags made level lev+1 */
    double time;
    std::vector<IBox> boxes_tagged_level;
    std::vector<uint8_t> mask; /* boxes layout of the tagged level */
    std::vector<IBox> new_boxes;
};

/* ---- Berger-Rigoutsos clustering on the block grid ---- */
struct BlockSet {
    const std::vector<uint8_t> &bits;
    int nb;
    /* optional integral volume of bits, (nb+1)^3 entries: sum[(z m + y) m +
     * x] = set blocks in [0, x) x [0, y) x [0, z), m = nb + 1 */
    const std::vector<int> *sum = nullptr;
    bool at(int x, int y, int z) const {
        return bits[((size_t)z * nb + y) * nb + x] != 0;
    }
    /* set blocks in [x0, x1] x [y0, y1] x [z0, z1] (needs sum) */
    long long box_sum(int x0, int x1, int y0, int y1, int z0, int z1) const {
        const size_t m = (size_t)nb + 1;
        auto S = [&](int x, int y, int z) { return (long long)(*sum)[((size_t)z * m + y) * m + x]; };
        ++x1;
        ++y1;
        ++z1;
        return S(x1, y1, z1) - S(x0, y1, z1) - S(x1, y0, z1) - S(x1, y1, z0) + S(x0, y0, z1) +
               S(x0, y1, z0) + S(x1, y0, z0) - S(x0, y0, z0);
    }
};

/* The integral volume of an nb^3 block set (prefix sums along x, y, z),
 * built on `threads` host threads. */
inline std::vector<int> integral_volume(const std::vector<uint8_t> &bits, int nb, int threads) {
    const size_t m = (size_t)nb + 1;
    std::vector<int> s(m * m * m, 0);
    (void)threads;
#pragma omp parallel for schedule(static) num_threads(threads)
    for (int z = 0; z < nb; ++z)
        for (int y = 0; y < nb; ++y) {
            const uint8_t *p = &bits[((size_t)z * nb + y) * nb];
            int *q = &s[((size_t)(z + 1) * m + (y + 1)) * m + 1];
            int run = 0;
            for (int x = 0; x < nb; ++x) {
                run += p[x] != 0;
                q[x] = run;
            }
        }
#pragma omp parallel for schedule(static) num_threads(threads)
    for (int z = 1; z <= nb; ++z)
        for (int y = 2; y <= nb; ++y) {
            int *q = &s[((size_t)z * m + y) * m];
            const int *r = q - m;
            for (size_t x = 1; x < m; ++x) q[x] += r[x];
        }
#pragma omp parallel for schedule(static) num_threads(threads)
    for (int y = 1; y <= nb; ++y)
        for (int z = 2; z <= nb; ++z) {
            int *q = &s[((size_t)z * m + y) * m];
            const int *r = q - m * m;
            for (size_t x = 1; x < m; ++x) q[x] += r[x];
        }
    return s;
}

/* Cut of a signature h[0..n-1] (both ends non-zero): position p in
 * [1, n-1] splitting [0, p) | [p, n); kind 2 hole, 1 inflection, 0 none. */
inline int signature_cut(const std::vector<long long> &h, int &kind, long long &strength) {
    const int n = (int)h.size();
    kind = 0;
    strength = 0;
    if (n < 2) return -1;
    const double mid = 0.5 * n;
    int best = -1;
    for (int i = 1; i < n - 1; ++i)
        if (h[i] == 0) {
            /* cut just after the hole; keep the hole nearest the middle */
            const int p = i + 1 <= n - 1 ? i + 1 : i;
            if (best < 0 || std::fabs(p - mid) < std::fabs(best - mid)) best = p;
        }
    if (best > 0) {
        kind = 2;
        return best;
    }
    /* second difference d[i] = h[i-1] - 2 h[i] + h[i+1], i in [1, n-2];
     * zero crossing between i-1 and i (both interior): cut at p = i */
    for (int i = 2; i < n - 1; ++i) {
        const long long a = h[i - 2] - 2 * h[i - 1] + h[i];
        const long long b = h[i - 1] - 2 * h[i] + h[i + 1];
        if ((a < 0 && b > 0) || (a > 0 && b < 0)) {
            const long long st = a > b ? a - b : b - a;
            if (st > strength || (st == strength && best > 0 &&
                                  std::fabs(i - mid) < std::fabs(best - mid))) {
                strength = st;
                best = i;
            }
        }
    }
    if (best > 0) kind = 1;
    return best;
}

/* Halves with at least this many blocks between them are clustered as
 * separate OpenMP tasks when the caller runs cluster_impl<true> inside a
 * parallel region; the clusters come out in the same order either way. */
constexpr long long kClusterTaskBlocks = 1 << 15;

template <bool Tasks>
inline void cluster_impl(const BlockSet &t, IBox bx, double eff, std::vector<IBox> &out) {
    /* signatures over bx, then shrink to the tags' bounding box */
    std::vector<long long> sig[3];
    for (int d = 0; d < 3; ++d) sig[d].assign(bx.hi[d] - bx.lo[d] + 1, 0);
    long long ntag = 0;
    if (t.sum) {
        /* from the integral volume: O(side) instead of O(volume) */
        const int *lo = bx.lo, *hi = bx.hi;
        for (int x = lo[0]; x <= hi[0]; ++x)
            sig[0][x - lo[0]] = t.box_sum(x, x, lo[1], hi[1], lo[2], hi[2]);
        for (int y = lo[1]; y <= hi[1]; ++y)
            sig[1][y - lo[1]] = t.box_sum(lo[0], hi[0], y, y, lo[2], hi[2]);
        for (int z = lo[2]; z <= hi[2]; ++z)
            sig[2][z - lo[2]] = t.box_sum(lo[0], hi[0], lo[1], hi[1], z, z);
        for (long long v : sig[0]) ntag += v;
    } else {
        /* row by row without branches: x counts per element, y and z
         * counts per row sum */
        const int nx = bx.hi[0] - bx.lo[0] + 1;
        std::vector<int> sx(nx, 0);
        for (int z = bx.lo[2]; z <= bx.hi[2]; ++z)
            for (int y = bx.lo[1]; y <= bx.hi[1]; ++y) {
                const uint8_t *p = &t.bits[((size_t)z * t.nb + y) * t.nb + bx.lo[0]];
                int row = 0;
                for (int x = 0; x < nx; ++x) {
                    const int v = p[x] != 0;
                    sx[x] += v;
                    row += v;
                }
                sig[1][y - bx.lo[1]] += row;
                sig[2][z - bx.lo[2]] += row;
                ntag += row;
            }
        for (int x = 0; x < nx; ++x) sig[0][x] = sx[x];
    }
    if (ntag == 0) return;
    IBox b = bx;
    for (int d = 0; d < 3; ++d) {
        int a = 0, e = (int)sig[d].size() - 1;
        while (sig[d][a] == 0) ++a;
        while (sig[d][e] == 0) --e;
        b.lo[d] = bx.lo[d] + a;
        b.hi[d] = bx.lo[d] + e;
        sig[d] = std::vector<long long>(sig[d].begin() + a, sig[d].begin() + e + 1);
    }
    if ((double)ntag >= eff * (double)b.volume()) {
        out.push_back(b);
        return;
    }
    int dir = -1, pos = -1, bestkind = -1;
    long long beststr = -1;
    for (int d = 0; d < 3; ++d) {
        int kind;
        long long st;
        const int p = signature_cut(sig[d], kind, st);
        if (p <= 0) continue;
        const bool better = kind > bestkind || (kind == bestkind && kind == 1 && st > beststr) ||
                            (kind == bestkind && kind == 2 &&
                             b.hi[d] - b.lo[d] > b.hi[dir] - b.lo[dir]);
        if (better) {
            dir = d;
            pos = p;
            bestkind = kind;
            beststr = st;
        }
    }
    if (bestkind == 1 && beststr <= 2) bestkind = 0; /* too weak: bisect */
    if (bestkind <= 0) {
        dir = 0;
        for (int d = 1; d < 3; ++d)
            if (b.hi[d] - b.lo[d] > b.hi[dir] - b.lo[dir]) dir = d;
        pos = (b.hi[dir] - b.lo[dir] + 1) / 2;
        if (pos == 0) { /* a single block (cannot happen: eff <= 1) */
            out.push_back(b);
            return;
        }
    }
    IBox l = b, r = b;
    l.hi[dir] = b.lo[dir] + pos - 1;
    r.lo[dir] = b.lo[dir] + pos;
    if (Tasks && b.volume() >= kClusterTaskBlocks) {
        std::vector<IBox> lo_out, hi_out;
#pragma omp task default(none) shared(t, lo_out) firstprivate(l, eff)
        cluster_impl<true>(t, l, eff, lo_out);
#pragma omp task default(none) shared(t, hi_out) firstprivate(r, eff)
        cluster_impl<true>(t, r, eff, hi_out);
#pragma omp taskwait
        out.insert(out.end(), lo_out.begin(), lo_out.end());
        out.insert(out.end(), hi_out.begin(), hi_out.end());
        return;
    }
    cluster_impl<Tasks>(t, l, eff, out);
    cluster_impl<Tasks>(t, r, eff, out);
}

inline void cluster(const BlockSet &t, IBox bx, double eff, std::vector<IBox> &out) {
    cluster_impl<false>(t, bx, eff, out);
}

/* Host threads for the parallel parts of one regrid.  Hierarchies stepped
 * on several host threads at once (one per served request) regrid
 * concurrently; each then takes an equal share of the cores instead of a
 * full team of its own, and a regrid inside a parallel region takes one. */
class RegridTeam {
  public:
    RegridTeam() : n_(active().fetch_add(1) + 1) {}
    ~RegridTeam() { active().fetch_sub(1); }
    RegridTeam(const RegridTeam &) = delete;
    RegridTeam &operator=(const RegridTeam &) = delete;
    int threads() const {
#ifdef _OPENMP
        if (omp_in_parallel()) return 1;
        return std::max(1, omp_get_max_threads() / std::max(1, n_));
#else
        return 1;
#endif
    }

  private:
    static std::atomic<int> &active() {
        static std::atomic<int> a{0};
        return a;
    }
    int n_;
};

/* cluster() with the large halves as OpenMP tasks of a team of its own
 * (threads: the caller's share of the host cores). */
inline void cluster_parallel(const BlockSet &t, IBox bx, double eff, std::vector<IBox> &out,
                             int threads) {
    if (threads <= 1) {
        cluster_impl<false>(t, bx, eff, out);
        return;
    }
#pragma omp parallel num_threads(threads) default(none) shared(t, bx, eff, out)
#pragma omp single
    cluster_impl<true>(t, bx, eff, out);
}

/* Stable LSD radix sort of (key, index) pairs by key, 11 bits per pass. */
inline void radix_sort_keyed(std::vector<std::pair<unsigned long long, unsigned>> &v,
                             std::vector<std::pair<unsigned long long, unsigned>> &tmp,
                             int key_bits) {
    constexpr int kBits = 11, kBuckets = 1 << kBits;
    tmp.resize(v.size());
    std::vector<size_t> count(kBuckets);
    for (int shift = 0; shift < key_bits; shift += kBits) {
        std::fill(count.begin(), count.end(), 0);
        for (const auto &e : v) ++count[(e.first >> shift) & (kBuckets - 1)];
        size_t sum = 0;
        for (size_t &c : count) {
            const size_t n = c;
            c = sum;
            sum += n;
        }
        for (const auto &e : v) tmp[count[(e.first >> shift) & (kBuckets - 1)]++] = e;
        v.swap(tmp);
    }
}

/* Boxes sharing a whole face are merged (BoxList::simplify): along each
 * direction d in turn, the boxes ordered by (lo[e], hi[e], lo[f], hi[f],
 * lo[d]) and neighbours in that order merged, until no direction merges
 * anything.  The boxes are disjoint, so that key is unique and any sort
 * gives the same order; with coordinates in [0, 4096) it is packed into one
 * 64-bit integer (as many bits per coordinate as the largest needs) and
 * radix-sorted.  A direction is skipped while the boxes
 * have not changed since it last merged nothing (it would merge nothing
 * again), so the merges, and the result, are those of full passes. */
inline void simplify(std::vector<IBox> &v) {
    bool small = true;
    int maxc = 0;
    for (const IBox &x : v)
        for (int d = 0; d < 3; ++d) {
            small = small && x.lo[d] >= 0 && x.hi[d] < 4096;
            maxc = std::max(maxc, x.hi[d]);
        }
    /* bits per packed coordinate: as many as the largest one needs */
    int cb = 1;
    while (cb < 12 && (maxc >> cb) != 0) ++cb;
    std::vector<std::pair<unsigned long long, unsigned>> keyed, tmp;
    std::vector<IBox> sorted;
    int clean = 0; /* directions in a row known to merge nothing */
    for (int d = 0; clean < 3; d = (d + 1) % 3) {
        const int e = (d + 1) % 3, f = (d + 2) % 3;
        if (small) {
            keyed.resize(v.size());
            for (size_t q = 0; q < v.size(); ++q) {
                const IBox &a = v[q];
                keyed[q].first = ((unsigned long long)a.lo[e] << (4 * cb)) |
                                 ((unsigned long long)a.hi[e] << (3 * cb)) |
                                 ((unsigned long long)a.lo[f] << (2 * cb)) |
                                 ((unsigned long long)a.hi[f] << cb) |
                                 (unsigned long long)a.lo[d];
                keyed[q].second = (unsigned)q;
            }
            radix_sort_keyed(keyed, tmp, 5 * cb);
            sorted.resize(v.size());
            for (size_t q = 0; q < v.size(); ++q) sorted[q] = v[keyed[q].second];
            v.swap(sorted);
        } else {
            std::sort(v.begin(), v.end(), [&](const IBox &a, const IBox &b) {
                if (a.lo[e] != b.lo[e]) return a.lo[e] < b.lo[e];
                if (a.hi[e] != b.hi[e]) return a.hi[e] < b.hi[e];
                if (a.lo[f] != b.lo[f]) return a.lo[f] < b.lo[f];
                if (a.hi[f] != b.hi[f]) return a.hi[f] < b.hi[f];
                return a.lo[d] < b.lo[d];
            });
        }
        std::vector<IBox> res;
        bool merged = false;
        for (const IBox &x : v) {
            if (!res.empty()) {
                IBox &p = res.back();
                if (p.lo[e] == x.lo[e] && p.hi[e] == x.hi[e] && p.lo[f] == x.lo[f] &&
                    p.hi[f] == x.hi[f] && p.hi[d] + 1 == x.lo[d]) {
                    p.hi[d] = x.hi[d];
                    merged = true;
                    continue;
                }
            }
            res.push_back(x);
        }
        v.swap(res);
        /* merging along d leaves nothing to merge along d */
        clean = merged ? 1 : clean + 1;
    }
}

/* Boxes longer than w along an axis chopped into near-equal pieces. */
inline void max_size(std::vector<IBox> &v, int w) {
    for (int d = 0; d < 3; ++d) {
        std::vector<IBox> res;
        for (const IBox &x : v) {
            const int len = x.hi[d] - x.lo[d] + 1;
            const int n = (len + w - 1) / w;
            int lo = x.lo[d];
            for (int q = 0; q < n; ++q) {
                const int sz = len / n + (q < len % n ? 1 : 0);
                IBox y = x;
                y.lo[d] = lo;
                y.hi[d] = lo + sz - 1;
                lo += sz;
                res.push_back(y);
            }
        }
        v.swap(res);
    }
}

/* Set blocks inside window [lo, hi] (block coordinates) as boxes: x-runs,
 * merged along y, then along z. */
inline void runs_to_boxes(const BlockSet &t, const int lo[3], const int hi[3],
                          std::vector<IBox> &out) {
    std::vector<IBox> runs;
    for (int z = lo[2]; z <= hi[2]; ++z)
        for (int y = lo[1]; y <= hi[1]; ++y) {
            int x = lo[0];
            while (x <= hi[0]) {
                if (!t.at(x, y, z)) {
                    ++x;
                    continue;
                }
                int x1 = x;
                while (x1 + 1 <= hi[0] && t.at(x1 + 1, y, z)) ++x1;
                runs.push_back(IBox{{x, y, z}, {x1, y, z}});
                x = x1 + 1;
            }
        }
    auto merge = [&](int d) {
        std::vector<IBox> res;
        for (const IBox &r : runs) {
            bool merged = false;
            for (IBox &p : res) {
                bool same = p.hi[d] + 1 == r.lo[d];
                for (int e = 0; e < 3 && same; ++e)
                    if (e != d) same = p.lo[e] == r.lo[e] && p.hi[e] == r.hi[e];
                if (same) {
                    p.hi[d] = r.hi[d];
                    merged = true;
                    break;
                }
            }
            if (!merged) res.push_back(r);
        }
        runs.swap(res);
    };
    merge(1);
    merge(2);
    out.insert(out.end(), runs.begin(), runs.end());
}

/* Boxes (block coordinates) covering the set blocks of `tags` (nb^3 blocks,
 * x fastest), inside the allowed blocks, at most w blocks per side:
 * clustering 0 Berger-Rigoutsos to efficiency grid_eff over the whole
 * domain, then nesting, merging and chopping; 2 the same inside every
 * aligned window of w^3 blocks (the windows that hold tags are clustered
 * independently, in parallel); 1 aligned windows of fully tagged runs. */
inline std::vector<IBox> make_boxes(const std::vector<uint8_t> &tagbits,
                                    const std::vector<uint8_t> &allowed, int nb, int clustering,
                                    double grid_eff, int w) {
    const BlockSet tags{tagbits, nb};
    const BlockSet nest{allowed, nb};
    const RegridTeam team;
    const int nthreads = team.threads();
    std::vector<IBox> bb;
    auto nested = [&](const std::vector<IBox> &cl, std::vector<IBox> &out) {
        for (const IBox &x : cl) {
            bool all = true;
            for (int z = x.lo[2]; z <= x.hi[2] && all; ++z)
                for (int y = x.lo[1]; y <= x.hi[1] && all; ++y)
                    for (int xx = x.lo[0]; xx <= x.hi[0] && all; ++xx) all = nest.at(xx, y, z);
            if (all) out.push_back(x);
            else runs_to_boxes(nest, x.lo, x.hi, out); /* the cluster within the nesting */
        }
    };
    auto order = [](std::vector<IBox> &v) {
        std::sort(v.begin(), v.end(), [](const IBox &a, const IBox &b) {
            for (int d = 2; d >= 0; --d)
                if (a.lo[d] != b.lo[d]) return a.lo[d] < b.lo[d];
            return false;
        });
    };
    if (clustering == 1 || clustering == 2) {
        const int nw = (nb + w - 1) / w;
        const long long nwin = (long long)nw * nw * nw;
        std::vector<std::vector<IBox>> per(nwin);
#pragma omp parallel for schedule(dynamic, 8) num_threads(nthreads)
        for (long long q = 0; q < nwin; ++q) {
            const int wx = (int)(q % nw) * w, wy = (int)((q / nw) % nw) * w,
                      wz = (int)(q / ((long long)nw * nw)) * w;
            const int lo[3] = {wx, wy, wz};
            const int hi[3] = {std::min(wx + w, nb) - 1, std::min(wy + w, nb) - 1,
                               std::min(wz + w, nb) - 1};
            bool any = false;
            for (int z = lo[2]; z <= hi[2] && !any; ++z)
                for (int y = lo[1]; y <= hi[1] && !any; ++y)
                    for (int x = lo[0]; x <= hi[0] && !any; ++x) any = tags.at(x, y, z);
            if (!any) continue;
            if (clustering == 1) {
                runs_to_boxes(tags, lo, hi, per[q]);
            } else {
                std::vector<IBox> cl;
                cluster(tags, IBox{{lo[0], lo[1], lo[2]}, {hi[0], hi[1], hi[2]}}, grid_eff, cl);
                nested(cl, per[q]);
            }
        }
        for (auto &v : per) bb.insert(bb.end(), v.begin(), v.end());
        if (clustering == 2) {
            simplify(bb);
            max_size(bb, w);
        }
        order(bb);
        return bb;
    }
    /* signatures from an integral volume where it fits in 64 MiB */
    std::vector<int> sum;
    BlockSet tagsum{tagbits, nb};
    if ((long long)(nb + 1) * (nb + 1) * (nb + 1) * sizeof(int) <= (64LL << 20)) {
        sum = integral_volume(tagbits, nb, nthreads);
        tagsum.sum = &sum;
    }
    std::vector<IBox> cl;
    cluster_parallel(tagsum, IBox{{0, 0, 0}, {nb - 1, nb - 1, nb - 1}}, grid_eff, cl, nthreads);
    nested(cl, bb);
    simplify(bb);
    max_size(bb, w);
    order(bb);
    return bb;
}

/* Tags of a level (mask over the valid cells of `boxes`, box after box, x
 * fastest), each grown by buf cells and coarsened to blocks of cb cells,
 * periodically wrapped on nb blocks per side. */
inline std::vector<uint8_t> mask_to_blocks(const std::vector<uint8_t> &mask,
                                           const std::vector<IBox> &boxes, int cb, int buf,
                                           int nb) {
    auto fdiv = [](int a, int b) { return a >= 0 ? a / b : -((-a + b - 1) / b); };
    auto pmod = [](int a, int n) {
        const int r = a % n;
        return r < 0 ? r + n : r;
    };
    std::vector<uint8_t> blk((size_t)nb * nb * nb, 0);
    size_t q = 0;
    for (const IBox &bx : boxes)
        for (int k = bx.lo[2]; k <= bx.hi[2]; ++k)
            for (int j = bx.lo[1]; j <= bx.hi[1]; ++j)
                for (int i = bx.lo[0]; i <= bx.hi[0]; ++i, ++q) {
                    if (!mask[q]) continue;
                    const int b0[3] = {fdiv(i - buf, cb), fdiv(j - buf, cb), fdiv(k - buf, cb)};
                    const int b1[3] = {fdiv(i + buf, cb), fdiv(j + buf, cb), fdiv(k + buf, cb)};
                    for (int bk = b0[2]; bk <= b1[2]; ++bk)
                        for (int bj = b0[1]; bj <= b1[1]; ++bj)
                            for (int bi = b0[0]; bi <= b1[0]; ++bi)
                                blk[((size_t)pmod(bk, nb) * nb + pmod(bj, nb)) * nb +
                                    pmod(bi, nb)] = 1;
                }
    return blk;
}

template <class B>
class Driver {
  public:
    using Level = typename B::Level;

    Driver(B &backend, const Config &cfg) : b(backend), c(cfg) {
        if (c.max_level < 0 || c.N0 <= 0 || c.blocking_factor < 2 ||
            c.max_grid_size % c.blocking_factor != 0 || c.blocking_factor % 2 != 0)
            throw std::invalid_argument("invalid AMR configuration");
        shadow_hierarchy = false;
        for (double x : c.te_crit)
            if (x != DBL_MAX) shadow_hierarchy = true;
        for (int l = 0; l <= c.max_level; ++l) {
            dimN.push_back(c.N0 << l);
            dx.push_back(c.L / (double)dimN[l]);
            dt.push_back(dx[l] * c.cfl);
            regrid_dt.push_back(c.regrid_dt / std::pow(2., l));
            last_regrid_time.push_back(c.t_start);
        }
        levels.resize(c.max_level + 1);
        boxes.resize(c.max_level + 1);
        te_valid.assign(c.max_level + 1, false);
    }

    ~Driver() {
        for (int l = 0; l <= finest; ++l) b.destroy(levels[l]);
        if (shadow_defined) b.destroy(shadow);
    }

    /* Level 0 from the caller's data: boxes of max_grid_size cells. */
    void init_coarse(const std::function<void(Level &)> &fill) {
        boxes[0] = chop(0, c.N0, c.max_grid_size);
        levels[0] = b.create(0, boxes[0], dimN[0]);
        fill(levels[0]);
        b.set_time(levels[0], kNew, c.t_start, 0);
        b.set_time(levels[0], kOld, -DBL_MAX, 0);
        finest = 0;
    }

    /* One coarse step (Evolve's loop body). */
    void step() { advance(0); }

    /* The hierarchy's state between coarse steps (Checkpoint::Write). */
    Checkpoint checkpoint() {
        if (shadow_defined) throw std::runtime_error("checkpoint with a shadow level pending");
        Checkpoint k;
        k.finest = finest;
        k.N0 = c.N0;
        k.nghost = c.nghost;
        k.max_level = c.max_level;
        k.blocking_factor = c.blocking_factor;
        for (int l = 0; l <= finest; ++l) {
            LevelState s;
            s.boxes = boxes[l];
            s.t_new = b.time(levels[l], kNew);
            s.t_old = b.time(levels[l], kOld);
            s.s_new = b.istep(levels[l], kNew);
            s.s_old = b.istep(levels[l], kOld);
            s.data_new = b.read_valid(levels[l], kNew);
            s.data_old = b.read_valid(levels[l], kOld);
            long long cells = 0;
            for (const IBox &x : boxes[l]) cells += x.volume();
            k.ncomp = cells ? (int)((long long)s.data_new.size() / cells) : 0;
            k.levels.push_back(std::move(s));
        }
        k.last_regrid_time = last_regrid_time;
        for (const Sched &q : schedule) k.schedule.push_back({q.lowest, q.t});
        for (bool v : te_valid) k.te_valid.push_back(v ? 1 : 0);
        k.cell_updates = cell_updates;
        k.lr_nregrids = lr_nregrids;
        k.lr_no_local = lr_no_local;
        k.lr_do_global = lr_do_global;
        k.lr_last_numpts = lr_last_numpts;
        return k;
    }

    /* Replaces the hierarchy by a checkpoint's (Checkpoint::Read); the
     * configuration must describe the same grid (coarse size, levels,
     * blocking factor). */
    void restart(const Checkpoint &k) {
        if (k.N0 != c.N0 || k.max_level != c.max_level || k.blocking_factor != c.blocking_factor ||
            k.finest < 0 || k.finest > c.max_level || (int)k.levels.size() != k.finest + 1 ||
            (int)k.last_regrid_time.size() != c.max_level + 1 ||
            (int)k.te_valid.size() != c.max_level + 1)
            throw std::invalid_argument("checkpoint does not match the hierarchy's configuration");
        for (int l = finest; l >= 0; --l)
            if (levels[l]) b.destroy(levels[l]);
        if (shadow_defined) b.destroy(shadow);
        shadow_defined = false;
        for (int l = 0; l <= c.max_level; ++l) {
            levels[l] = Level{};
            boxes[l].clear();
        }
        finest = k.finest;
        for (int l = 0; l <= finest; ++l) {
            const LevelState &s = k.levels[l];
            boxes[l] = s.boxes;
            levels[l] = b.create(l, boxes[l], dimN[l]);
            b.write_valid(levels[l], kNew, s.data_new);
            b.write_valid(levels[l], kOld, s.data_old);
            b.set_time(levels[l], kNew, s.t_new, s.s_new);
            b.set_time(levels[l], kOld, s.t_old, s.s_old);
        }
        last_regrid_time = k.last_regrid_time;
        schedule.clear();
        for (const auto &q : k.schedule) schedule.push_back(Sched{q.first, q.second});
        for (int l = 0; l <= c.max_level; ++l) te_valid[l] = k.te_valid[l] != 0;
        cell_updates = k.cell_updates;
        lr_nregrids = k.lr_nregrids;
        lr_no_local = k.lr_no_local;
        lr_do_global = k.lr_do_global;
        lr_last_numpts = k.lr_last_numpts;
    }

    /* ---- queries ---- */
    int finest = 0;
    bool shadow_hierarchy = false;
    std::vector<std::vector<IBox>> boxes;
    std::vector<Level> levels;
    std::vector<double> dt, dx;
    std::vector<int> dimN;
    std::vector<RegridRecord> regrids;
    bool record_regrids = false;
    long long cell_updates = 0;
    /* With record_trace, the time stepper's operations in order, one string
     * "<op> <level> <time>" each: advance (level, time before the step),
     * schedule (level, regrid time), shadow (-1, shadow time after its
     * step), average_down (coarse level, its time), truncation_errors
     * (level, time), regrid (base level, time). */
    std::vector<std::string> trace;
    bool record_trace = false;

    /* Host wall-clock time spent in the backend operations, by phase.  With
     * sync_timers, queued device work is waited for at both ends of every
     * timed operation, so that the times are those of the operation. */
    struct Timer {
        const char *name;
        double sec;
        long long calls;
    };
    enum { kTAdvance, kTSync, kTShadow, kTTag, kTGrids, kTCreate, kTFill, kTDestroy,
           kTRefresh, kNTimers };
    Timer timers[kNTimers] = {{"advance", 0, 0},          {"synchronize", 0, 0},
                              {"shadow", 0, 0},           {"regrid.tag", 0, 0},
                              {"regrid.new_grids", 0, 0}, {"regrid.create", 0, 0},
                              {"regrid.fill", 0, 0},      {"regrid.destroy", 0, 0},
                              {"regrid.refresh", 0, 0}};
    bool sync_timers = false;

  private:
    struct Clock {
        Driver *d;
        int id;
        std::chrono::steady_clock::time_point t0;
        Clock(Driver *dr, int i) : d(dr), id(i) {
            if (d->sync_timers) d->b.sync();
            t0 = std::chrono::steady_clock::now();
        }
        ~Clock() {
            if (d->sync_timers) d->b.sync();
            d->timers[id].sec +=
                std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
            d->timers[id].calls++;
        }
    };

    B &b;
    Config c;
    Level shadow{};
    bool shadow_defined = false;
    std::vector<bool> te_valid;
    struct Sched {
        int lowest;
        double t;
        bool matches(double time) const {
            double teps = t * 1e-12;
            return t > time - teps && t < time + teps;
        }
    };
    std::vector<Sched> schedule;
    std::vector<double> regrid_dt, last_regrid_time;

    /* One trace event: "<op> <level> <time>", the time printed exactly. */
    void note(const char *op, int lev, double t) {
        if (!record_trace) return;
        char buf[96];
        std::snprintf(buf, sizeof(buf), "%s %d %.17g", op, lev, t);
        trace.push_back(buf);
    }

    /* ---- RegridScheduler ---- */
    int find_schedule(double t) const {
        for (size_t q = 0; q < schedule.size(); ++q)
            if (schedule[q].matches(t)) return (int)q;
        return -1;
    }
    void schedule_regrid(int lev, double t) {
        int id = find_schedule(t);
        if (id < 0) schedule.push_back(Sched{lev, t});
        else schedule[id].lowest = std::min(lev, schedule[id].lowest);
    }
    bool do_regrid_at(int lev, double t) const {
        int id = find_schedule(t);
        return id >= 0 && schedule[id].lowest == lev;
    }
    bool need_te(int lev, double t) const {
        int id = find_schedule(t);
        return id >= 0 && lev >= schedule[id].lowest;
    }
    void did_regrid(double t) {
        int id = find_schedule(t);
        if (id >= 0) schedule.erase(schedule.begin() + id);
    }

    /* ---- project hook: Sledgehamr::DoCreateLevelIf ---- */
    bool create_level_if(int lev, double time) const {
        if (lev <= 0) return true;
        if (c.string_width_threshold <= 0) return true;
        /* StringWidth(lev-1, eta) = 1 / (sqrt(2 lambda) eta dx[lev-1]) */
        const double mr = std::sqrt(2. * c.string_lambda) * time;
        const double width = 1. / (mr * dx[lev - 1]);
        return width <= c.string_width_threshold;
    }

    double tnew(int lev) { return b.time(levels[lev], kNew); }
    int istep_new(int lev) { return b.istep(levels[lev], kNew); }

    /* ---- TimeStepper::Advance ---- */
    void advance(int lev) {
        if (shadow_hierarchy) schedule_regrid_if_needed(lev);
        else no_shadow_regrid(lev);
        note("advance", lev, tnew(lev));
        {
            Clock ck(this, kTAdvance);
            b.advance(lev, levels[lev], lev > 0 ? &levels[lev - 1] : nullptr, dt[lev], dx[lev],
                      false);
        }
        te_valid[lev] = false;
        for (const IBox &bx : boxes[lev]) cell_updates += bx.volume();
        if (lev != finest) {
            advance(lev + 1);
            advance(lev + 1);
        }
        synchronize_levels(lev);
        do_regrid_if_scheduled(lev);
        if (lev == 0)
            for (int l = 1; l <= finest; ++l)
                b.set_time(levels[l], kNew, tnew(0), istep_new(l));
    }

    void synchronize_levels(int lev) {
        Clock ck(this, kTSync);
        const bool te = need_te(lev, tnew(lev));
        if (lev < finest) {
            if (!(shadow_hierarchy && te)) {
                note("average_down", lev, tnew(lev));
                b.average_down(levels[lev + 1], kNew, levels[lev], kNew);
                te_valid[lev + 1] = false;
            }
        }
        if (lev >= 1 - (shadow_hierarchy ? 1 : 0) && te) {
            note("truncation_errors", lev, tnew(lev));
            if (lev == 0) {
                const double ts = b.time(shadow, kNew);
                if (!(std::fabs(ts - tnew(0)) < tnew(0) * 1e-8))
                    throw std::runtime_error("shadow level not in sync with the coarse level");
                b.average_down_te(levels[0], shadow);
                b.destroy(shadow);
                shadow_defined = false;
            } else {
                b.average_down_te(levels[lev], levels[lev - 1]);
            }
            te_valid[lev] = true;
        }
    }

    /* TimeStepper::ScheduleRegrid */
    void schedule_regrid_if_needed(int lev) {
        const double time = tnew(lev);
        const int istep = istep_new(lev);
        if (do_regrid_at(lev, time + dt[lev])) return;
        if (b.time(levels[lev], kOld) == time) return;
        if (lev >= c.max_level) return;
        if (istep % 2 == 0 && lev > 0) return;
        const double next = lev > 0 ? time + 3. * dt[lev] : time + 2. * dt[lev];
        if (!create_level_if(lev + 1, next)) return;
        if (next <= last_regrid_time[lev] + regrid_dt[lev] && !lr_global_requested(lev)) return;
        if (lev == 0 && b.time(levels[0], kOld) == -DBL_MAX) return;
        schedule_regrid(lev, time + dt[lev]);
        note("schedule", lev, time + dt[lev]);
        if (lev == 0) create_shadow_level();
    }

    /* Sledgehamr::CreateShadowLevel + Integrator::Advance(-1) */
    void create_shadow_level() {
        Clock ck(this, kTShadow);
        std::vector<IBox> sb;
        for (const IBox &bx : boxes[0]) {
            IBox s;
            for (int d = 0; d < 3; ++d) {
                s.lo[d] = bx.lo[d] / 2;
                s.hi[d] = bx.hi[d] / 2;
            }
            sb.push_back(s);
        }
        if (shadow_defined) b.destroy(shadow);
        shadow = b.create(-1, sb, dimN[0] / 2);
        shadow_defined = true;
        const double t_old = b.time(levels[0], kOld);
        b.average_down(levels[0], kOld, shadow, kOld);
        b.set_time(shadow, kOld, t_old, 0);
        b.advance(-1, shadow, nullptr, 2. * dt[0], 2. * dx[0], true);
        note("shadow", -1, b.time(shadow, kNew));
    }

    void do_regrid_if_scheduled(int lev) {
        const double time = tnew(lev);
        if (!do_regrid_at(lev, time)) return;
        do_regrid(lev, time);
        did_regrid(time);
    }

    /* TimeStepper::NoShadowRegrid */
    void no_shadow_regrid(int lev) {
        const double time = tnew(lev);
        if (lev >= c.max_level) return;
        if (time + dt[lev] <= last_regrid_time[lev] + regrid_dt[lev] && !lr_global_requested(lev))
            return;
        if (!create_level_if(lev + 1, time + dt[lev])) return;
        do_regrid(lev, time);
    }

    /* TimeStepper::DoRegrid: a local regrid first, the global one if it
     * does not succeed (time_stepper.cpp:346-397). */
    void do_regrid(int lev, double time) {
        if (attempt_local_regrid(lev)) {
            note("local_regrid", lev, time);
        } else {
            note("regrid", lev, time);
            regrid(lev, time);
            did_global_regrid(lev);
        }
        for (int l = lev; l <= finest; ++l) last_regrid_time[l] = time;
    }

    /* ---- LocalRegrid (source/local_regrid/local_regrid.cpp) ----
     * Levels grow by blocking-factor blocks next to their coarse/fine
     * boundaries where tagged cells of the level below come closer than
     * n_error_buf + 1 fine cells, lower levels grow to keep them nested, and
     * the hierarchy keeps every existing box; volume thresholds veto it in
     * favour of a global regrid (now, or at the next opportunity of the
     * level that asked for it). */
    std::vector<uint8_t> lr_no_local, lr_do_global;
    std::vector<long long> lr_last_numpts;
    int lr_nregrids = 0, lr_veto_level = -1;

    bool lr_global_requested(int lev) const {
        return lev < (int)lr_do_global.size() && lr_do_global[lev];
    }
    long long level_cells(int l) const {
        long long n = 0;
        for (const IBox &x : boxes[l]) n += x.volume();
        return n;
    }
    /* LocalRegrid::DidGlobalRegrid */
    void did_global_regrid(int lev) {
        lr_no_local.assign(c.max_level + 1, 0);
        lr_do_global.assign(c.max_level + 1, 0);
        lr_nregrids = 0;
        for (int l = lev + 1; l < (int)lr_last_numpts.size(); ++l)
            lr_last_numpts[l] = l <= finest ? level_cells(l) : 0;
    }
    /* wrapped_index of LocalRegrid::WrapIndices: for block b of level l
     * (1-based, 0 and N+1 wrapping around) a cell inside it */
    int lr_wrapped(int l, int b) const {
        const int bf = c.blocking_factor, nb = dimN[l] / bf;
        if (b == 0) return dimN[l] - bf / 2;
        if (b == nb + 1) return bf / 2;
        return (int)((static_cast<double>(b) - 0.5) * static_cast<double>(bf));
    }
    /* owner map of a level at block resolution (1: a box covers the block) */
    std::vector<uint8_t> block_cover(int l) const {
        const int bf = c.blocking_factor, nb = dimN[l] / bf;
        std::vector<uint8_t> cov((size_t)nb * nb * nb, 0);
        for (const IBox &x : boxes[l])
            for (int k = x.lo[2] / bf; k <= x.hi[2] / bf; ++k)
                for (int j = x.lo[1] / bf; j <= x.hi[1] / bf; ++j)
                    for (int i = x.lo[0] / bf; i <= x.hi[0] / bf; ++i)
                        cov[((size_t)k * nb + j) * nb + i] = 1;
        return cov;
    }
    bool covers_cell(const std::vector<uint8_t> &cov, int l, int i, int j, int k) const {
        const int bf = c.blocking_factor, nb = dimN[l] / bf;
        return cov[((size_t)(k / bf) * nb + j / bf) * nb + i / bf] != 0;
    }

    /* LocalRegrid::DetermineNewBoxArray(lev): blocks of level lev+1 to add
     * (into add[lev+1]) next to tagged cells of level lev closer than
     * (n_error_buf + 1) fine cells to a coarse/fine boundary; returns the
     * shortest distance found (-1 if none). */
    double lr_new_blocks(int lev, std::vector<std::vector<uint8_t>> &add) {
        const double threshold = (double)(c.n_error_buf + 1) * (c.n_error_buf + 1);
        const int ibff = c.blocking_factor;
        const double bff = static_cast<double>(ibff);
        const int nbf = dimN[lev + 1] / ibff;
        const std::vector<uint8_t> cov = block_cover(lev + 1);
        const double time = tnew(lev);
        /* ErrorEst of level lev (its cell mask, boxes layout) */
        if (c.params_mod_norm0) b.params_mod_from_norm0(levels[0], time);
        const std::vector<uint8_t> mask =
            b.tag(levels[lev], shadow_hierarchy, time, lev, dt[lev], dx[lev]);
        long long best = -1;
        size_t q0 = 0;
        for (const IBox &bx : boxes[lev]) {
            const int nx = bx.hi[0] - bx.lo[0] + 1, ny = bx.hi[1] - bx.lo[1] + 1;
            int c0[3], c1[3], xs[3];
            for (int d = 0; d < 3; ++d) {
                c0[d] = static_cast<int>(static_cast<double>(bx.lo[d] * 2) / bff) + 1;
                c1[d] = static_cast<int>(static_cast<double>(bx.hi[d] * 2) / bff) + 1;
                xs[d] = c1[d] - c0[d] + 1;
            }
            /* GetBoxCoarseFineBorders: blocks around the box's blocks that
             * level lev+1 does not cover */
            const int bx0 = xs[0] + 2, bx1 = xs[1] + 2;
            std::vector<uint8_t> border((size_t)bx0 * bx1 * (xs[2] + 2));
            auto bref = [&](int i, int j, int k) -> uint8_t & {
                return border[((size_t)k * bx1 + j) * bx0 + i];
            };
            int remaining = 0;
            for (int k = -1; k <= xs[2]; ++k)
                for (int j = -1; j <= xs[1]; ++j)
                    for (int i = -1; i <= xs[0]; ++i) {
                        const bool open = !covers_cell(cov, lev + 1, lr_wrapped(lev + 1, c0[0] + i),
                                                       lr_wrapped(lev + 1, c0[1] + j),
                                                       lr_wrapped(lev + 1, c0[2] + k));
                        bref(i + 1, j + 1, k + 1) = open;
                        remaining += open;
                    }
            if (remaining > 0) {
                /* TagAndMeasure / CheckBorders over the tagged cells */
                for (int k = bx.lo[2]; k <= bx.hi[2]; ++k)
                    for (int j = bx.lo[1]; j <= bx.hi[1]; ++j)
                        for (int i = bx.lo[0]; i <= bx.hi[0]; ++i) {
                            const size_t m = q0 + (size_t)(i - bx.lo[0]) +
                                             (size_t)nx * ((j - bx.lo[1]) + (size_t)ny * (k - bx.lo[2]));
                            if (!mask[m]) continue;
                            const int ci[3] = {i, j, k};
                            int fi[3], cfi[3];
                            for (int d = 0; d < 3; ++d) {
                                fi[d] = ci[d] * 2;
                                cfi[d] = static_cast<int>(static_cast<double>(fi[d]) / bff) + 1;
                            }
                            for (int kk = -1; kk <= 1; ++kk)
                                for (int jj = -1; jj <= 1; ++jj)
                                    for (int ii = -1; ii <= 1; ++ii) {
                                        const int cii[3] = {ii, jj, kk};
                                        int ref[3];
                                        for (int d = 0; d < 3; ++d) ref[d] = cfi[d] - c0[d] + cii[d] + 1;
                                        if (!bref(ref[0], ref[1], ref[2])) continue;
                                        long long d_sq = 0;
                                        for (int d = 0; d < 3; ++d) {
                                            const long long smt = (long long)ibff * (cfi[d] + cii[d] - 1);
                                            const long long bgt = (long long)ibff * (cfi[d] + cii[d]) - 1;
                                            const long long f = fi[d];
                                            d_sq += (smt < f && f < bgt)
                                                        ? 0
                                                        : std::min((f - smt) * (f - smt), (f - bgt) * (f - bgt));
                                        }
                                        if (best < 0 || d_sq < best) best = d_sq;
                                        if ((double)d_sq < threshold) {
                                            bref(ref[0], ref[1], ref[2]) = 0;
                                            int blk[3];
                                            for (int d = 0; d < 3; ++d)
                                                blk[d] = static_cast<int>(
                                                    static_cast<double>(lr_wrapped(lev + 1, cfi[d] + cii[d])) / bff - 0.5);
                                            add[lev + 1][((size_t)blk[2] * nbf + blk[1]) * nbf + blk[0]] = 1;
                                        }
                                    }
                        }
            }
            q0 += (size_t)bx.volume();
        }
        return best >= 0 ? std::sqrt(static_cast<double>(best)) : -1.;
    }

    /* LocalRegrid::FixNesting(lev): blocks of level lev-1 to add so that the
     * blocks added to level lev, grown by nghost + 4 cells, lie in it */
    void lr_fix_nesting(int lev, std::vector<std::vector<uint8_t>> &add) {
        const int bf = c.blocking_factor, nb = dimN[lev] / bf, nbc = dimN[lev - 1] / bf;
        const std::vector<uint8_t> cov = block_cover(lev - 1);
        const int g = c.nghost + 4, Nc = dimN[lev - 1];
        const double bfc = static_cast<double>(bf);
        auto cdiv = [](int a) { return a >= 0 ? a / 2 : -((-a + 1) / 2); };
        for (int k = 0; k < nb; ++k)
            for (int j = 0; j < nb; ++j)
                for (int i = 0; i < nb; ++i) {
                    if (!add[lev][((size_t)k * nb + j) * nb + i]) continue;
                    /* the block grown by g cells, coarsened by 2 */
                    int lo[3], hi[3];
                    const int bl[3] = {i, j, k};
                    for (int d = 0; d < 3; ++d) {
                        lo[d] = cdiv(bl[d] * bf - g);
                        hi[d] = cdiv((bl[d] + 1) * bf - 1 + g);
                    }
                    /* WrapBoxArray: the periodic pieces inside [0, Nc) */
                    for (int sz = -1; sz <= 1; ++sz)
                        for (int sy = -1; sy <= 1; ++sy)
                            for (int sx = -1; sx <= 1; ++sx) {
                                const int sh[3] = {sx, sy, sz};
                                int plo[3], phi[3];
                                bool empty = false;
                                for (int d = 0; d < 3; ++d) {
                                    plo[d] = std::max(lo[d], sh[d] * Nc) - sh[d] * Nc;
                                    phi[d] = std::min(hi[d], (sh[d] + 1) * Nc - 1) - sh[d] * Nc;
                                    empty = empty || plo[d] > phi[d];
                                }
                                if (empty) continue;
                                int cl[3], ch[3];
                                for (int d = 0; d < 3; ++d) {
                                    cl[d] = static_cast<int>(static_cast<double>(plo[d]) / bfc + 1.);
                                    ch[d] = static_cast<int>(static_cast<double>(phi[d]) / bfc + 2.);
                                }
                                for (int cx = cl[0]; cx <= ch[0]; ++cx)
                                    for (int cy = cl[1]; cy <= ch[1]; ++cy)
                                        for (int cz = cl[2]; cz <= ch[2]; ++cz) {
                                            const int ct[3] = {lr_wrapped(lev - 1, cx),
                                                               lr_wrapped(lev - 1, cy),
                                                               lr_wrapped(lev - 1, cz)};
                                            if (covers_cell(cov, lev - 1, ct[0], ct[1], ct[2])) continue;
                                            int blk[3];
                                            for (int d = 0; d < 3; ++d)
                                                blk[d] = static_cast<int>(static_cast<double>(ct[d]) / bfc - 0.5);
                                            add[lev - 1][((size_t)blk[2] * nbc + blk[1]) * nbc + blk[0]] = 1;
                                        }
                            }
                }
    }

    /* the added blocks of a level as boxes (cells) */
    std::vector<IBox> lr_boxes(int l, const std::vector<uint8_t> &blk) const {
        const int bf = c.blocking_factor, nb = dimN[l] / bf;
        const BlockSet t{blk, nb};
        const int lo[3] = {0, 0, 0}, hi[3] = {nb - 1, nb - 1, nb - 1};
        std::vector<IBox> bb;
        runs_to_boxes(t, lo, hi, bb);
        simplify(bb);
        max_size(bb, c.max_grid_size / bf);
        std::vector<IBox> out;
        for (const IBox &r : bb)
            out.push_back(IBox{{r.lo[0] * bf, r.lo[1] * bf, r.lo[2] * bf},
                               {(r.hi[0] + 1) * bf - 1, (r.hi[1] + 1) * bf - 1,
                                (r.hi[2] + 1) * bf - 1}});
        return out;
    }

    /* LocalRegrid::AttemptRegrid / DoAttemptRegrid: true when the local
     * regrid succeeded (boxes added, or deliberately nothing done) */
    bool attempt_local_regrid(int lev) {
        if ((int)lr_no_local.size() != c.max_level + 1) {
            lr_no_local.assign(c.max_level + 1, 0);
            lr_do_global.assign(c.max_level + 1, 0);
        }
        /* Prechecks */
        if (lr_nregrids++ >= c.max_local_regrids) return false;
        if (c.volume_threshold_weak <= 1.) {
            lr_veto_level = lev - 1;
            return false;
        }
        lr_veto_level = -1;
        if (lr_do_global[lev]) return false;
        if (lev == finest) return false;
        /* InitializeLocalRegrid */
        while ((int)lr_last_numpts.size() <= finest)
            lr_last_numpts.push_back(level_cells((int)lr_last_numpts.size()));
        /* DetermineAllBoxArrays */
        std::vector<std::vector<uint8_t>> add(finest + 1);
        for (int l = 0; l <= finest; ++l) {
            const int nb = dimN[l] / c.blocking_factor;
            add[l].assign((size_t)nb * nb * nb, 0);
        }
        std::vector<double> min_distance(finest + 1, -1.);
        {
            Clock ck(this, kTTag);
            for (int l = lev; l < finest && !lr_no_local[l]; ++l)
                min_distance[l + 1] = lr_new_blocks(l, add);
        }
        /* FixAllNesting */
        for (int l = finest; l > 1; --l) lr_fix_nesting(l, add);
        std::vector<std::vector<IBox>> nbx(finest + 1);
        for (int l = 1; l <= finest; ++l) nbx[l] = lr_boxes(l, add[l]);
        /* CheckForVeto */
        bool veto = false;
        std::vector<double> latest(finest + 1, -1.);
        for (int l = 1; l <= finest; ++l) {
            long long Nb = 0;
            for (const IBox &x : nbx[l]) Nb += x.volume();
            const double Nc = (double)level_cells(l);
            double Nr = (double)lr_last_numpts[l];
            if (Nr == 0) Nr = Nc;
            const double fV = ((double)Nb + Nc) / Nr;
            if (fV > c.volume_threshold_weak) veto = true;
            if (fV > c.volume_threshold_strong && lr_veto_level == -1) lr_veto_level = l - 1;
            if (l > lev) { /* ComputeLatestPossibleRegridTime */
                const double dt_delay = min_distance[l] >= 0
                                            ? min_distance[l] / c.n_error_buf * regrid_dt[l]
                                            : DBL_MAX;
                latest[l] = tnew(l) + dt_delay;
            }
        }
        if (veto) { /* DealWithVeto */
            if (lr_veto_level >= lev || lr_veto_level == 0) return false;
            lr_do_global[lr_veto_level] = 1;
            double nsteps = istep_new(lr_veto_level) % 2 == 0 ? 1 : 2;
            if (shadow_hierarchy) nsteps = 0;
            const double target = tnew(lr_veto_level) + nsteps * dt[lr_veto_level];
            bool can_wait = true;
            for (int l = lev + 1; l <= finest; ++l)
                if (latest[l] < target) can_wait = false;
            if (can_wait) {
                for (int l = lev; l <= finest; ++l) lr_no_local[l] = 1;
                return true;
            }
        }
        /* AddAllBoxes.  The new boxes are interpolated from their coarse
         * level, which the GPU reads with its ghost cells; the average-down
         * at the end of the step left those stale, so they are refreshed
         * from the coarsest level up first, as the global regrid refreshes
         * a level before remaking the one above it */
        bool grows = false;
        for (int l = 1; l <= finest; ++l) grows = grows || !nbx[l].empty();
        if (grows) {
            Clock ck(this, kTRefresh);
            for (int l = 0; l < finest; ++l)
                b.refresh_ghosts(levels[l], kNew, l > 0 ? &levels[l - 1] : nullptr);
        }
        for (int l = 1; l <= finest; ++l)
            if (!nbx[l].empty()) lr_add_boxes(l, nbx[l]);
        return true;
    }

    /* LocalRegrid::AddBoxes: level l with its boxes followed by the new
     * ones, both time levels of the new boxes filled at their times (from
     * the coarse level), the existing cells kept.  With truncation-error
     * tags the old time levels of this level and of the coarse one hold the
     * errors after a regrid step, so what the new boxes receive there is as
     * meaningless as the rest of that buffer; the next step swaps the time
     * levels and overwrites it before anything reads it */
    void lr_add_boxes(int l, const std::vector<IBox> &add) {
        std::vector<IBox> nb = boxes[l];
        nb.insert(nb.end(), add.begin(), add.end());
        const double tn = b.time(levels[l], kNew), to = b.time(levels[l], kOld);
        const int sn = b.istep(levels[l], kNew), so = b.istep(levels[l], kOld);
        Level fresh;
        {
            Clock ck(this, kTCreate);
            fresh = b.create(l, nb, dimN[l]);
        }
        {
            Clock ck(this, kTFill);
            b.extend(fresh, levels[l], levels[l - 1], tn, to);
        }
        {
            Clock ck(this, kTDestroy);
            b.destroy(levels[l]);
        }
        levels[l] = fresh;
        boxes[l] = nb;
        b.set_time(levels[l], kNew, tn, sn);
        b.set_time(levels[l], kOld, to, so);
        te_valid[l] = false;
        if (l < finest) { /* the coarse level of the next extension */
            Clock ck(this, kTRefresh);
            b.refresh_ghosts(levels[l], kNew, &levels[l - 1]);
        }
    }

    /* ---- new grids ---- */
    static std::vector<IBox> chop(int lo_unused, int N, int mg) {
        std::vector<IBox> r;
        for (int z = 0; z < N; z += mg)
            for (int y = 0; y < N; y += mg)
                for (int x = 0; x < N; x += mg)
                    r.push_back(IBox{{x, y, z},
                                     {std::min(x + mg, N) - 1, std::min(y + mg, N) - 1,
                                      std::min(z + mg, N) - 1}});
        return r;
    }

    static int pmod(int a, int n) {
        int r = a % n;
        return r < 0 ? r + n : r;
    }
    static int fdiv(int a, int b) { return a >= 0 ? a / b : -((-a + b - 1) / b); }

    /* Sledgehamr::ErrorEst: tags of level l at `time` (empty if skipped). */
    /* Tags of level l for the grids of level l+1: the buffered tags at
     * block resolution (blocks of blocking_factor cells of level l+1), and
     * with record_regrids the cell mask too.  Empty when not tagging. */
    struct Tags {
        std::vector<uint8_t> blocks, mask;
    };
    int block_cells() const { return c.blocking_factor / 2; } /* in level-l cells */
    Tags error_est(int l, double time) {
        Tags t;
        if (time == c.t_start && shadow_hierarchy) return t;
        if (!create_level_if(l + 1, time)) return t;
        if (shadow_hierarchy && !te_valid[l])
            throw std::runtime_error("tagging with truncation errors but none computed on level " +
                                     std::to_string(l));
        const int cb = block_cells();
        if (dimN[l] % cb != 0) throw std::runtime_error("level size not a multiple of the block");
        const int nb = dimN[l] / cb;
        Clock ck(this, kTTag);
        /* FirstOrderPhaseTransition::SetParamsTruncationModifier: the field
         * maxima of level 0 at this time (FirstOrderPhaseTransition.cpp:
         * 133-157) */
        if (c.params_mod_norm0) b.params_mod_from_norm0(levels[0], time);
        if (record_regrids) {
            t.mask = b.tag(levels[l], shadow_hierarchy, time, l, dt[l], dx[l]);
            t.blocks = mask_to_blocks(t.mask, boxes[l], cb, c.n_error_buf, nb);
        } else {
            t.blocks = b.tag_blocks(levels[l], shadow_hierarchy, time, l, dt[l], dx[l], cb,
                                    c.n_error_buf, nb);
        }
        return t;
    }

    /* New boxes of level l+1 from the block tags of level l, nested in the
     * (new) boxes of level l. */
    std::vector<IBox> new_grids(int l, std::vector<uint8_t> blk,
                                const std::vector<IBox> &nest_boxes) {
        const int bf = c.blocking_factor;
        const int cb = block_cells();       /* block size in level-l cells */
        const int Nl = dimN[l];
        const int nb = Nl / cb;             /* blocks per side */
        /* nesting: a block is allowed when the block grown by m level-l
         * cells lies in level l (every block on level 0) */
        std::vector<uint8_t> allowed((size_t)nb * nb * nb, 1);
        if (l >= 1) {
            const int m = (c.nghost + 1) / 2 + 1;
            const int lb = c.blocking_factor; /* level-l boxes are unions of these */
            const int nlb = Nl / lb;
            std::vector<uint8_t> cov((size_t)nlb * nlb * nlb, 0);
            for (const IBox &bx : nest_boxes)
                for (int k = bx.lo[2] / lb; k <= bx.hi[2] / lb; ++k)
                    for (int j = bx.lo[1] / lb; j <= bx.hi[1] / lb; ++j)
                        for (int i = bx.lo[0] / lb; i <= bx.hi[0] / lb; ++i)
                            cov[((size_t)k * nlb + j) * nlb + i] = 1;
            const RegridTeam team;
            const int nthreads = team.threads();
#pragma omp parallel for schedule(static) num_threads(nthreads)
            for (int bk = 0; bk < nb; ++bk)
                for (int bj = 0; bj < nb; ++bj)
                    for (int bi = 0; bi < nb; ++bi) {
                        const int lo[3] = {bi * cb - m, bj * cb - m, bk * cb - m};
                        const int hi[3] = {(bi + 1) * cb + m - 1, (bj + 1) * cb + m - 1,
                                           (bk + 1) * cb + m - 1};
                        bool ok = true;
                        for (int z = fdiv(lo[2], lb); ok && z <= fdiv(hi[2], lb); ++z)
                            for (int y = fdiv(lo[1], lb); ok && y <= fdiv(hi[1], lb); ++y)
                                for (int x = fdiv(lo[0], lb); ok && x <= fdiv(hi[0], lb); ++x)
                                    ok = cov[((size_t)pmod(z, nlb) * nlb + pmod(y, nlb)) * nlb +
                                             pmod(x, nlb)] != 0;
                        const size_t q = ((size_t)bk * nb + bj) * nb + bi;
                        allowed[q] = ok;
                        if (!ok) blk[q] = 0;
                    }
        }
        const int w = c.max_grid_size / bf; /* blocks per box side at most */
        const std::vector<IBox> bb = make_boxes(blk, allowed, nb, c.clustering, c.grid_eff, w);
        std::vector<IBox> out;
        out.reserve(bb.size());
        for (const IBox &r : bb)
            out.push_back(IBox{{r.lo[0] * bf, r.lo[1] * bf, r.lo[2] * bf},
                               {(r.hi[0] + 1) * bf - 1, (r.hi[1] + 1) * bf - 1,
                                (r.hi[2] + 1) * bf - 1}});
        return out;
    }

    /* AmrCore::regrid(lbase, time) with the grids above. */
    void regrid(int lbase, double time) {
        const int top = std::min(finest, c.max_level - 1);
        /* tags of every level on its current grids first (ErrorEst) */
        std::vector<Tags> tags(top + 1);
        std::vector<std::vector<IBox>> old_boxes = boxes;
        for (int l = lbase; l <= top; ++l) tags[l] = error_est(l, time);
        int new_finest = lbase;
        for (int l = lbase; l <= top; ++l) {
            std::vector<IBox> nb;
            if (!tags[l].blocks.empty()) {
                Clock ck(this, kTGrids);
                nb = new_grids(l, std::move(tags[l].blocks), boxes[l]);
            }
            if (record_regrids) {
                RegridRecord rr;
                rr.lev = l;
                rr.time = time;
                rr.boxes_tagged_level = old_boxes[l];
                rr.mask = tags[l].mask;
                rr.new_boxes = nb;
                regrids.push_back(rr);
            }
            if (nb.empty()) break;
            const int f = l + 1;
            {
                Clock ck(this, kTRefresh);
                b.refresh_ghosts(levels[l], kNew, l > 0 ? &levels[l - 1] : nullptr);
            }
            if (f <= finest) {
                /* RemakeLevel: fill the new layout from the old one and the
                 * coarse level; the old time level is redefined, times kept */
                const double tn = b.time(levels[f], kNew), to = b.time(levels[f], kOld);
                const int sn = b.istep(levels[f], kNew), so = b.istep(levels[f], kOld);
                Level fresh;
                {
                    Clock ck(this, kTCreate);
                    fresh = b.create(f, nb, dimN[f]);
                }
                {
                    Clock ck(this, kTFill);
                    b.remake(fresh, levels[f], levels[l], time);
                }
                {
                    Clock ck(this, kTDestroy);
                    b.destroy(levels[f]);
                }
                levels[f] = fresh;
                b.set_time(levels[f], kNew, tn, sn);
                b.set_time(levels[f], kOld, to, so);
            } else {
                /* MakeNewLevelFromCoarse */
                Level fresh;
                {
                    Clock ck(this, kTCreate);
                    fresh = b.create(f, nb, dimN[f]);
                }
                {
                    Clock ck(this, kTFill);
                    b.fill_from_coarse(fresh, levels[l], time);
                }
                levels[f] = fresh;
                b.set_time(levels[f], kNew, time, 0);
                b.set_time(levels[f], kOld, -DBL_MAX, 0);
            }
            boxes[f] = nb;
            te_valid[f] = false;
            new_finest = f;
            if (f > finest) break; /* at most one new level per regrid */
        }
        /* ClearLevel for the levels above the new finest */
        for (int l = finest; l > new_finest; --l) {
            b.destroy(levels[l]);
            levels[l] = Level{};
            boxes[l].clear();
        }
        finest = new_finest;
    }
};

} // namespace shamr

#endif
