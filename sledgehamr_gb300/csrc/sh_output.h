/* The datasets of sledgehamr's level and slice output files, assembled on
 * the host from a level's valid cells.
 *
 * Input: the level's boxes in order and its valid cells in the boxes layout
 * of sh_level_read (per box, per component, x fastest), as MFIter visits
 * the boxes of a single-rank level.
 *
 * level_datasets follows LevelWriter::WriteSingleLevel
 * (source/output_types/level_writer.h:80-171): per box b (1-based count)
 * and component f a dataset "<field>_<ident>_<b>" of the box's cells,
 * x slowest and z fastest, averaged over downsample^3 blocks in the output
 * precision (each cell's value times 1/downsample^3 added in double and
 * stored back in the output type, in the reference's k, j, i order); for
 * truncation errors (ident "te") only cells with all-even indices count and
 * each output cell holds the maximum of its cells and zero.  Then
 * "Header_<ident>" = {t, ranks, finest level, N, downsample, boxes} and,
 * if there are boxes, their bounds "lex_", "ley_", "lez_" (lower) and
 * "hex_", "hey_", "hez_" (upper, exclusive), stored as F64.
 *
 * slice_datasets follows Slices::WriteSingleSlice
 * (source/output_types/slices.cpp:58-145): the plane at index
 * floor(N * location[d1]) (rounded up to even) along d1, per box cutting
 * it and component a dataset "<field>_<ident>_<b>" of 32-bit floats, d2
 * slowest and d3 fastest (even cells only, halved, for truncation errors),
 * then "Header_<ident>" = {t, ranks, finest level, N, boxes} and the
 * bounds "le1_", "le2_", "he1_", "he2_".
 *
 * The reference leaves downsample factors that do not divide a box
 * undefined (level_writer.h:68-86 only bounds them by the blocking
 * factor); here they are rejected.  Host only, free of CUDA.
 */
#ifndef SH_OUTPUT_H_
#define SH_OUTPUT_H_

#include <new>
#include <string>
#include <vector>

#include "sh_hdf5.h"
#include "sledgehamr_gb300.h"

namespace sh {
namespace out {

/* A level's valid cells on the host. */
struct HostLevel {
    const sh_box *boxes = nullptr;
    int nbox = 0;
    int ncomp = 0;
    const double *cells = nullptr;           /* boxes layout */
    const char *const *names = nullptr;      /* ncomp component names */
    double t = 0.;
    int finest_level = 0;
    int dim_n = 0;                           /* cells per side of the level's domain */
    int ranks = 1;
};

inline long long box_cells(const sh_box &b) {
    return (long long)(b.hi[0] - b.lo[0] + 1) * (b.hi[1] - b.lo[1] + 1) *
           (b.hi[2] - b.lo[2] + 1);
}

inline bool check_level(const HostLevel &L, std::string *err) {
    if (L.nbox < 0 || L.ncomp < 1 || (L.nbox > 0 && (!L.boxes || !L.cells)) || !L.names) {
        *err = "level output: invalid level description";
        return false;
    }
    for (int f = 0; f < L.ncomp; ++f)
        if (!L.names[f] || !h5::valid_name(L.names[f])) {
            *err = "level output: invalid component name";
            return false;
        }
    for (int b = 0; b < L.nbox; ++b)
        for (int d = 0; d < 3; ++d)
            if (L.boxes[b].hi[d] < L.boxes[b].lo[d]) {
                *err = "level output: empty box";
                return false;
            }
    return true;
}

template <typename T>
bool level_datasets_t(h5::Writer &w, const HostLevel &L, const std::string &ident, bool te,
                      int downsample, std::string *err) {
    const int ndist = te ? 2 : 1;
    const int gd = downsample * ndist;
    const double volfac = 1. / ((double)downsample * downsample * downsample);
    std::vector<double> lo[3], hi[3];
    std::vector<long long> base(L.nbox + 1, 0);
    for (int b = 0; b < L.nbox; ++b) {
        const sh_box &bx = L.boxes[b];
        for (int d = 0; d < 3; ++d) {
            const int ext = bx.hi[d] - bx.lo[d] + 1;
            if (ext % gd != 0 || (te && bx.lo[d] % 2 != 0)) {
                *err = "level output: box " + std::to_string(b) +
                       " is not a multiple of the downsample factor" +
                       (te ? " times 2 at even offsets" : "");
                return false;
            }
            lo[d].push_back(bx.lo[d]);
            hi[d].push_back(bx.hi[d] + 1);
        }
        base[b + 1] = base[b] + box_cells(bx) * L.ncomp;
    }
    /* every (box, component) dataset independently on the host threads,
     * then added in the reference's order */
    const long long nset = (long long)L.nbox * L.ncomp;
    std::vector<std::vector<unsigned char>> bytes(nset);
    /* an exception must not leave the OpenMP region (std::terminate): an
     * allocation failure on a host thread is recorded and rethrown after it,
     * so the entry point still returns SH_ERR_NOMEM */
    bool out_of_memory = false;
#pragma omp parallel for schedule(dynamic, 1)
    for (long long q = 0; q < nset; ++q) try {
        const int b = (int)(q / L.ncomp), f = (int)(q % L.ncomp);
        const sh_box &bx = L.boxes[b];
        const int ext[3] = {bx.hi[0] - bx.lo[0] + 1, bx.hi[1] - bx.lo[1] + 1,
                            bx.hi[2] - bx.lo[2] + 1};
        const int dy = ext[1] / gd, dz = ext[2] / gd;
        const long long len = (long long)(ext[0] / gd) * dy * dz;
        const double *src = L.cells + base[b] + (long long)f * box_cells(bx);
        std::vector<T> o((size_t)len, T(0));
        for (int k = 0; k < ext[2]; ++k)
            for (int j = 0; j < ext[1]; ++j)
                for (int i = 0; i < ext[0]; ++i) {
                    const int gi = bx.lo[0] + i, gj = bx.lo[1] + j, gk = bx.lo[2] + k;
                    if (te && (gi % 2 != 0 || gj % 2 != 0 || gk % 2 != 0)) continue;
                    const long long ind =
                        (long long)(i / gd) * dy * dz + (long long)(j / gd) * dz + k / gd;
                    const double v = src[i + (long long)ext[0] * (j + (long long)ext[1] * k)];
                    if (te) {
                        const T c = static_cast<T>(v);
                        o[ind] = c < o[ind] ? o[ind] : c; /* std::max(c, o) */
                    } else {
                        o[ind] = static_cast<T>(o[ind] + v * volfac);
                    }
                }
        bytes[q].resize(sizeof(T) * (size_t)len);
        if (len) std::memcpy(bytes[q].data(), o.data(), bytes[q].size());
    } catch (const std::bad_alloc &) {
#pragma omp atomic write
        out_of_memory = true;
    }
    if (out_of_memory) throw std::bad_alloc();
    for (long long q = 0; q < nset; ++q) {
        const int b = (int)(q / L.ncomp), f = (int)(q % L.ncomp);
        const std::string name =
            std::string(L.names[f]) + "_" + ident + "_" + std::to_string(b + 1);
        const uint64_t len = bytes[q].size() / sizeof(T);
        if (!w.add_bytes(name, (int)sizeof(T), std::move(bytes[q]), len, err)) return false;
    }
    const double header[6] = {L.t, (double)L.ranks, (double)L.finest_level, (double)L.dim_n,
                              (double)downsample, (double)L.nbox};
    if (!w.add_f64("Header_" + ident, header, 6, err)) return false;
    if (L.nbox == 0) return true;
    static const char *const kAxis[3] = {"x", "y", "z"};
    for (int d = 0; d < 3; ++d)
        if (!w.add_f64(std::string("le") + kAxis[d] + "_" + ident, lo[d].data(), L.nbox, err))
            return false;
    for (int d = 0; d < 3; ++d)
        if (!w.add_f64(std::string("he") + kAxis[d] + "_" + ident, hi[d].data(), L.nbox, err))
            return false;
    return true;
}

/* precision 32 or 64 */
inline bool level_datasets(h5::Writer &w, const HostLevel &L, const std::string &ident,
                           bool te, int downsample, int precision, std::string *err) {
    if (!check_level(L, err)) return false;
    if (downsample < 1 || (downsample & (downsample - 1)) != 0) {
        *err = "level output: the downsample factor must be a power of 2";
        return false;
    }
    if (precision == 32) return level_datasets_t<float>(w, L, ident, te, downsample, err);
    if (precision == 64) return level_datasets_t<double>(w, L, ident, te, downsample, err);
    *err = "level output: precision must be 32 or 64";
    return false;
}

/* Slice through the plane normal to d1 with in-plane axes d2 (slow) and d3
 * (fast). */
inline bool slice_datasets(h5::Writer &w, const HostLevel &L, const std::string &ident,
                           int d1, int d2, int d3, bool te, const double location[3],
                           std::string *err) {
    if (!check_level(L, err)) return false;
    const int ndist = te ? 2 : 1;
    int s = static_cast<int>(static_cast<double>(L.dim_n) * location[d1]);
    if (s % 2 == 1) s++;
    std::vector<double> le1, le2, he1, he2;
    long long base = 0;
    for (int b = 0; b < L.nbox; ++b) {
        const sh_box &bx = L.boxes[b];
        const long long vol = box_cells(bx);
        const long long ext[3] = {bx.hi[0] - bx.lo[0] + 1, bx.hi[1] - bx.lo[1] + 1,
                                  bx.hi[2] - bx.lo[2] + 1};
        if (bx.lo[d1] <= s && bx.hi[d1] >= s) {
            const int l1 = bx.lo[d2], l2 = bx.lo[d3], h1 = bx.hi[d2] + 1, h2 = bx.hi[d3] + 1;
            if (te && ((h1 - l1) % 2 != 0 || (h2 - l2) % 2 != 0 || l1 % 2 != 0 || l2 % 2 != 0)) {
                *err = "slice output: truncation-error boxes must be even";
                return false;
            }
            le1.push_back(l1);
            le2.push_back(l2);
            he1.push_back(h1);
            he2.push_back(h2);
            const int dim1 = (h1 - l1) / ndist, dim2 = (h2 - l2) / ndist;
            const long long len = (long long)dim1 * dim2;
            std::vector<float> o((size_t)len, 0.f);
            for (int f = 0; f < L.ncomp; ++f) {
                const double *src = L.cells + base + (long long)f * vol;
                for (int j = l2; j < h2; ++j)
                    for (int i = l1; i < h1; ++i) {
                        if (te && (i % 2 != 0 || j % 2 != 0)) continue;
                        const long long ind =
                            (long long)((i - l1) / ndist) * dim2 + (j - l2) / ndist;
                        int c[3];
                        c[d1] = s;
                        c[d2] = i;
                        c[d3] = j;
                        const long long at = (c[0] - bx.lo[0]) +
                                             ext[0] * ((c[1] - bx.lo[1]) +
                                                       ext[1] * (long long)(c[2] - bx.lo[2]));
                        o[ind] = static_cast<float>(src[at]);
                    }
                const std::string name = std::string(L.names[f]) + "_" + ident + "_" +
                                         std::to_string(le1.size());
                if (!w.add_f32(name, o.data(), (uint64_t)len, err)) return false;
            }
        }
        base += vol * L.ncomp;
    }
    const double header[5] = {L.t, (double)L.ranks, (double)L.finest_level, (double)L.dim_n,
                              (double)le1.size()};
    if (!w.add_f64("Header_" + ident, header, 5, err)) return false;
    if (le1.empty()) return true;
    const uint64_t n = le1.size();
    return w.add_f64("le1_" + ident, le1.data(), n, err) &&
           w.add_f64("le2_" + ident, le2.data(), n, err) &&
           w.add_f64("he1_" + ident, he1.data(), n, err) &&
           w.add_f64("he2_" + ident, he2.data(), n, err);
}

/* The three slices of Slices::Write (slices.cpp:30-41): "x", "y", "z", or
 * "te_x", "te_y", "te_z" for truncation errors. */
inline bool slices_datasets(h5::Writer &w, const HostLevel &L, bool te, const double location[3],
                            std::string *err) {
    const std::string p = te ? "te_" : "";
    return slice_datasets(w, L, p + "x", 0, 1, 2, te, location, err) &&
           slice_datasets(w, L, p + "y", 1, 0, 2, te, location, err) &&
           slice_datasets(w, L, p + "z", 2, 0, 1, te, location, err);
}

} // namespace out
} // namespace sh

#endif // SH_OUTPUT_H_
