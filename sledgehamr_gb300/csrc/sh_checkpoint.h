/* Checkpoint files of an AMR hierarchy (shamr::Checkpoint), host only and
 * free of CUDA, shared by the library and the oracle.
 *
 * A checkpoint is a folder, as the reference's Checkpoint::Write makes one
 * (source/output_types/checkpoint.cpp:18-98, names from checkpoint.h:37-52):
 *   Meta.hdf5   the reference's header datasets, written as its
 *               utils::hdf5::Write does (integers stored as F64):
 *                 Header[8] = {t of level 0, MPI ranks (1), finest level,
 *                              coarse cells per side, nghost, components,
 *                              outputs (1), index of the checkpoint output (0)}
 *                 blocking_factors[finest+1], isteps[finest+1],
 *                 next_id[1], last_time_written[1]
 *               and this library's datasets needed to continue exactly:
 *                 sh_format[1] (1), sh_boxes_<l>[6 per box] (lo, hi),
 *                 sh_times_<l>[4] (t_new, t_old, istep_new, istep_old),
 *                 sh_last_regrid_time[max_level+1], sh_schedule[2 per entry]
 *                 (lowest level, time), sh_te_valid[max_level+1],
 *                 sh_cell_updates[1], sh_grid[3] (max_level, blocking factor,
 *                 components), sh_local_regrid (attempts, the sizes and
 *                 contents of the per-level no-local and global-requested
 *                 flags and of the cells at the last global regrid);
 *   Level_<l>_new.bin, Level_<l>_old.bin
 *               the valid cells of both time levels of level l as raw FP64
 *               (little endian), box after box, component-major inside a
 *               box, x fastest.  The reference stores grid_new with ghost
 *               cells in AMReX's VisMF format (Level_<l>/Cell), which needs
 *               AMReX to read; these files hold the same values of the valid
 *               cells in a plain layout.
 */
#ifndef SH_CHECKPOINT_H_
#define SH_CHECKPOINT_H_

#include <sys/stat.h>

#include <cerrno>
#include <cstdio>
#include <string>
#include <vector>

#include "sh_amr_driver.h"
#include "sh_hdf5.h"

namespace shamr {

inline bool ck_fail(std::string *err, const std::string &m) {
    if (err) *err = m;
    return false;
}

inline bool write_raw(const std::string &path, const std::vector<double> &v, std::string *err) {
    FILE *f = std::fopen(path.c_str(), "wb");
    if (!f) return ck_fail(err, "cannot create " + path);
    bool ok = v.empty() || std::fwrite(v.data(), sizeof(double), v.size(), f) == v.size();
    ok = (std::fclose(f) == 0) && ok;
    return ok ? true : ck_fail(err, "write to " + path + " failed");
}

inline bool read_raw(const std::string &path, size_t n, std::vector<double> *v,
                     std::string *err) {
    FILE *f = std::fopen(path.c_str(), "rb");
    if (!f) return ck_fail(err, "cannot open " + path);
    v->assign(n, 0.);
    bool ok = n == 0 || std::fread(v->data(), sizeof(double), n, f) == n;
    const bool at_end = std::fgetc(f) == EOF;
    std::fclose(f);
    if (!ok || !at_end) return ck_fail(err, path + ": size does not match its boxes");
    return true;
}

inline bool write_checkpoint(const Checkpoint &k, const std::string &folder, std::string *err) {
    if (!sh::h5::little_endian_host()) return ck_fail(err, "checkpoints need a little-endian host");
    if (::mkdir(folder.c_str(), 0777) != 0 && errno != EEXIST)
        return ck_fail(err, "cannot create folder " + folder);
    sh::h5::Writer w;
    const int nl = k.finest + 1;
    const double t0 = nl > 0 ? k.levels[0].t_new : 0.;
    const double header[8] = {t0, 1., (double)k.finest, (double)k.N0, (double)k.nghost,
                              (double)k.ncomp, 1., 0.};
    std::vector<double> bf(nl, (double)k.blocking_factor), isteps(nl);
    for (int l = 0; l < nl; ++l) isteps[l] = k.levels[l].s_new;
    const double next_id = 1., last = t0, format = 1.;
    bool ok = w.add_f64("Header", header, 8, err) && w.add_f64("blocking_factors", bf.data(), nl, err) &&
              w.add_f64("isteps", isteps.data(), nl, err) && w.add_f64("next_id", &next_id, 1, err) &&
              w.add_f64("last_time_written", &last, 1, err) && w.add_f64("sh_format", &format, 1, err);
    for (int l = 0; ok && l < nl; ++l) {
        const LevelState &s = k.levels[l];
        std::vector<double> bx;
        for (const IBox &b : s.boxes)
            for (int q = 0; q < 6; ++q) bx.push_back(q < 3 ? b.lo[q] : b.hi[q - 3]);
        const double times[4] = {s.t_new, s.t_old, (double)s.s_new, (double)s.s_old};
        ok = w.add_f64("sh_boxes_" + std::to_string(l), bx.data(), bx.size(), err) &&
             w.add_f64("sh_times_" + std::to_string(l), times, 4, err);
    }
    std::vector<double> sched, tev;
    for (const auto &q : k.schedule) {
        sched.push_back(q.first);
        sched.push_back(q.second);
    }
    for (uint8_t v : k.te_valid) tev.push_back(v);
    const double cu = (double)k.cell_updates;
    const double grid[3] = {(double)k.max_level, (double)k.blocking_factor, (double)k.ncomp};
    /* local regrid state: attempts, then per level no-local, global
     * requested, cells at the last global regrid */
    std::vector<double> lr = {(double)k.lr_nregrids, (double)k.lr_no_local.size(),
                              (double)k.lr_do_global.size(), (double)k.lr_last_numpts.size()};
    for (uint8_t v : k.lr_no_local) lr.push_back(v);
    for (uint8_t v : k.lr_do_global) lr.push_back(v);
    for (long long v : k.lr_last_numpts) lr.push_back((double)v);
    ok = ok && w.add_f64("sh_local_regrid", lr.data(), lr.size(), err) &&
         w.add_f64("sh_last_regrid_time", k.last_regrid_time.data(), k.last_regrid_time.size(),
                   err) &&
         w.add_f64("sh_schedule", sched.data(), sched.size(), err) &&
         w.add_f64("sh_te_valid", tev.data(), tev.size(), err) &&
         w.add_f64("sh_cell_updates", &cu, 1, err) && w.add_f64("sh_grid", grid, 3, err) &&
         w.write(folder + "/Meta.hdf5", err);
    for (int l = 0; ok && l < nl; ++l)
        ok = write_raw(folder + "/Level_" + std::to_string(l) + "_new.bin", k.levels[l].data_new,
                       err) &&
             write_raw(folder + "/Level_" + std::to_string(l) + "_old.bin", k.levels[l].data_old,
                       err);
    return ok;
}

inline bool read_checkpoint(const std::string &folder, Checkpoint *k, std::string *err) {
    sh::h5::Reader r;
    if (!r.open(folder + "/Meta.hdf5", err)) return false;
    std::vector<double> header, isteps, fmt, grid, lrt, sched, tev, cu;
    if (!r.get("Header", &header, err) || !r.get("isteps", &isteps, err) ||
        !r.get("sh_format", &fmt, err) || !r.get("sh_grid", &grid, err) ||
        !r.get("sh_last_regrid_time", &lrt, err) || !r.get("sh_schedule", &sched, err) ||
        !r.get("sh_te_valid", &tev, err) || !r.get("sh_cell_updates", &cu, err))
        return false;
    if (header.size() != 8 || fmt.size() != 1 || fmt[0] != 1. || grid.size() != 3 ||
        cu.size() != 1 || sched.size() % 2 != 0)
        return ck_fail(err, folder + ": not a checkpoint of this library's format");
    k->finest = (int)header[2];
    k->N0 = (int)header[3];
    k->nghost = (int)header[4];
    k->ncomp = (int)header[5];
    k->max_level = (int)grid[0];
    k->blocking_factor = (int)grid[1];
    if (k->finest < 0 || k->finest > k->max_level || (int)isteps.size() != k->finest + 1 ||
        k->ncomp <= 0)
        return ck_fail(err, folder + ": inconsistent checkpoint header");
    k->last_regrid_time = lrt;
    k->schedule.clear();
    for (size_t q = 0; q < sched.size(); q += 2) k->schedule.push_back({(int)sched[q], sched[q + 1]});
    k->te_valid.assign(tev.begin(), tev.end());
    k->cell_updates = (long long)cu[0];
    std::vector<double> lr;
    if (!r.get("sh_local_regrid", &lr, err)) return false;
    if (lr.size() < 4 || lr.size() != 4 + (size_t)lr[1] + (size_t)lr[2] + (size_t)lr[3])
        return ck_fail(err, folder + ": bad local regrid state");
    k->lr_nregrids = (int)lr[0];
    size_t q = 4;
    k->lr_no_local.assign(lr.begin() + q, lr.begin() + q + (size_t)lr[1]);
    q += (size_t)lr[1];
    k->lr_do_global.assign(lr.begin() + q, lr.begin() + q + (size_t)lr[2]);
    q += (size_t)lr[2];
    k->lr_last_numpts.clear();
    for (size_t e = 0; e < (size_t)lr[3]; ++e) k->lr_last_numpts.push_back((long long)lr[q + e]);
    k->levels.assign(k->finest + 1, LevelState());
    for (int l = 0; l <= k->finest; ++l) {
        LevelState &s = k->levels[l];
        std::vector<double> bx, times;
        if (!r.get("sh_boxes_" + std::to_string(l), &bx, err) ||
            !r.get("sh_times_" + std::to_string(l), &times, err))
            return false;
        if (bx.size() % 6 != 0 || times.size() != 4)
            return ck_fail(err, folder + ": bad boxes or times of level " + std::to_string(l));
        long long cells = 0;
        for (size_t q = 0; q < bx.size(); q += 6) {
            IBox b{{(int)bx[q], (int)bx[q + 1], (int)bx[q + 2]},
                   {(int)bx[q + 3], (int)bx[q + 4], (int)bx[q + 5]}};
            if (b.hi[0] < b.lo[0] || b.hi[1] < b.lo[1] || b.hi[2] < b.lo[2])
                return ck_fail(err, folder + ": empty box");
            cells += b.volume();
            s.boxes.push_back(b);
        }
        s.t_new = times[0];
        s.t_old = times[1];
        s.s_new = (int)times[2];
        s.s_old = (int)times[3];
        const size_t n = (size_t)cells * k->ncomp;
        if (!read_raw(folder + "/Level_" + std::to_string(l) + "_new.bin", n, &s.data_new, err) ||
            !read_raw(folder + "/Level_" + std::to_string(l) + "_old.bin", n, &s.data_old, err))
            return false;
    }
    return true;
}

} // namespace shamr

#endif // SH_CHECKPOINT_H_
