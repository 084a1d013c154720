/* Output files in sledgehamr's formats: an HDF5 file builder and the level
 * and slice writers on top of it (sh_hdf5.h, sh_output.h).  Host code; the
 * level variants read the level's valid cells through sh_level_read. */
#include <new>
#include <string>
#include <vector>

#include "sh_hdf5.h"
#include "sh_output.h"
#include "sledgehamr_gb300.h"

struct sh_h5file {
    sh::h5::Writer w;
    std::string err;
};

namespace {

/* bad_alloc and other exceptions of the host containers become a status */
template <typename F>
int guarded(sh_h5file *f, F &&fn) {
    try {
        return fn();
    } catch (const std::bad_alloc &) {
        f->err = "out of host memory";
        return SH_ERR_NOMEM;
    } catch (const std::exception &e) {
        f->err = e.what();
        return SH_ERR_ARG;
    }
}

/* A device level's valid cells, component names and time on the host. */
struct Downloaded {
    std::vector<sh_box> boxes;
    std::vector<double> cells;
    std::vector<const char *> names;
    double t = 0.;
    int dim_n = 0;
};

int download(sh_ctx *ctx, const sh_level *L, int which, Downloaded &d, std::string *err) {
    int ncomp = 0, nbox = 0, project = -1, with_gw = 0;
    long long nvalid = 0;
    int rc = sh_level_info(L, &ncomp, &nbox, &nvalid);
    if (rc == SH_OK) rc = sh_level_project(L, &project, &with_gw);
    if (rc != SH_OK) return rc;
    d.boxes.resize(nbox);
    int got = 0;
    rc = sh_level_boxes(L, d.boxes.data(), nbox, &got);
    if (rc != SH_OK) return rc;
    int lo[3], hi[3];
    rc = sh_level_domain(L, lo, hi);
    if (rc != SH_OK) return rc;
    d.dim_n = hi[0] - lo[0] + 1;
    int istep = 0;
    rc = sh_level_time(L, which, &d.t, &istep);
    if (rc != SH_OK) return rc;
    d.names.resize(ncomp);
    for (int c = 0; c < ncomp; ++c) {
        rc = sh_project_comp_name(project, c, &d.names[c]);
        if (rc != SH_OK) {
            *err = "no name for component " + std::to_string(c);
            return rc;
        }
    }
    d.cells.resize((size_t)nvalid * ncomp);
    rc = sh_level_read(ctx, L, which, 1, d.cells.data());
    if (rc != SH_OK) *err = sh_ctx_last_error(ctx);
    return rc;
}

sh::out::HostLevel host_level(const sh_box *boxes, int nbox, int ncomp, const double *cells,
                              const char *const *names, double t, int finest, int dim_n) {
    sh::out::HostLevel L;
    L.boxes = boxes;
    L.nbox = nbox;
    L.ncomp = ncomp;
    L.cells = cells;
    L.names = names;
    L.t = t;
    L.finest_level = finest;
    L.dim_n = dim_n;
    return L;
}

} // namespace

extern "C" {

int sh_h5_create(sh_h5file **out) {
    if (!out) return SH_ERR_ARG;
    *out = new (std::nothrow) sh_h5file();
    return *out ? SH_OK : SH_ERR_NOMEM;
}

int sh_h5_destroy(sh_h5file *f) {
    delete f;
    return SH_OK;
}

const char *sh_h5_last_error(const sh_h5file *f) { return f ? f->err.c_str() : ""; }

int sh_h5_count(const sh_h5file *f, long long *n) {
    if (!f || !n) return SH_ERR_ARG;
    *n = (long long)f->w.size();
    return SH_OK;
}

int sh_h5_add(sh_h5file *f, const char *name, int type, const void *data, long long n) {
    if (!f) return SH_ERR_ARG;
    if (!name || n < 0 || (n > 0 && !data)) {
        f->err = "sh_h5_add: invalid arguments";
        return SH_ERR_ARG;
    }
    return guarded(f, [&] {
        bool ok = false;
        switch (type) {
        case SH_H5_F32:
            ok = f->w.add_f32(name, static_cast<const float *>(data), (uint64_t)n, &f->err);
            break;
        case SH_H5_F64:
            ok = f->w.add_f64(name, static_cast<const double *>(data), (uint64_t)n, &f->err);
            break;
        case SH_H5_I32:
            ok = f->w.add_int_as_f64(name, static_cast<const int32_t *>(data), (uint64_t)n,
                                     &f->err);
            break;
        case SH_H5_I64:
            ok = f->w.add_int_as_f64(name, static_cast<const int64_t *>(data), (uint64_t)n,
                                     &f->err);
            break;
        default:
            f->err = "sh_h5_add: unknown type";
        }
        return ok ? SH_OK : SH_ERR_ARG;
    });
}

int sh_h5_write(sh_h5file *f, const char *path) {
    if (!f) return SH_ERR_ARG;
    if (!path) {
        f->err = "sh_h5_write: no path";
        return SH_ERR_ARG;
    }
    return guarded(f, [&] { return f->w.write(path, &f->err) ? SH_OK : SH_ERR_ARG; });
}

int sh_output_level_host(const sh_box *boxes, int nbox, int ncomp, const double *cells,
                         const char *const *names, double t, int finest_level, int dim_n,
                         int truncation_error, int downsample, int precision, sh_h5file *f) {
    if (!f) return SH_ERR_ARG;
    return guarded(f, [&] {
        const auto L = host_level(boxes, nbox, ncomp, cells, names, t, finest_level, dim_n);
        const bool te = truncation_error != 0;
        return sh::out::level_datasets(f->w, L, te ? "te" : "data", te, downsample, precision,
                                       &f->err)
                   ? SH_OK
                   : SH_ERR_ARG;
    });
}

int sh_output_slices_host(const sh_box *boxes, int nbox, int ncomp, const double *cells,
                          const char *const *names, double t, int finest_level, int dim_n,
                          int truncation_error, const double location[3], sh_h5file *f) {
    if (!f) return SH_ERR_ARG;
    if (!location) {
        f->err = "slice output: no location";
        return SH_ERR_ARG;
    }
    return guarded(f, [&] {
        const auto L = host_level(boxes, nbox, ncomp, cells, names, t, finest_level, dim_n);
        return sh::out::slices_datasets(f->w, L, truncation_error != 0, location, &f->err)
                   ? SH_OK
                   : SH_ERR_ARG;
    });
}

int sh_output_level(sh_ctx *ctx, const sh_level *level, int truncation_error, int finest_level,
                    int downsample, int precision, sh_h5file *f) {
    if (!ctx || !level || !f) return SH_ERR_ARG;
    return guarded(f, [&] {
        Downloaded d;
        const int rc = download(ctx, level, truncation_error ? SH_OLD : SH_NEW, d, &f->err);
        if (rc != SH_OK) return rc;
        return sh_output_level_host(d.boxes.data(), (int)d.boxes.size(), (int)d.names.size(),
                                    d.cells.data(), d.names.data(), d.t, finest_level, d.dim_n,
                                    truncation_error, downsample, precision, f);
    });
}

int sh_output_slices(sh_ctx *ctx, const sh_level *level, int truncation_error,
                     int finest_level, const double location[3], sh_h5file *f) {
    if (!ctx || !level || !f) return SH_ERR_ARG;
    return guarded(f, [&] {
        Downloaded d;
        const int rc = download(ctx, level, truncation_error ? SH_OLD : SH_NEW, d, &f->err);
        if (rc != SH_OK) return rc;
        return sh_output_slices_host(d.boxes.data(), (int)d.boxes.size(), (int)d.names.size(),
                                     d.cells.data(), d.names.data(), d.t, finest_level,
                                     d.dim_n, truncation_error, location, f);
    });
}

} // extern "C"
