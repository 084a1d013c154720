"""Oracle for the level and slice output datasets (test infrastructure only).

A numpy restatement of sledgehamr's LevelWriter::WriteSingleLevel
(source/output_types/level_writer.h:80-171) and Slices::WriteSingleSlice
(source/output_types/slices.cpp:58-145), used by the tests to check the
library's writers (sh_output_level*, sh_output_slices*).  The per-cell loops
of the reference are replaced by strided array operations that keep, for
every output cell, the reference's order of contributions (k outer, then j,
then i) and its arithmetic: each contribution v / downsample^3 is added in
double precision to the value held in the output type and rounded back to
it; truncation errors keep max(value, held value) as std::max does.

Inputs are a level's valid cells in the boxes layout (per box, per
component, x fastest).  Returns {dataset name: numpy array} as the
reference writes them (float32 / float64 data, integers as float64).
"""
import numpy as np


def _box_arrays(boxes, cells, ncomp):
    """Per box a (ncomp, ex, ey, ez) array (x slowest) of its cells."""
    out = []
    base = 0
    for lo, hi in boxes:
        ex, ey, ez = (hi[d] - lo[d] + 1 for d in range(3))
        vol = ex * ey * ez
        a = np.asarray(cells[base:base + ncomp * vol]).reshape(ncomp, ez, ey, ex)
        out.append(a.transpose(0, 3, 2, 1))
        base += ncomp * vol
    return out


def level_datasets(boxes, cells, names, t, finest_level, dim_n, ident, te, downsample,
                   precision, ranks=1):
    T = np.float32 if precision == 32 else np.float64
    gd = downsample * (2 if te else 1)
    volfac = 1.0 / float(downsample) ** 3
    out = {}
    for b, ((lo, hi), a) in enumerate(zip(boxes, _box_arrays(boxes, cells, len(names)))):
        ext = [hi[d] - lo[d] + 1 for d in range(3)]
        dims = [e // gd for e in ext]
        for f, name in enumerate(names):
            o = np.zeros(dims, dtype=T)
            x = a[f]
            step = 2 if te else 1
            # offsets inside a block in the reference's k, j, i loop order
            for dk in range(0, gd, step):
                for dj in range(0, gd, step):
                    for di in range(0, gd, step):
                        v = x[di::gd, dj::gd, dk::gd]
                        if te:
                            c = v.astype(T)
                            o = np.where(c < o, o, c)
                        else:
                            o = (o.astype(np.float64) + v * volfac).astype(T)
            out[f"{name}_{ident}_{b + 1}"] = o.reshape(-1)
    out[f"Header_{ident}"] = np.array([t, ranks, finest_level, dim_n, downsample, len(boxes)],
                                      dtype=np.float64)
    if boxes:
        for d, ax in enumerate("xyz"):
            out[f"le{ax}_{ident}"] = np.array([lo[d] for lo, _ in boxes], dtype=np.float64)
        for d, ax in enumerate("xyz"):
            out[f"he{ax}_{ident}"] = np.array([hi[d] + 1 for _, hi in boxes], dtype=np.float64)
    return out


def slice_datasets(boxes, cells, names, t, finest_level, dim_n, ident, d1, d2, d3, te,
                   location, ranks=1):
    s = int(float(dim_n) * location[d1])
    if s % 2 == 1:
        s += 1
    step = 2 if te else 1
    out = {}
    le1, le2, he1, he2 = [], [], [], []
    for (lo, hi), a in zip(boxes, _box_arrays(boxes, cells, len(names))):
        if not (lo[d1] <= s <= hi[d1]):
            continue
        le1.append(lo[d2])
        le2.append(lo[d3])
        he1.append(hi[d2] + 1)
        he2.append(hi[d3] + 1)
        for f, name in enumerate(names):
            # the plane keeps the other two axes in increasing order
            plane = np.take(a[f], s - lo[d1], axis=d1)
            if d2 > d3:
                plane = plane.T
            o = plane[::step, ::step].astype(np.float32)
            out[f"{name}_{ident}_{len(le1)}"] = o.reshape(-1)
    out[f"Header_{ident}"] = np.array([t, ranks, finest_level, dim_n, len(le1)],
                                      dtype=np.float64)
    if le1:
        out[f"le1_{ident}"] = np.array(le1, dtype=np.float64)
        out[f"le2_{ident}"] = np.array(le2, dtype=np.float64)
        out[f"he1_{ident}"] = np.array(he1, dtype=np.float64)
        out[f"he2_{ident}"] = np.array(he2, dtype=np.float64)
    return out


def slices_datasets(boxes, cells, names, t, finest_level, dim_n, te, location):
    p = "te_" if te else ""
    out = {}
    for ident, d1, d2, d3 in ((p + "x", 0, 1, 2), (p + "y", 1, 0, 2), (p + "z", 2, 0, 1)):
        out.update(slice_datasets(boxes, cells, names, t, finest_level, dim_n, ident, d1, d2,
                                  d3, te, location))
    return out
