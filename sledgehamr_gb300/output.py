"""Output files in sledgehamr's formats, readable by pySledgehamr.Output.

sledgehamr's output types (source/io_module.cpp:50-100) write HDF5 files of
one-dimensional datasets under <output_folder>/<name>/<id>/
(output_module.cpp:79-85).  This module writes the same files through the
library's HDF5 writer (sh_h5_*, sh_output_* in include/sledgehamr_gb300.h):

  write_boxes        coarse_box / full_box (+ _truncation_error):
                     LevelWriter::Write (output_types/level_writer.cpp:96-124)
  write_slices       slices (+ _truncation_error): Slices::Write
                     (output_types/slices.cpp:13-45)
  write_spectra      spectra: Spectrum::Compute's datasets
                     (output_types/spectrum.cpp:103-111)
  write_gw_spectrum  gw_spectra: GravitationalWaves::ComputeSpectrum's
                     datasets (gravitational_waves.cpp:313-320)
  write_projections  projections: Projection::Compute's datasets
                     (output_types/projection.cpp:76-86)

The spectra, GW spectra and projections themselves come from
Level.scalar_spectrum / Level.gw_spectrum / projection.
"""
from __future__ import annotations

import ctypes as C
import os
from typing import Mapping, Sequence

import numpy as np

from . import _lib
from ._lib import ShBox

SH_H5_F32 = 4
SH_H5_F64 = 8
SH_H5_I32 = -4
SH_H5_I64 = -8

_TYPES = {np.dtype(np.float32): SH_H5_F32, np.dtype(np.float64): SH_H5_F64,
          np.dtype(np.int32): SH_H5_I32, np.dtype(np.int64): SH_H5_I64}


class H5Error(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"sledgehamr_gb300 output error {code}: {msg}")
        self.code = code


class H5File:
    """Datasets collected for one HDF5 file (sh_h5file)."""

    def __init__(self):
        self.lib = _lib.load()
        h = C.c_void_p()
        rc = self.lib.sh_h5_create(C.byref(h))
        if rc != 0:
            raise H5Error(rc, "sh_h5_create")
        self.h = h

    def check(self, rc: int, what: str):
        if rc != 0:
            raise H5Error(rc, f"{what}: {self.lib.sh_h5_last_error(self.h).decode()}")

    def add(self, name: str, data) -> None:
        """float32 / float64 data keep their type; int32 / int64 are stored
        as float64, as sledgehamr stores integers."""
        a = np.ascontiguousarray(data)
        if a.dtype not in _TYPES:
            a = a.astype(np.float64)
        self.check(self.lib.sh_h5_add(self.h, name.encode(), _TYPES[a.dtype],
                                      C.c_void_p(a.ctypes.data), a.size), f"add {name}")

    def __len__(self) -> int:
        n = C.c_longlong()
        self.lib.sh_h5_count(self.h, C.byref(n))
        return n.value

    def write(self, path: str) -> None:
        self.check(self.lib.sh_h5_write(self.h, os.fsencode(path)), f"write {path}")

    def close(self):
        if getattr(self, "h", None):
            self.lib.sh_h5_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def comp_names(project: str, with_gw: bool = False) -> list[str]:
    """Component names of a level of the project (GetScalarFieldName)."""
    from . import project_id, project_ncomp
    lib = _lib.load()
    pid = project_id(project)
    nc, _ = project_ncomp(project, with_gw)
    out = []
    for c in range(nc):
        s = C.c_char_p()
        rc = lib.sh_project_comp_name(pid, c, C.byref(s))
        if rc != 0:
            raise H5Error(rc, f"no name for component {c} of {project}")
        out.append(s.value.decode())
    return out


def output_folder(prefix: str, name: str, output_id: int) -> str:
    """<prefix>/<name>/<id>/ (OutputModule::Write), created if missing;
    files written there replace files of the same name."""
    folder = os.path.join(prefix, name, str(output_id))
    os.makedirs(folder, exist_ok=True)
    return folder


def _handle(level):
    return level.h


def level_file(ctx, level, finest_level: int, truncation_error: bool = False,
               downsample: int = 1, precision: int = 32) -> H5File:
    """The datasets of one level's file: "data" from time level NEW and, with
    truncation_error, "te" from the errors in time level OLD."""
    f = H5File()
    f.check(ctx.lib.sh_output_level(ctx.h, _handle(level), 0, finest_level, downsample,
                                    precision, f.h), "level data")
    if truncation_error:
        f.check(ctx.lib.sh_output_level(ctx.h, _handle(level), 1, finest_level, downsample,
                                        precision, f.h), "level truncation errors")
    return f


def slices_file(ctx, level, finest_level: int, truncation_error: bool = False,
                location: Sequence[float] = (0., 0., 0.)) -> H5File:
    f = H5File()
    loc = (C.c_double * 3)(*location)
    f.check(ctx.lib.sh_output_slices(ctx.h, _handle(level), 0, finest_level, loc, f.h),
            "slices")
    if truncation_error:
        f.check(ctx.lib.sh_output_slices(ctx.h, _handle(level), 1, finest_level, loc, f.h),
                "truncation-error slices")
    return f


def write_boxes(folder: str, ctx, levels: Sequence, truncation_error: bool = False,
                downsample: int = 1, precision: int = 32) -> list[str]:
    """<folder>/Level_<lev>/0.hdf5 for levels[0..] (coarse_box: the coarse
    level alone; full_box: every level)."""
    paths = []
    for lev, level in enumerate(levels):
        sub = os.path.join(folder, f"Level_{lev}")
        os.makedirs(sub, exist_ok=True)
        p = os.path.join(sub, "0.hdf5")
        level_file(ctx, level, len(levels) - 1, truncation_error, downsample,
                   precision).write(p)
        paths.append(p)
    return paths


def write_slices(folder: str, ctx, levels: Sequence, truncation_error: bool = False,
                 location: Sequence[float] = (0., 0., 0.), finest_level: int | None = None,
                 first_level: int = 0) -> list[str]:
    """<folder>/Level_<lev>/0.hdf5 with the x, y and z slices of each level
    (levels[q] is level first_level + q; sledgehamr skips levels without
    truncation errors for the truncation-error slices)."""
    finest = len(levels) - 1 + first_level if finest_level is None else finest_level
    paths = []
    for q, level in enumerate(levels):
        sub = os.path.join(folder, f"Level_{first_level + q}")
        os.makedirs(sub, exist_ok=True)
        p = os.path.join(sub, "0.hdf5")
        slices_file(ctx, level, finest, truncation_error, location).write(p)
        paths.append(p)
    return paths


def write_spectra(path: str, t: float, dim_n: int, k_sq, spectra: Mapping[str, np.ndarray]):
    """spectra.hdf5: Header {t, N, kmax}, k_sq, one dataset per spectrum."""
    f = H5File()
    k_sq = np.asarray(k_sq)
    f.add("Header", np.array([t, dim_n, k_sq.size], dtype=np.float64))
    f.add("k_sq", k_sq.astype(np.int64))
    for ident, bins in spectra.items():
        f.add(ident, np.asarray(bins, dtype=np.float64))
    f.write(path)


def write_gw_spectrum(path: str, t: float, dim_n: int, L: float, zero_padding: int,
                      unbinned: bool, ks, spectrum):
    """spectra.hdf5 of gw_spectra: Header {t, N, kmax, L, zero padding,
    unbinned}, k, Spectrum."""
    f = H5File()
    ks = np.asarray(ks)
    f.add("Header", np.array([t, dim_n, ks.size, L, zero_padding, int(unbinned)],
                             dtype=np.float64))
    f.add("k", ks.astype(np.int64))
    f.add("Spectrum", np.asarray(spectrum, dtype=np.float64))
    f.write(path)


def write_projections(path: str, t: float, dim_n: int,
                      projections: Mapping[str, tuple[np.ndarray, np.ndarray]]):
    """projections.hdf5: Header {t, N}, <ident>_data and <ident>_n
    (x slowest)."""
    f = H5File()
    f.add("Header", np.array([t, dim_n], dtype=np.float64))
    for ident, (data, n) in projections.items():
        f.add(ident + "_data", np.asarray(data, dtype=np.float64).reshape(-1))
        f.add(ident + "_n", np.asarray(n, dtype=np.int32).reshape(-1))
    f.write(path)


def level_datasets_host(boxes, cells: np.ndarray, names: Sequence[str], t: float,
                        finest_level: int, dim_n: int, truncation_error: bool = False,
                        downsample: int = 1, precision: int = 32) -> H5File:
    """The level datasets from host data (boxes layout), for callers that
    hold a level on the host."""
    f = H5File()
    arr, cells, cnames = _host_args(boxes, cells, names)
    f.check(f.lib.sh_output_level_host(arr, len(boxes), len(names), C.c_void_p(cells.ctypes.data),
                                       cnames, t, finest_level, dim_n, int(truncation_error),
                                       downsample, precision, f.h), "level data (host)")
    return f


def slices_datasets_host(boxes, cells: np.ndarray, names: Sequence[str], t: float,
                         finest_level: int, dim_n: int, truncation_error: bool = False,
                         location: Sequence[float] = (0., 0., 0.)) -> H5File:
    f = H5File()
    arr, cells, cnames = _host_args(boxes, cells, names)
    loc = (C.c_double * 3)(*location)
    f.check(f.lib.sh_output_slices_host(arr, len(boxes), len(names),
                                        C.c_void_p(cells.ctypes.data), cnames, t, finest_level,
                                        dim_n, int(truncation_error), loc, f.h),
            "slices (host)")
    return f


def _host_args(boxes, cells, names):
    arr = (ShBox * max(len(boxes), 1))()
    for q, (lo, hi) in enumerate(boxes):
        arr[q].lo[:] = list(lo)
        arr[q].hi[:] = list(hi)
    cells = np.ascontiguousarray(cells, dtype=np.float64)
    cnames = (C.c_char_p * len(names))(*[n.encode() for n in names])
    return arr, cells, cnames
