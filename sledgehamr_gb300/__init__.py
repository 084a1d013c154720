"""sledgehamr_gb300: sledgehamr's time-stepping hot path on a GB300 GPU.

Python host mirror of the library's C ABI (include/sledgehamr_gb300.h).  The
names follow the reference's operations: a :class:`Level` holds a level's two
time levels (grid_new / grid_old), :meth:`Level.advance` is
Integrator::Advance, :meth:`Level.fill_patch` is LevelSynchronizer::FillPatch,
:func:`average_down` / :func:`average_down_te` are AverageDownTo /
ComputeTruncationErrors, :meth:`Level.tag` is ErrorEst and
:meth:`Level.gw_spectrum` is GravitationalWaves::ComputeSpectrum.  The
output files of sledgehamr's IOModule are written by
:mod:`sledgehamr_gb300.output`.

All compute runs in libsledgehamr_gb300.so on the GPU; there is no CPU path.
"""
from __future__ import annotations

import ctypes as C
from typing import Sequence

import numpy as np

from . import _lib
from ._lib import SH_NEW, SH_OLD, SH_ADVANCE_NO_SWAP, ShAmrConfig, ShBox, ShRequest

# integrator.type (source/integrators/integrator.h:12-23)
LSSSPRK3 = 10
LEAPFROG = 11
RKN_TABLEAU = 20
RKN4 = 21
RKN5 = 22

# sh_level_reduce operations
REDUCE_MAX_ABS = 0  # AMReX MultiFab::norm0
REDUCE_MIN = 1
REDUCE_MAX = 2
REDUCE_SUM = 3
REDUCE_SUM_SQ = 4
REDUCE_COUNT_NONFINITE = 5
REDUCE_SUM_MODULUS = 6  # sum of sqrt(c^2 + (c+1)^2): the radial mode |Psi|

# project ids compiled into the library
PROJECTS = ("AxionStrings", "MinimalExample", "NextToMinimalExample",
            "FirstOrderPhaseTransition", "AxionStringsLap1", "AxionStringsLap2",
            "AxionStringsLap3")


class ShError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"sledgehamr_gb300 error {code}: {msg}")
        self.code = code


def _ptr(a):
    if a is None:
        return None
    return C.c_void_p(a.ctypes.data)


def _f64(a, n=None):
    if a is None:
        return None
    a = np.ascontiguousarray(np.asarray(a, dtype=np.float64))
    if n is not None and a.size < n:
        raise ValueError("array too short")
    return a


def project_id(name: str) -> int:
    lib = _lib.load()
    pid = C.c_int(-1)
    rc = lib.sh_project_find(name.encode(), C.byref(pid))
    if rc != 0:
        raise ShError(rc, f"unknown project {name!r}")
    return pid.value


def project_ncomp(name: str, with_gw: bool = False) -> tuple[int, int]:
    lib = _lib.load()
    nc, npair = C.c_int(), C.c_int()
    rc = lib.sh_project_ncomp(project_id(name), int(with_gw), C.byref(nc), C.byref(npair))
    if rc != 0:
        raise ShError(rc, f"project {name} with_gw={with_gw}")
    return nc.value, npair.value


def spectrum_bins(dim: int) -> np.ndarray:
    """Sorted unique k^2 of a dim^3 grid (pySledgehamr CreateUniqueVals)."""
    lib = _lib.load()
    n = C.c_int()
    lib.sh_spectrum_bins(dim, None, 0, C.byref(n))
    out = np.empty(n.value, dtype=np.int64)
    rc = lib.sh_spectrum_bins(dim, _ptr(out), n.value, C.byref(n))
    if rc != 0:
        raise ShError(rc, "sh_spectrum_bins")
    return out


def index_to_k(dim: int, projection_type: int) -> np.ndarray:
    lib = _lib.load()
    out = np.empty(dim, dtype=np.float64)
    rc = lib.sh_index_to_k(dim, projection_type, _ptr(out))
    if rc != 0:
        raise ShError(rc, "sh_index_to_k")
    return out


class Context:
    """A CUDA device and stream (sh_ctx)."""

    def __init__(self, device: int = 0):
        self.lib = _lib.load()
        h = C.c_void_p()
        rc = self.lib.sh_ctx_create(device, C.byref(h))
        if rc != 0:
            raise ShError(rc, f"could not create a context on device {device}")
        self.h = h

    def check(self, rc: int, what: str = ""):
        if rc != 0:
            msg = self.lib.sh_ctx_last_error(self.h)
            raise ShError(rc, f"{what}: {msg.decode() if msg else ''}")

    @property
    def stream(self) -> int:
        return self.lib.sh_ctx_stream(self.h) or 0

    def set_stream(self, stream_ptr: int | None):
        self.check(self.lib.sh_ctx_set_stream(self.h, C.c_void_p(stream_ptr or 0)), "set_stream")

    def synchronize(self):
        self.check(self.lib.sh_ctx_synchronize(self.h), "synchronize")

    @property
    def kernel_launches(self) -> int:
        return int(self.lib.sh_ctx_kernel_launches(self.h))

    def profile(self, enable: bool = True):
        """Start (clearing) or stop per-kernel CUDA-event timing."""
        self.check(self.lib.sh_ctx_profile(self.h, int(enable)), "profile")

    def profile_read(self, category: str) -> tuple[float, int]:
        """(summed device ms, launches) of a kernel category since profile()."""
        ms, n = C.c_double(), C.c_longlong()
        self.check(self.lib.sh_ctx_profile_read(self.h, category.encode(), C.byref(ms),
                                                C.byref(n)), "profile_read")
        return ms.value, n.value

    def close(self):
        if getattr(self, "h", None):
            self.lib.sh_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # -- convenience -----------------------------------------------------------
    def evolve_periodic(self, project: str, integrator: int, state: np.ndarray, t0: float,
                        dt: float, dx: float, nsteps: int, params: Sequence[float] = (),
                        gw_params: Sequence[float] = (), with_gw: bool = False,
                        nghost: int = 2, max_grid: int = 0, tableau=None, init_new=None,
                        ko_order: int = 0, ko_strength=None) -> np.ndarray:
        """nsteps steps of a periodic cubic level; state in canonical layout
        (ncomp, N, N, N) with x fastest."""
        st = _f64(state)
        ncomp, N = st.shape[0], st.shape[-1]
        out = np.empty_like(st)
        tab = _f64(tableau)
        nst = 0 if tableau is None else self._nstages(tab)
        p = _f64(list(params) or [0.0])
        g = _f64(list(gw_params) or [0.0])
        ko = _f64(ko_strength)
        rc = self.lib.sh_evolve_periodic(
            self.h, project_id(project), integrator, _ptr(tab), nst, N, max_grid, nghost,
            ncomp, int(with_gw), _ptr(st), _ptr(_f64(init_new)), _ptr(out), t0, dt, dx, nsteps,
            _ptr(p), len(params), _ptr(g), len(gw_params), ko_order, _ptr(ko))
        self.check(rc, "sh_evolve_periodic")
        return out

    @staticmethod
    def _nstages(tab: np.ndarray) -> int:
        for s in range(1, 9):
            if tab.size == 3 * s + s * (s + 1) // 2:
                return s
        raise ValueError("tableau length does not match any stage count")


def chop_boxes(N: int, max_grid: int) -> list[tuple[tuple[int, int, int], tuple[int, int, int]]]:
    mg = N if max_grid <= 0 or max_grid >= N else max_grid
    out = []
    for z in range(0, N, mg):
        for y in range(0, N, mg):
            for x in range(0, N, mg):
                out.append(((x, y, z), (min(x + mg, N) - 1, min(y + mg, N) - 1,
                                        min(z + mg, N) - 1)))
    return out


class Level:
    """A level of boxes with two time levels (sh_level)."""

    def __init__(self, ctx: Context, project: str, boxes, domain_lo, domain_hi, nghost: int,
                 with_gw: bool = False, precision: int = 0):
        """precision: PREC_FP64 (default) or PREC_FP32_KAHAN (FP32 values with
        Kahan compensations; RKN4 axion-string levels, sh_level_create_prec)."""
        self.ctx = ctx
        self.project = project
        self.precision = precision
        arr = (ShBox * len(boxes))()
        for q, (lo, hi) in enumerate(boxes):
            arr[q].lo[:] = list(lo)
            arr[q].hi[:] = list(hi)
        dlo = (C.c_int * 3)(*domain_lo)
        dhi = (C.c_int * 3)(*domain_hi)
        h = C.c_void_p()
        ctx.check(ctx.lib.sh_level_create_prec(ctx.h, project_id(project), int(with_gw), dlo,
                                               dhi, arr, len(boxes), nghost, precision,
                                               C.byref(h)),
                  "sh_level_create")
        self.h = h
        self.boxes = [(tuple(lo), tuple(hi)) for lo, hi in boxes]
        nc, nb, nv = C.c_int(), C.c_int(), C.c_longlong()
        ctx.lib.sh_level_info(h, C.byref(nc), C.byref(nb), C.byref(nv))
        self.ncomp, self.nbox, self.nvalid = nc.value, nb.value, nv.value
        self.domain = (tuple(domain_lo), tuple(domain_hi))

    @classmethod
    def periodic(cls, ctx: Context, project: str, N: int, nghost: int, max_grid: int = 0,
                 with_gw: bool = False, precision: int = 0) -> "Level":
        return cls(ctx, project, chop_boxes(N, max_grid), (0, 0, 0), (N - 1, N - 1, N - 1),
                   nghost, with_gw, precision)

    def close(self):
        if getattr(self, "h", None):
            self.ctx.lib.sh_level_destroy(self.ctx.h, self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def time(self, which: int = SH_NEW) -> tuple[float, int]:
        t, s = C.c_double(), C.c_int()
        self.ctx.lib.sh_level_time(self.h, which, C.byref(t), C.byref(s))
        return t.value, s.value

    def set_time(self, t: float, which: int = SH_NEW, istep: int = 0):
        self.ctx.lib.sh_level_set_time(self.h, which, t, istep)

    def write(self, data: np.ndarray, which: int = SH_NEW, layout: int = 0):
        a = _f64(data)
        if a.size != self.nvalid * self.ncomp:
            raise ValueError("data size does not match the level")
        self.ctx.check(self.ctx.lib.sh_level_write(self.ctx.h, self.h, which, layout, _ptr(a)),
                       "sh_level_write")

    def reduce(self, op: int, comp: int, which: int = SH_NEW) -> float:
        """sh_level_reduce: op (REDUCE_*) of component comp over the valid
        cells (fixed FP64 order, reproducible bit for bit)."""
        return _reduce(self.ctx, self.h, which, op, comp)

    def check_finite(self, which: int = SH_NEW) -> int:
        """sh_level_check_finite: 0, else raises ShError(SH_ERR_NONFINITE)."""
        return _check_finite(self.ctx, self.h, which)

    def string_tags(self, time: float, lev: int, dt: float, dx: float, params_tag=()) -> int:
        """Cosmology::GetStringTags: cells whose project tag hook is true."""
        return _string_tags(self.ctx, self.h, time, lev, dt, dx, params_tag)

    def mean_radial_mode(self, comp: int = 0, which: int = SH_NEW) -> float:
        """<r> = mean sqrt(Psi1^2 + Psi2^2) over the valid cells
        (NextToMinimalExample::WriteAvg), Psi1 = comp, Psi2 = comp + 1."""
        return self.reduce(REDUCE_SUM_MODULUS, comp, which) / self.nvalid

    def read(self, which: int = SH_NEW, layout: int = 0) -> np.ndarray:
        out = np.empty(self.nvalid * self.ncomp, dtype=np.float64)
        self.ctx.check(self.ctx.lib.sh_level_read(self.ctx.h, self.h, which, layout, _ptr(out)),
                       "sh_level_read")
        if layout == 0:
            N = self.domain[1][0] - self.domain[0][0] + 1
            return out.reshape(self.ncomp, N, N, N)
        return out

    def write_device(self, dev_ptr: int, which: int = SH_NEW, layout: int = 0):
        self.ctx.check(self.ctx.lib.sh_level_write_device(self.ctx.h, self.h, which, layout,
                                                          C.c_void_p(dev_ptr)),
                       "sh_level_write_device")

    def read_device(self, dev_ptr: int, which: int = SH_NEW, layout: int = 0):
        self.ctx.check(self.ctx.lib.sh_level_read_device(self.ctx.h, self.h, which, layout,
                                                         C.c_void_p(dev_ptr)),
                       "sh_level_read_device")

    def fill_patch(self, which: int = SH_NEW):
        self.ctx.check(self.ctx.lib.sh_level_fill_patch(self.ctx.h, self.h, which),
                       "sh_level_fill_patch")

    def advance(self, integrator: int, dt: float, dx: float, params: Sequence[float] = (),
                gw_params: Sequence[float] = (), tableau=None, ko_order: int = 0,
                ko_strength=None, flags: int = 0):
        tab = _f64(tableau)
        nst = 0 if tableau is None else Context._nstages(tab)
        p = _f64(list(params) or [0.0])
        g = _f64(list(gw_params) or [0.0])
        self.ctx.check(self.ctx.lib.sh_level_advance(
            self.ctx.h, self.h, integrator, _ptr(tab), nst, dt, dx, _ptr(p), len(params),
            _ptr(g), len(gw_params), ko_order, _ptr(_f64(ko_strength)), flags),
            "sh_level_advance")

    def rhs(self, time: float, lev: int, dt: float, dx: float, params=(), gw_params=(),
            which: int = SH_NEW, ko_order: int = 0, ko_strength=None) -> np.ndarray:
        out = np.empty(self.nvalid * self.ncomp, dtype=np.float64)
        p = _f64(list(params) or [0.0])
        g = _f64(list(gw_params) or [0.0])
        self.ctx.check(self.ctx.lib.sh_level_rhs(
            self.ctx.h, self.h, which, time, lev, dt, dx, _ptr(p), len(params), _ptr(g),
            len(gw_params), ko_order, _ptr(_f64(ko_strength)), _ptr(out)), "sh_level_rhs")
        return out

    def tag(self, time: float, lev: int, dt: float, dx: float, use_te: bool = False,
            te_crit=None, params_tag=(), params_mod=(), want_list: bool = False):
        """Returns (mask in boxes layout, counts, tag list or None)."""
        mask = np.empty(self.nvalid, dtype=np.uint8)
        counts = np.zeros(2 + self.ncomp, dtype=np.int64)
        tc = _f64(te_crit) if te_crit is not None else None
        pt = _f64(list(params_tag) or [0.0])
        pm = _f64(list(params_mod) or [0.0])
        lst = np.empty(self.nvalid if want_list else 1, dtype=np.int32)
        nt = C.c_longlong()
        self.ctx.check(self.ctx.lib.sh_tag(
            self.ctx.h, self.h, int(use_te), time, lev, dt, dx, _ptr(tc), _ptr(pt),
            len(params_tag), _ptr(pm), len(params_mod), _ptr(mask), _ptr(counts),
            _ptr(lst) if want_list else None, self.nvalid if want_list else 0, C.byref(nt)),
            "sh_tag")
        return mask, counts, (lst[: nt.value].copy() if want_list else None)

    def scalar_spectrum(self, fn: int, dx: float, comp: int = 0):
        """Spectrum::Compute of an output function (sh_scalar_spectrum):
        (bins, k^2 of the bins)."""
        N = self.domain[1][0] - self.domain[0][0] + 1
        cap = 3 * (N // 2 + 1) ** 2 + 16
        bins = np.empty(cap, dtype=np.float64)
        ks = np.empty(cap, dtype=np.int64)
        nb = C.c_int()
        self.ctx.check(self.ctx.lib.sh_scalar_spectrum(self.ctx.h, self.h, fn, comp, float(dx),
                                                       _ptr(bins), _ptr(ks), cap, C.byref(nb)),
                       "sh_scalar_spectrum")
        return bins[: nb.value].copy(), ks[: nb.value].copy()

    def add_bubbles(self, centres, profile, inv_dx: float, Lcut: float, dx: float,
                    comp_phi: int = 0, comp_dphi: int = 1, which: int = SH_NEW):
        """FirstOrderPhaseTransition bubble injection (sh_level_add_bubbles):
        centres (nb, 3), profile (2, nbins) for the field and its momentum."""
        xyz = _f64(centres)
        prof = _f64(profile)
        self.ctx.check(self.ctx.lib.sh_level_add_bubbles(
            self.ctx.h, self.h, which, comp_phi, comp_dphi, xyz.size // 3, _ptr(xyz), _ptr(prof),
            prof.size // 2, float(inv_dx), float(Lcut), float(dx)), "sh_level_add_bubbles")

    def gw_spectrum(self, zero_padding: int = 1, projection_type: int = 2, unbinned: bool = True,
                    comps: Sequence[int] | None = None):
        N = self.domain[1][0] - self.domain[0][0] + 1
        P = N * zero_padding
        cap = 3 * (P // 2 + 1) ** 2 + 16
        bins = np.empty(cap, dtype=np.float64)
        ks = np.empty(cap, dtype=np.int64)
        nb = C.c_int()
        c6 = None if comps is None else np.ascontiguousarray(np.asarray(comps, dtype=np.int32))
        self.ctx.check(self.ctx.lib.sh_gw_spectrum(
            self.ctx.h, self.h, _ptr(c6), zero_padding, projection_type, int(unbinned),
            _ptr(bins), _ptr(ks), cap, C.byref(nb)), "sh_gw_spectrum")
        return bins[: nb.value].copy(), ks[: nb.value].copy()


def average_down(ctx: Context, fine: Level, crse: Level, which_f: int = SH_NEW,
                 which_c: int = SH_NEW):
    ctx.check(ctx.lib.sh_average_down(ctx.h, fine.h, which_f, crse.h, which_c), "sh_average_down")


def average_down_te(ctx: Context, fine: Level, crse: Level):
    ctx.check(ctx.lib.sh_average_down_te(ctx.h, fine.h, crse.h), "sh_average_down_te")


def _check_finite(ctx: Context, h, which: int) -> int:
    n = C.c_longlong()
    ctx.check(ctx.lib.sh_level_check_finite(ctx.h, h, which, C.byref(n)), "sh_level_check_finite")
    return n.value


def _string_tags(ctx: Context, h, time, lev, dt, dx, params_tag=()) -> int:
    n = C.c_longlong()
    pt = _f64(list(params_tag) or [0.0])
    ctx.check(ctx.lib.sh_level_string_tags(ctx.h, h, float(time), int(lev), float(dt), float(dx),
                                           _ptr(pt), len(params_tag), C.byref(n)),
              "sh_level_string_tags")
    return n.value


def string_xi(string_tags: int, dx: float, L: float, eta: float) -> float:
    """Cosmology::Xi: string length parameter from a string-tag count."""
    lib = _lib.load()
    out = C.c_double()
    rc = lib.sh_string_xi(int(string_tags), float(dx), float(L), float(eta), C.byref(out))
    if rc != 0:
        raise ShError(rc, "sh_string_xi")
    return out.value


def _reduce(ctx: Context, h, which: int, op: int, comp: int) -> float:
    out = C.c_double()
    ctx.check(ctx.lib.sh_level_reduce(ctx.h, h, which, op, comp, C.byref(out)), "sh_level_reduce")
    return out.value


def amr_config(project: str, **kw) -> ShAmrConfig:
    """sh_amr_config with the library defaults, then the given fields
    (te_crit, params, gw_params as sequences)."""
    lib = _lib.load()
    cfg = ShAmrConfig()
    lib.sh_amr_config_defaults(C.byref(cfg))
    cfg.project = project_id(project)
    for k, v in kw.items():
        if k in ("te_crit",):
            for n, x in enumerate(v):
                cfg.te_crit[n] = x
        elif k == "params":
            for n, x in enumerate(v):
                cfg.params[n] = x
            cfg.nparams = len(v)
        elif k == "gw_params":
            for n, x in enumerate(v):
                cfg.gw_params[n] = x
            cfg.ngw = len(v)
        elif k in ("params_tag", "params_mod"):
            arr = getattr(cfg, k)
            for n, x in enumerate(v):
                arr[n] = x
            setattr(cfg, "n" + k, len(v))
        else:
            setattr(cfg, k, v)
    return cfg


def parse_trace(text: str) -> list[tuple[str, int, float]]:
    """Lines "<op> <level> <time>" of an AMR operation trace."""
    out = []
    for line in text.splitlines():
        op, lev, t = line.split()
        out.append((op, int(lev), float(t)))
    return out


def _boxes_of(arr, n):
    return [((arr[q].lo[0], arr[q].lo[1], arr[q].lo[2]), (arr[q].hi[0], arr[q].hi[1], arr[q].hi[2]))
            for q in range(n)]


class LevelView:
    """Read access to a level owned by an Amr hierarchy."""

    def __init__(self, ctx: Context, handle):
        self.ctx, self.h = ctx, handle
        nc, nb, nv = C.c_int(), C.c_int(), C.c_longlong()
        ctx.lib.sh_level_info(handle, C.byref(nc), C.byref(nb), C.byref(nv))
        self.ncomp, self.nbox, self.nvalid = nc.value, nb.value, nv.value
        arr = (ShBox * max(self.nbox, 1))()
        n = C.c_int()
        ctx.lib.sh_level_boxes(handle, arr, self.nbox, C.byref(n))
        self.boxes = _boxes_of(arr, n.value)
        lo, hi = (C.c_int * 3)(), (C.c_int * 3)()
        ctx.lib.sh_level_domain(handle, lo, hi)
        self.domain = (tuple(lo), tuple(hi))

    def reduce(self, op: int, comp: int, which: int = SH_NEW) -> float:
        return _reduce(self.ctx, self.h, which, op, comp)

    def gw_spectrum(self, zero_padding: int = 1, projection_type: int = 2, unbinned: bool = True,
                    comps: Sequence[int] | None = None):
        return Level.gw_spectrum(self, zero_padding, projection_type, unbinned, comps)

    def add_bubbles(self, centres, profile, inv_dx: float, Lcut: float, dx: float,
                    comp_phi: int = 0, comp_dphi: int = 1, which: int = SH_NEW):
        Level.add_bubbles(self, centres, profile, inv_dx, Lcut, dx, comp_phi, comp_dphi, which)

    def check_finite(self, which: int = SH_NEW) -> int:
        return _check_finite(self.ctx, self.h, which)

    def string_tags(self, time: float, lev: int, dt: float, dx: float, params_tag=()) -> int:
        return _string_tags(self.ctx, self.h, time, lev, dt, dx, params_tag)

    def mean_radial_mode(self, comp: int = 0, which: int = SH_NEW) -> float:
        return self.reduce(REDUCE_SUM_MODULUS, comp, which) / self.nvalid

    def read(self, which: int = SH_NEW) -> np.ndarray:
        out = np.empty(self.nvalid * self.ncomp, dtype=np.float64)
        self.ctx.check(self.ctx.lib.sh_level_read(self.ctx.h, self.h, which, 1, _ptr(out)),
                       "sh_level_read")
        return out

    def write(self, data: np.ndarray, which: int = SH_NEW):
        """Valid cells in the boxes layout (as read returns them)."""
        a = _f64(data)
        if a.size != self.nvalid * self.ncomp:
            raise ValueError("data size does not match the level")
        self.ctx.check(self.ctx.lib.sh_level_write(self.ctx.h, self.h, which, 1, _ptr(a)),
                       "sh_level_write")

    def time(self, which: int = SH_NEW):
        t, s = C.c_double(), C.c_int()
        self.ctx.lib.sh_level_time(self.h, which, C.byref(t), C.byref(s))
        return t.value, s.value


class Amr:
    """AMR hierarchy advanced by the library's time stepper (sh_amr)."""

    def __init__(self, ctx: Context, cfg: ShAmrConfig, level0: np.ndarray | None):
        """level0 None: a zero state (bubbles etc. go onto level(0) before the
        first step)."""
        self.ctx = ctx
        self.cfg = cfg
        a = None if level0 is None else _f64(level0)
        h = C.c_void_p()
        ctx.check(ctx.lib.sh_amr_create(ctx.h, C.byref(cfg), _ptr(a), C.byref(h)),
                  "sh_amr_create")
        self.h = h

    @classmethod
    def restart(cls, ctx: Context, cfg: ShAmrConfig, folder: str) -> "Amr":
        """A hierarchy from a checkpoint folder (sh_amr_restart)."""
        self = cls.__new__(cls)
        self.ctx = ctx
        self.cfg = cfg
        h = C.c_void_p()
        ctx.check(ctx.lib.sh_amr_restart(ctx.h, C.byref(cfg), str(folder).encode(), C.byref(h)),
                  "sh_amr_restart")
        self.h = h
        return self

    def checkpoint(self, folder: str):
        """Checkpoint::Write of the hierarchy into folder (sh_amr_checkpoint)."""
        self.ctx.check(self.ctx.lib.sh_amr_checkpoint(self.ctx.h, self.h, str(folder).encode()),
                       "sh_amr_checkpoint")

    def step(self, n: int = 1):
        self.ctx.check(self.ctx.lib.sh_amr_step(self.ctx.h, self.h, n), "sh_amr_step")

    def info(self):
        f, cu, nr = C.c_int(), C.c_longlong(), C.c_int()
        self.ctx.lib.sh_amr_info(self.h, C.byref(f), C.byref(cu), C.byref(nr))
        return {"finest": f.value, "cell_updates": cu.value, "nregrids": nr.value}

    def set_tag_params(self, params_tag=(), params_mod=()):
        pt = _f64(list(params_tag) or [0.0])
        pm = _f64(list(params_mod) or [0.0])
        self.ctx.check(self.ctx.lib.sh_amr_set_tag_params(self.h, _ptr(pt), len(params_tag),
                                                          _ptr(pm), len(params_mod)),
                       "sh_amr_set_tag_params")

    def set_timer_sync(self, on: bool = True):
        self.ctx.check(self.ctx.lib.sh_amr_set_timer_sync(self.h, int(on)), "set_timer_sync")

    def timers(self) -> dict:
        """Host seconds and calls per time-stepper phase (sh_amr_timer)."""
        out = {}
        q = 0
        name, sec, calls = C.c_char_p(), C.c_double(), C.c_longlong()
        while self.ctx.lib.sh_amr_timer(self.h, q, C.byref(name), C.byref(sec),
                                        C.byref(calls)) == 0:
            out[name.value.decode()] = (sec.value, calls.value)
            q += 1
        return out

    def set_trace(self, on: bool = True):
        self.ctx.check(self.ctx.lib.sh_amr_set_trace(self.h, int(on)), "sh_amr_set_trace")

    def trace(self) -> list[tuple[str, int, float]]:
        """The time stepper's operations so far: (op, level, time)."""
        n = C.c_longlong()
        self.ctx.check(self.ctx.lib.sh_amr_trace(self.h, None, 0, C.byref(n)), "sh_amr_trace")
        buf = C.create_string_buffer(n.value + 1)
        self.ctx.check(self.ctx.lib.sh_amr_trace(self.h, buf, n.value + 1, C.byref(n)),
                       "sh_amr_trace")
        return parse_trace(buf.value.decode())

    def level(self, lev: int) -> LevelView:
        h = C.c_void_p()
        self.ctx.check(self.ctx.lib.sh_amr_level(self.h, lev, C.byref(h)), "sh_amr_level")
        return LevelView(self.ctx, h)

    def regrid_record(self, q: int):
        lev, t = C.c_int(), C.c_double()
        nt, nn, nm = C.c_int(), C.c_int(), C.c_longlong()
        lib = self.ctx.lib
        self.ctx.check(lib.sh_amr_regrid_record(self.h, q, C.byref(lev), C.byref(t), None, 0,
                                                C.byref(nt), None, 0, C.byref(nm), None, 0,
                                                C.byref(nn)), "regrid_record")
        tb = (ShBox * max(nt.value, 1))()
        nb = (ShBox * max(nn.value, 1))()
        mask = np.empty(max(nm.value, 1), dtype=np.uint8)
        self.ctx.check(lib.sh_amr_regrid_record(self.h, q, C.byref(lev), C.byref(t), tb,
                                                nt.value, C.byref(nt), _ptr(mask), nm.value,
                                                C.byref(nm), nb, nn.value, C.byref(nn)),
                       "regrid_record")
        return {"lev": lev.value, "time": t.value, "tagged_boxes": _boxes_of(tb, nt.value),
                "mask": mask[: nm.value].copy(), "new_boxes": _boxes_of(nb, nn.value)}

    def close(self):
        if getattr(self, "h", None):
            self.ctx.lib.sh_amr_destroy(self.ctx.h, self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# output functions of projections and scalar spectra
OUT_COMPONENT = _lib.SH_OUT_COMPONENT
OUT_COMPONENT_SQ = _lib.SH_OUT_COMPONENT_SQ
OUT_A_PRIME2 = _lib.SH_OUT_A_PRIME2
OUT_A_PRIME_SCREENED = _lib.SH_OUT_A_PRIME_SCREENED
OUT_R_PRIME2 = _lib.SH_OUT_R_PRIME2


def projection(ctx: Context, levels, fn: int, comp: int = 0, mode: int = 0):
    """Line-of-sight projection along z over the given levels (coarse to
    fine; Level or LevelView objects): (data, n) on the finest pixel grid,
    data[x, y] (sh_projection)."""
    hs = (C.c_void_p * len(levels))(*[lv.h.value if isinstance(lv.h, C.c_void_p) else lv.h
                                      for lv in levels])
    last = levels[-1]
    N = last.domain[1][0] - last.domain[0][0] + 1
    data = np.empty((N, N), dtype=np.float64)
    n = np.empty((N, N), dtype=np.int32)
    ctx.check(ctx.lib.sh_projection(ctx.h, hs, len(levels), fn, comp, mode, _ptr(data),
                                    _ptr(n)), "sh_projection")
    return data, n


# ensemble families and precisions (sh_ensemble_create)
FAMILY_AXION_LAP1 = _lib.SH_FAMILY_AXION_LAP1
FAMILY_AXION_LAP2 = _lib.SH_FAMILY_AXION_LAP2
FAMILY_FOPT_GW = _lib.SH_FAMILY_FOPT_GW
PREC_FP64 = _lib.SH_PREC_FP64
PREC_FP32_KAHAN = _lib.SH_PREC_FP32_KAHAN
PREC_FP32 = _lib.SH_PREC_FP32
_FAMILY_NCOMP = {FAMILY_AXION_LAP1: 4, FAMILY_AXION_LAP2: 4, FAMILY_FOPT_GW: 14}


class Ensemble:
    """Many periodic realisations of one physics family stepped together
    (sh_ensemble).  ``params`` holds four numbers per realisation:
    (lambda, c, 0, 0) for the axion families, (q2, q3, q4, 0) for FOPT_GW."""

    def __init__(self, ctx: Context, family: int, precision: int, N: Sequence[int],
                 dx: Sequence[float], params=None):
        self.ctx = ctx
        self.family = family
        self.N = [int(n) for n in N]
        self.ncomp = _FAMILY_NCOMP.get(family, 0)  # unknown families: rejected below
        n = np.ascontiguousarray(np.asarray(self.N, dtype=np.int32))
        d = _f64(dx, len(self.N))
        p = None if params is None else _f64(params, 4 * len(self.N))
        h = C.c_void_p()
        rc = ctx.lib.sh_ensemble_create(ctx.h, family, precision, len(self.N), _ptr(n), _ptr(d),
                                        _ptr(p), C.byref(h))
        if rc != 0:
            raise ShError(rc, "sh_ensemble_create failed")
        self.h = h

    def check(self, rc: int, what: str):
        if rc != 0:
            msg = self.ctx.lib.sh_ensemble_last_error(self.h) or b""
            raise ShError(rc, f"{what}: {msg.decode(errors='replace')}")

    def info(self) -> dict:
        f, p, nr, nc, tz = C.c_int(), C.c_int(), C.c_int(), C.c_int(), C.c_int()
        cells, nbytes = C.c_longlong(), C.c_longlong()
        self.check(self.ctx.lib.sh_ensemble_info(self.h, C.byref(f), C.byref(p), C.byref(nr),
                                                 C.byref(nc), C.byref(cells), C.byref(nbytes),
                                                 C.byref(tz)), "sh_ensemble_info")
        return {"family": f.value, "precision": p.value, "nreal": nr.value, "ncomp": nc.value,
                "cells": cells.value, "device_bytes": nbytes.value, "tile_nz": tz.value}

    def kernel_launches(self) -> int:
        return int(self.ctx.lib.sh_ensemble_kernel_launches(self.h))

    @classmethod
    def pool(cls, ctx: Context, family: int, precision: int, capacity_cells: int = 0):
        """An empty pool (sh_ensemble_create_pool); members via admit()."""
        self = cls.__new__(cls)
        self.ctx = ctx
        self.family = family
        self.N = []
        self.ncomp = _FAMILY_NCOMP.get(family, 0)
        h = C.c_void_p()
        rc = ctx.lib.sh_ensemble_create_pool(ctx.h, family, precision, int(capacity_cells),
                                             C.byref(h))
        if rc != 0:
            raise ShError(rc, "sh_ensemble_create_pool failed")
        self.h = h
        return self

    def admit(self, N: int, dx: float, params=(0, 0, 0, 0), dt: float = 0.0):
        """A new member (zero state); None when the pool has no room."""
        p = _f64(list(params) + [0.0] * (4 - len(params)))
        slot = C.c_int()
        rc = self.ctx.lib.sh_ensemble_admit(self.h, int(N), float(dx), _ptr(p), float(dt),
                                            C.byref(slot))
        if rc == _lib.SH_ERR_NOMEM:
            return None
        self.check(rc, "admit")
        while len(self.N) <= slot.value:
            self.N.append(0)
        self.N[slot.value] = int(N)
        return slot.value

    def release(self, slot: int):
        self.check(self.ctx.lib.sh_ensemble_release(self.h, int(slot)), "release")

    def pool_info(self) -> dict:
        cap, fr, big, m = C.c_longlong(), C.c_longlong(), C.c_longlong(), C.c_int()
        self.check(self.ctx.lib.sh_ensemble_pool_info(self.h, C.byref(cap), C.byref(fr),
                                                      C.byref(big), C.byref(m)), "pool_info")
        return {"capacity": cap.value, "free": fr.value, "largest_free": big.value,
                "members": m.value}

    def set_time(self, t: float):
        self.check(self.ctx.lib.sh_ensemble_set_time(self.h, float(t)), "set_time")

    def time(self) -> float:
        t = C.c_double()
        self.check(self.ctx.lib.sh_ensemble_time(self.h, C.byref(t)), "time")
        return t.value

    def write(self, r: int, state: np.ndarray):
        a = _f64(state, self.ncomp * self.N[r] ** 3)
        self.check(self.ctx.lib.sh_ensemble_write(self.h, r, _ptr(a)), "write")

    def read(self, r: int) -> np.ndarray:
        N = self.N[r]
        out = np.empty((self.ncomp, N, N, N), dtype=np.float64)
        self.check(self.ctx.lib.sh_ensemble_read(self.h, r, _ptr(out)), "read")
        return out

    def set_graph(self, on: bool = True):
        self.check(self.ctx.lib.sh_ensemble_set_graph(self.h, int(on)), "set_graph")

    def step(self, dt: float, nsteps: int = 1):
        self.check(self.ctx.lib.sh_ensemble_step(self.h, float(dt), int(nsteps)), "step")

    def set_staging(self, staging: int):
        """0: stencil planes through registers; 1: tensor copies (TMA)."""
        self.check(self.ctx.lib.sh_ensemble_set_staging(self.h, int(staging)), "set_staging")

    def staging(self) -> int:
        s = C.c_int()
        self.check(self.ctx.lib.sh_ensemble_staging(self.h, C.byref(s)), "staging")
        return s.value

    def tune(self, dt: float, tile_nz: int = 0) -> int:
        ch = C.c_int()
        self.check(self.ctx.lib.sh_ensemble_tune(self.h, int(tile_nz), float(dt), C.byref(ch)),
                   "tune")
        return ch.value

    def energy(self) -> np.ndarray:
        e = np.empty(max(len(self.N), 1), dtype=np.float64)
        self.check(self.ctx.lib.sh_ensemble_energy(self.h, _ptr(e)), "energy")
        return e

    def string_count(self) -> np.ndarray:
        c = np.empty(max(len(self.N), 1), dtype=np.int64)
        self.check(self.ctx.lib.sh_ensemble_string_count(self.h, _ptr(c)), "string_count")
        return c

    def add_bubbles(self, r: int, centres, profile, inv_dx: float, Lcut: float):
        """Bubbles into realisation r (FOPT_GW): centres (nb, 3), profile
        (2, nbins) for Phi and dPhi (sh_level_add_bubbles)."""
        xyz = _f64(centres)
        prof = _f64(profile)
        self.check(self.ctx.lib.sh_ensemble_add_bubbles(
            self.h, r, xyz.size // 3, _ptr(xyz), _ptr(prof), prof.size // 2, float(inv_dx),
            float(Lcut)), "add_bubbles")

    def set_spectrum_precision(self, precision: int):
        """PREC_FP64 (default) or PREC_FP32 transforms and TT projection for
        the GW spectra (FP64 bin sums either way)."""
        self.check(self.ctx.lib.sh_ensemble_set_spectrum_precision(self.h, precision),
                   "set_spectrum_precision")

    def gw_spectrum(self, r: int, zero_padding: int = 1, projection_type: int = 2,
                    unbinned: bool = True):
        P = self.N[r] * zero_padding
        cap = 3 * (P // 2 + 1) ** 2 + 16
        bins = np.empty(cap, dtype=np.float64)
        ks = np.empty(cap, dtype=np.int64)
        nb = C.c_int()
        self.check(self.ctx.lib.sh_ensemble_gw_spectrum(
            self.h, r, zero_padding, projection_type, int(unbinned), _ptr(bins), _ptr(ks), cap,
            C.byref(nb)), "gw_spectrum")
        return bins[: nb.value].copy(), ks[: nb.value].copy()

    def close(self):
        if getattr(self, "h", None):
            self.ctx.lib.sh_ensemble_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


class Server:
    """Serving loop over a pool of FOPT + GW runs (sh_server)."""

    def __init__(self, ctx: Context, precision: int = PREC_FP32_KAHAN, capacity_cells: int = 0):
        self.ctx = ctx
        h = C.c_void_p()
        rc = ctx.lib.sh_server_create(ctx.h, precision, int(capacity_cells), C.byref(h))
        if rc != 0:
            raise ShError(rc, "sh_server_create failed")
        self.h = h
        self._keep = {}

    def check(self, rc: int, what: str):
        if rc != 0:
            msg = self.ctx.lib.sh_server_last_error(self.h) or b""
            raise ShError(rc, f"{what}: {msg.decode(errors='replace')}")

    def submit(self, N: int, dx: float, dt: float, t_end: float, params, centres=None,
               profile=None, inv_dx: float = 1.0, Lcut: float = 0.0, zero_padding: int = 1,
               projection_type: int = 2, unbinned: bool = False, max_level: int = 0,
               te_crit=(1e300, 1e300), regrid_dt: float = 0.0, blocking_factor: int = 0,
               max_grid_size: int = 0) -> int:
        """A run; max_level >= 1 makes it an AMR hierarchy refined by the
        truncation errors of Phi and dPhi against te_crit."""
        r = ShRequest()
        r.max_level, r.blocking_factor, r.max_grid_size = int(max_level), int(blocking_factor), \
            int(max_grid_size)
        r.te_crit[0], r.te_crit[1] = float(te_crit[0]), float(te_crit[1])
        r.regrid_dt = float(regrid_dt)
        r.N, r.dx, r.dt, r.t_end = int(N), float(dx), float(dt), float(t_end)
        for q, v in enumerate(list(params)[:4]):
            r.params[q] = float(v)
        xyz = _f64(centres) if centres is not None else None
        prof = _f64(profile) if profile is not None else None
        r.nbubbles = 0 if xyz is None else xyz.size // 3
        r.xyz = None if xyz is None else xyz.ctypes.data
        r.profile = None if prof is None else prof.ctypes.data
        r.nbins = 0 if prof is None else prof.size // 2
        r.inv_dx, r.Lcut = float(inv_dx), float(Lcut)
        r.zero_padding, r.projection_type, r.unbinned = int(zero_padding), int(projection_type), \
            int(unbinned)
        rid = C.c_longlong()
        self.check(self.ctx.lib.sh_server_submit(self.h, C.byref(r), C.byref(rid)), "submit")
        return rid.value

    def step(self):
        a, q, c = C.c_int(), C.c_int(), C.c_int()
        self.check(self.ctx.lib.sh_server_step(self.h, C.byref(a), C.byref(q), C.byref(c)), "step")
        return a.value, q.value, c.value

    def status(self, rid: int):
        st = C.c_int()
        t = np.zeros(3)
        self.check(self.ctx.lib.sh_server_status(self.h, int(rid), C.byref(st), _ptr(t)),
                   "status")
        return st.value, t

    def result(self, rid: int):
        nb = C.c_int()
        self.check(self.ctx.lib.sh_server_result(self.h, int(rid), None, None, 0, C.byref(nb)),
                   "result")
        bins = np.empty(nb.value)
        ks = np.empty(nb.value, dtype=np.int64)
        self.check(self.ctx.lib.sh_server_result(self.h, int(rid), _ptr(bins), _ptr(ks),
                                                 nb.value, C.byref(nb)), "result")
        return bins, ks

    def info(self) -> dict:
        a, q = C.c_int(), C.c_int()
        cu, it, fr = C.c_longlong(), C.c_longlong(), C.c_longlong()
        self.check(self.ctx.lib.sh_server_info(self.h, C.byref(a), C.byref(q), C.byref(cu),
                                               C.byref(it), C.byref(fr)), "info")
        return {"running": a.value, "queued": q.value, "cell_updates": cu.value,
                "iterations": it.value, "free_cells": fr.value}

    def close(self):
        if getattr(self, "h", None):
            self.ctx.lib.sh_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
