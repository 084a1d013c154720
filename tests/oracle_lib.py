"""ctypes access to the ORACLE libraries (test infrastructure only).

Oracle()            -> oracle/_build/liboracle.so, the CPU restatement
Oracle(ref=True)    -> oracle/_ref/libshref.so, the same drivers around the
                       reference's own per-cell headers (only where the
                       sledgehamr sources were present to build it)
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_SO = os.path.join(ROOT, "oracle", "_build", "liboracle.so")
REF_SO = os.path.join(ROOT, "oracle", "_ref", "libshref.so")

PROJECT_IDS = {"AxionStrings": 0, "MinimalExample": 1, "NextToMinimalExample": 2,
               "FirstOrderPhaseTransition": 3, "AxionStringsLap1": 4, "AxionStringsLap2": 5,
               "AxionStringsLap3": 6}

vp = C.c_void_p


def _p(a):
    return None if a is None else C.c_void_p(a.ctypes.data)


def _f(a):
    return None if a is None else np.ascontiguousarray(np.asarray(a, dtype=np.float64))


def build_oracle():
    if not os.path.exists(ORACLE_SO):
        subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle")], check=True)


REF_INT_SO = os.path.join(ROOT, "oracle", "_ref", "libshref_int.so")


def ref_available() -> bool:
    return os.path.exists(REF_SO)


def ref_integrators_available() -> bool:
    return os.path.exists(REF_INT_SO)


def ref_int_evolve(project, integrator, state, t0, dt, dx, nsteps, params=(), gw_params=(),
                   with_gw=False, nghost=2):
    """nsteps steps of a periodic level by the reference's own integrators
    (rkn.cpp, lsssprk3.cpp, leapfrog.cpp compiled unchanged into
    oracle/_ref/libshref_int.so) with the reference's per-cell Rhs."""
    lib = C.CDLL(REF_INT_SO)
    f = lib.ref_int_evolve
    f.restype = C.c_int
    st = _f(state)
    out = np.empty_like(st)
    p = _f(list(params) or [0.0])
    g = _f(list(gw_params) or [0.0])
    rc = f(PROJECT_IDS[project], integrator, st.shape[-1], nghost, st.shape[0], int(with_gw),
           _p(st), _p(out), C.c_double(t0), C.c_double(dt), C.c_double(dx), nsteps, _p(p),
           len(params), _p(g), len(gw_params))
    if rc != 0:
        raise RuntimeError(f"ref_int_evolve rc={rc}")
    return out


class Oracle:
    def __init__(self, ref: bool = False):
        if ref:
            if not ref_available():
                raise FileNotFoundError(REF_SO)
            self.lib = C.CDLL(REF_SO)
            self.pre = "ref_"
        else:
            build_oracle()
            self.lib = C.CDLL(ORACLE_SO)
            self.pre = "orc_"

    def _fn(self, name):
        f = getattr(self.lib, self.pre + name)
        f.restype = C.c_int
        return f

    def evolve_periodic(self, project, integrator, state, t0, dt, dx, nsteps, params=(),
                        gw_params=(), with_gw=False, nghost=2, max_grid=0, tableau=None,
                        init_new=None, ko_order=0, ko_strength=None):
        st = _f(state)
        out = np.empty_like(st)
        tab = _f(tableau)
        nst = 0
        if tableau is not None:
            for s in range(1, 9):
                if tab.size == 3 * s + s * (s + 1) // 2:
                    nst = s
        p = _f(list(params) or [0.0])
        g = _f(list(gw_params) or [0.0])
        rc = self._fn("evolve_periodic")(
            PROJECT_IDS[project], integrator, _p(tab), nst, st.shape[-1], max_grid, nghost,
            st.shape[0], int(with_gw), _p(st), _p(_f(init_new)), _p(out), C.c_double(t0),
            C.c_double(dt), C.c_double(dx), nsteps, _p(p), len(params), _p(g), len(gw_params),
            ko_order, _p(_f(ko_strength)))
        if rc != 0:
            raise RuntimeError(f"{self.pre}evolve_periodic rc={rc}")
        return out

    def fill_rhs(self, project, state, time, lev, dt, dx, params=(), gw_params=(),
                 with_gw=False, nghost=3, ko_order=0, ko_strength=None, rhs_init=None):
        st = _f(state)
        out = np.zeros_like(st) if rhs_init is None else _f(rhs_init).copy()
        p = _f(list(params) or [0.0])
        g = _f(list(gw_params) or [0.0])
        rc = self._fn("fill_rhs")(PROJECT_IDS[project], st.shape[-1], nghost, st.shape[0],
                                  int(with_gw), _p(st), _p(out), C.c_double(time), lev,
                                  C.c_double(dt), C.c_double(dx), _p(p), _p(g), ko_order,
                                  _p(_f(ko_strength)))
        if rc != 0:
            raise RuntimeError(f"fill_rhs rc={rc}")
        return out

    def avgdown_te(self, fine, crse, te):
        f, c, t = _f(fine), _f(crse).copy(), _f(te).copy()
        rc = self._fn("avgdown_te")(f.shape[0], c.shape[-1], _p(f), _p(c), _p(t))
        if rc != 0:
            raise RuntimeError("avgdown_te")
        return c, t

    def average_down(self, fine):
        f = _f(fine)
        Nc = f.shape[-1] // 2
        c = np.zeros((f.shape[0], Nc, Nc, Nc))
        rc = self._fn("average_down")(f.shape[0], Nc, _p(f), _p(c))
        if rc != 0:
            raise RuntimeError("average_down")
        return c

    def tag(self, project, state, te, time, lev, dt, dx, te_crit=None, params_tag=(),
            params_mod=(), max_grid=0):
        st = _f(state)
        ncomp, N = st.shape[0], st.shape[-1]
        mask = np.zeros((N, N, N), dtype=np.uint8)
        counts = np.zeros(2 + ncomp, dtype=np.int64)
        pt = _f(list(params_tag) or [0.0])
        pm = _f(list(params_mod) or [0.0])
        tc = _f(te_crit) if te_crit is not None else _f(np.full(ncomp, np.finfo(float).max))
        rc = self._fn("tag")(PROJECT_IDS[project], N, max_grid, ncomp, _p(st), _p(_f(te)),
                             C.c_double(time), lev, C.c_double(dt), C.c_double(dx), _p(tc),
                             _p(pt), _p(pm), _p(mask), C.c_void_p(counts.ctypes.data))
        if rc != 0:
            raise RuntimeError(f"tag rc={rc}")
        return mask, counts

    def gw_spectrum(self, comps6, zero_padding=1, projection_type=2, unbinned=True):
        c = _f(comps6)
        N = c.shape[-1]
        P = N * zero_padding
        cap = 3 * (P // 2 + 1) ** 2 + 16
        bins = np.empty(cap)
        ks = np.empty(cap, dtype=np.int64)
        nb = C.c_int()
        rc = self._fn("gw_spectrum")(_p(c), N, zero_padding, projection_type, int(unbinned),
                                     _p(bins), _p(ks), cap, C.byref(nb))
        if rc != 0:
            raise RuntimeError("gw_spectrum")
        return bins[: nb.value].copy(), ks[: nb.value].copy()

    def unique_k2(self, dim):
        cap = 3 * (dim // 2 + 1) ** 2 + 16
        out = np.empty(cap, dtype=np.int64)
        n = C.c_int()
        rc = self._fn("unique_k2")(dim, _p(out), cap, C.byref(n))
        if rc != 0:
            raise RuntimeError("unique_k2")
        return out[: n.value].copy()

    def index_to_k(self, dim, projection_type):
        out = np.empty(dim)
        self._fn("index_to_k")(dim, projection_type, _p(out))
        return out

    def stencil(self, kind, order, field, dx):
        f = _f(field)
        out = np.empty_like(f)
        rc = self._fn("stencil")(kind, order, f.shape[-1], _p(f), C.c_double(dx), _p(out))
        if rc != 0:
            raise RuntimeError("stencil")
        return out


class OracleAmr:
    """The oracle's AMR hierarchy (same time stepper, CPU numerics)."""

    def __init__(self, cfg, level0):
        build_oracle()
        self.lib = C.CDLL(ORACLE_SO)
        self.lib.orc_amr_create.restype = C.c_void_p
        self.lib.orc_amr_create.argtypes = [C.c_void_p, C.c_void_p]
        for n in ("orc_amr_step", "orc_amr_info", "orc_amr_boxes", "orc_amr_read",
                  "orc_amr_regrid_record"):
            getattr(self.lib, n).restype = C.c_int
        self.lib.orc_amr_destroy.argtypes = [C.c_void_p]
        a = _f(level0)
        self.h = self.lib.orc_amr_create(C.byref(cfg), _p(a))
        if not self.h:
            raise RuntimeError("orc_amr_create failed")
        self.h = C.c_void_p(self.h)
        self.ncomp = a.shape[0]
        self.N0 = a.shape[-1]

    def step(self, n=1):
        if self.lib.orc_amr_step(self.h, n) != 0:
            raise RuntimeError("orc_amr_step failed")

    def info(self):
        f, cu, nr = C.c_int(), C.c_longlong(), C.c_int()
        self.lib.orc_amr_info(self.h, C.byref(f), C.byref(cu), C.byref(nr))
        return {"finest": f.value, "cell_updates": cu.value, "nregrids": nr.value}

    @classmethod
    def restart(cls, cfg, folder):
        """A hierarchy from a checkpoint folder (orc_amr_restart)."""
        build_oracle()
        self = cls.__new__(cls)
        self.lib = C.CDLL(ORACLE_SO)
        self.lib.orc_amr_restart.restype = C.c_void_p
        self.lib.orc_amr_restart.argtypes = [C.c_void_p, C.c_char_p]
        for n in ("orc_amr_step", "orc_amr_info", "orc_amr_boxes", "orc_amr_read",
                  "orc_amr_regrid_record"):
            getattr(self.lib, n).restype = C.c_int
        self.lib.orc_amr_destroy.argtypes = [C.c_void_p]
        h = self.lib.orc_amr_restart(C.byref(cfg), str(folder).encode())
        if not h:
            raise RuntimeError("orc_amr_restart failed")
        self.h = C.c_void_p(h)
        self.N0 = cfg.N0
        from tests import hdf5_read
        self.ncomp = int(hdf5_read.File(os.path.join(str(folder), "Meta.hdf5"))["Header"][5])
        return self

    def checkpoint(self, folder):
        f = self.lib.orc_amr_checkpoint
        f.restype = C.c_int
        f.argtypes = [C.c_void_p, C.c_char_p]
        if f(self.h, str(folder).encode()) != 0:
            raise RuntimeError("orc_amr_checkpoint failed")

    def set_trace(self, on=True):
        self.lib.orc_amr_set_trace.restype = C.c_int
        self.lib.orc_amr_set_trace(self.h, int(on))

    def trace(self):
        """The time stepper's operations so far: (op, level, time)."""
        f = self.lib.orc_amr_trace
        f.restype = C.c_longlong
        f.argtypes = [C.c_void_p, C.c_char_p, C.c_longlong]
        n = f(self.h, None, 0)
        buf = C.create_string_buffer(n + 1)
        if f(self.h, buf, n + 1) < 0:
            raise RuntimeError("orc_amr_trace")
        out = []
        for line in buf.value.decode().splitlines():
            op, lev, t = line.split()
            out.append((op, int(lev), float(t)))
        return out

    def boxes(self, lev):
        out = np.empty(6 * 100000, dtype=np.int32)
        n = self.lib.orc_amr_boxes(self.h, lev, _p(out), 100000)
        if n < 0:
            raise RuntimeError("orc_amr_boxes")
        b = out[: 6 * n].reshape(n, 6)
        return [(tuple(int(x) for x in r[:3]), tuple(int(x) for x in r[3:])) for r in b]

    def read(self, lev, which=0):
        bx = self.boxes(lev)
        nv = sum((h[0] - l[0] + 1) * (h[1] - l[1] + 1) * (h[2] - l[2] + 1) for l, h in bx)
        out = np.empty(nv * self.ncomp)
        t = C.c_double()
        self.lib.orc_amr_read(self.h, lev, which, _p(out), C.byref(t))
        return out, t.value

    def regrid_record(self, q):
        lev, t = C.c_int(), C.c_double()
        nt, nn, nm = C.c_int(), C.c_int(), C.c_longlong()
        self.lib.orc_amr_regrid_record(self.h, q, C.byref(lev), C.byref(t), None, 0,
                                       C.byref(nt), None, C.c_longlong(0), C.byref(nm), None, 0,
                                       C.byref(nn))
        tb = np.empty(6 * max(nt.value, 1), dtype=np.int32)
        nb = np.empty(6 * max(nn.value, 1), dtype=np.int32)
        mask = np.empty(max(nm.value, 1), dtype=np.uint8)
        self.lib.orc_amr_regrid_record(self.h, q, C.byref(lev), C.byref(t), _p(tb), nt.value,
                                       C.byref(nt), _p(mask), C.c_longlong(nm.value),
                                       C.byref(nm), _p(nb), nn.value, C.byref(nn))
        conv = lambda a, n: [(tuple(int(x) for x in r[:3]), tuple(int(x) for x in r[3:]))
                             for r in a[: 6 * n].reshape(n, 6)]
        return {"lev": lev.value, "time": t.value, "tagged_boxes": conv(tb, nt.value),
                "mask": mask[: nm.value].copy(), "new_boxes": conv(nb, nn.value)}

    def projection(self, fn, comp=0, mode=0, max_level=100):
        """Projection::Compute over the hierarchy (orc_amr_projection)."""
        f = self.lib.orc_amr_projection
        f.restype = C.c_int
        ml = min(max_level, self.info()["finest"])
        N = self.N0 << ml
        data = np.empty((N, N))
        n = np.empty((N, N), dtype=np.int32)
        rc = f(self.h, fn, comp, mode, ml, _p(data), C.c_void_p(n.ctypes.data))
        if rc != 0:
            raise RuntimeError("projection")
        return data, n

    def close(self):
        if self.h:
            self.lib.orc_amr_destroy(self.h)
            self.h = None


def oracle_add_bubbles(state, xyz, profile, inv_dx, Lcut, dx, comp_phi=0, comp_dphi=1,
                       ref=False):
    """Bubble injection on a periodic canonical state (orc_add_bubbles, or
    the reference's AddBubble through ref_add_bubbles with ref=True)."""
    st = np.ascontiguousarray(np.array(state, dtype=np.float64))
    ncomp, N = st.shape[0], st.shape[-1]
    x = _f(xyz)
    p = _f(profile)
    if ref:
        lib = C.CDLL(REF_SO)
        f = lib.ref_add_bubbles
        f.restype = C.c_int
        rc = f(N, ncomp, _p(st), x.size // 3, _p(x), _p(p), p.size // 2, C.c_double(inv_dx),
               C.c_double(Lcut), C.c_double(dx))
    else:
        build_oracle()
        lib = C.CDLL(ORACLE_SO)
        f = lib.orc_add_bubbles
        f.restype = C.c_int
        rc = f(N, ncomp, _p(st), comp_phi, comp_dphi, x.size // 3, _p(x), _p(p), p.size // 2,
               C.c_double(inv_dx), C.c_double(Lcut), C.c_double(dx))
    if rc != 0:
        raise RuntimeError("add_bubbles")
    return st


def oracle_out_function(state, fn, comp=0, ref=False):
    """Per-cell output function on a canonical state (orc_out_function, or
    the reference's own functions through ref_out_function)."""
    st = _f(state)
    ncomp, N = st.shape[0], st.shape[-1]
    out = np.empty((N, N, N))
    if ref:
        lib = C.CDLL(REF_SO)
        f = lib.ref_out_function
        f.restype = C.c_int
        rc = f(_p(st), N, ncomp, fn, _p(out))
    else:
        build_oracle()
        lib = C.CDLL(ORACLE_SO)
        f = lib.orc_out_function
        f.restype = C.c_int
        rc = f(_p(st), N, ncomp, fn, comp, _p(out))
    if rc != 0:
        raise RuntimeError("out_function")
    return out


def oracle_scalar_spectrum(state, fn, comp, L, t):
    """Spectrum::Compute on a canonical periodic state (orc_scalar_spectrum)."""
    build_oracle()
    lib = C.CDLL(ORACLE_SO)
    st = _f(state)
    ncomp, N = st.shape[0], st.shape[-1]
    cap = 3 * (N // 2 + 1) ** 2 + 16
    bins = np.empty(cap)
    ks = np.empty(cap, dtype=np.int64)
    nb = C.c_int()
    f = lib.orc_scalar_spectrum
    f.restype = C.c_int
    rc = f(_p(st), N, ncomp, fn, comp, C.c_double(L), C.c_double(t), _p(bins), _p(ks), cap,
           C.byref(nb))
    if rc != 0:
        raise RuntimeError("scalar_spectrum")
    return bins[: nb.value].copy(), ks[: nb.value].copy()
