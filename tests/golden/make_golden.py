"""Generates the golden fixtures of tests/golden/ from the sledgehamr
reference itself (run in a checkout where the reference sources exist).

  spectra_ks_<N>.npz   - the unique-k^2 bins and index_to_k arrays (types 1
                         and 2) stored in the reference's data/spectra_ks.hdf5,
                         located by exact byte match of their int64/float64
                         contents and copied out verbatim.
  ref_*.npz            - inputs and outputs of the reference's own per-cell
                         code (oracle/_ref/libshref.so, built by
                         oracle/build_ref.sh from the reference headers) driven
                         by the oracle's integrator sequences: evolutions,
                         Rhs evaluations, tag masks and truncation errors.

  ref_bubbles.npz      - the reference's FOPT bubble injection (AddBubble).
  hdf5_format.npz      - format fields of data/spectra_ks.hdf5 as h5py wrote
                         them, read with tests/hdf5_read.py: superblock bytes
                         8-39 and 48-55, the message types of a dataset's
                         header, its header prefix, and the dataspace,
                         fill-value and float64 datatype messages.

Usage: python tests/golden/make_golden.py [REFERENCE_ROOT] [--only=spectra,evolve,bubbles]
(the spectra step also writes hdf5_format.npz)
"""
from __future__ import annotations

import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from sledgehamr_gb300 import ic  # noqa: E402
from tests.oracle_lib import Oracle  # noqa: E402


def spectra_fixtures(ref_root: str):
    raw = open(os.path.join(ref_root, "data", "spectra_ks.hdf5"), "rb").read()
    orc = Oracle()
    for N in (32, 64):
        bins = orc.unique_k2(N).astype("<i8")
        k1 = orc.index_to_k(N, 1).astype("<f8")
        k2 = orc.index_to_k(N, 2).astype("<f8")
        out = {}
        for name, arr in (("bins", bins), ("k1", k1), ("k2", k2)):
            off = raw.find(arr.tobytes())
            if off < 0:
                raise SystemExit(f"{N}_{name}: no byte-exact match in spectra_ks.hdf5")
            out[name] = np.frombuffer(raw[off: off + arr.nbytes], dtype=arr.dtype).copy()
            out[name + "_offset"] = np.int64(off)
        np.savez_compressed(os.path.join(HERE, f"spectra_ks_{N}.npz"), **out)
        print(f"spectra_ks_{N}.npz: {len(out['bins'])} bins")


def hdf5_format_fixture(ref_root: str):
    from tests import hdf5_read
    f = hdf5_read.File(os.path.join(ref_root, "data", "spectra_ks.hdf5"))
    ds = f.datasets["32_k1"]
    msg = {m.type: m for m in ds.messages}
    hdr = f.buf[f.entries["32_k1"]:f.entries["32_k1"] + 16]
    u8 = lambda b: np.frombuffer(bytes(b), dtype=np.uint8).copy()  # noqa: E731
    np.savez_compressed(
        os.path.join(HERE, "hdf5_format.npz"),
        superblock_8_40=u8(f.buf[8:40]), superblock_48_56=u8(f.buf[48:56]),
        message_types=np.array([m.type for m in ds.messages], dtype=np.int64),
        message_flags=np.array([m.flags for m in ds.messages], dtype=np.int64),
        header_prefix=u8(hdr[:2] + hdr[4:12]), dataspace_head=u8(msg[1].data[:4]),
        fill_value=u8(msg[5].data), datatype_f64=u8(msg[3].data),
        layout_head=u8(msg[8].data[:2]))
    print("hdf5_format.npz")


def fopt_params(lambda_bar=0.8):
    numer = 3.0 + np.sqrt(9.0 - 8.0 * lambda_bar)
    return [0.0, -1.0, 3.0 * numer / (4.0 * lambda_bar), -numer * numer / (8.0 * lambda_bar),
            0.0, 0.0, 0.0]


def evolve_fixtures():
    ref = Oracle(ref=True)
    N, L = 16, 4.0
    dx, dt = L / N, 0.25 * L / N
    st = ic.axion_string_ic(N, L, kmax=6.0, seed=3)
    st[2:] = 0.3 * ic.axion_string_ic(N, L, kmax=6.0, seed=4)[:2]
    cases = {
        "ref_axion_rkn4": ("AxionStrings", 21, None),
        "ref_axion_rkn5": ("AxionStrings", 22, None),
        "ref_minimal_ssprk3": ("MinimalExample", 10, None),
        "ref_axion_leapfrog": ("AxionStrings", 11, None),
    }
    for name, (proj, integ, tab) in cases.items():
        out = ref.evolve_periodic(proj, integ, st, t0=1.0, dt=dt, dx=dx, nsteps=5, nghost=2)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), state_in=st, state_out=out,
                            t0=1.0, dt=dt, dx=dx, nsteps=5, nghost=2, integrator=integ,
                            project=proj)
        print(name)
    # FOPT + GW tensor, leapfrog (the C2 scheme), 12^3
    N2 = 12
    s14 = np.zeros((14, N2, N2, N2))
    s14[0] = 0.8 * ic.gaussian_field(N2, 3.0, 8.0, 11)
    s14[1] = 0.2 * ic.gaussian_field(N2, 3.0, 8.0, 12)
    s14[2:8] = 0.05 * np.stack([ic.gaussian_field(N2, 3.0, 8.0, 20 + q) for q in range(6)])
    dx2 = 0.25
    out = ref.evolve_periodic("FirstOrderPhaseTransition", 11, s14, t0=0.0, dt=0.05, dx=dx2,
                              nsteps=5, params=fopt_params(), gw_params=[-1.0, 1.0],
                              with_gw=True, nghost=2)
    np.savez_compressed(os.path.join(HERE, "ref_fopt_gw_leapfrog.npz"), state_in=s14,
                        state_out=out, t0=0.0, dt=0.05, dx=dx2, nsteps=5, nghost=2,
                        params=np.array(fopt_params()), gw_params=np.array([-1.0, 1.0]))
    print("ref_fopt_gw_leapfrog")
    # single Rhs evaluations: AxionStrings with GW hook, KO dissipation 2 and 3
    s16 = np.zeros((16, N, N, N))
    s16[:4] = st
    s16[4:] = 0.1 * np.stack([ic.gaussian_field(N, L, 6.0, 40 + q) for q in range(12)])
    rhs = ref.fill_rhs("AxionStrings", s16, 1.5, 0, dt, dx, with_gw=True, nghost=3)
    ko2 = ref.fill_rhs("MinimalExample", st, 1.5, 0, dt, dx, nghost=3, ko_order=2,
                       ko_strength=[0.1, 0.2, 0.3, 0.4])
    ko3 = ref.fill_rhs("MinimalExample", st, 1.5, 0, dt, dx, nghost=3, ko_order=3,
                       ko_strength=[0.1, 0.2, 0.3, 0.4])
    np.savez_compressed(os.path.join(HERE, "ref_rhs.npz"), state16=s16, rhs_axion_gw=rhs,
                        state4=st, rhs_ko2=ko2, rhs_ko3=ko3, time=1.5, dt=dt, dx=dx)
    print("ref_rhs")
    # tagging with truncation errors (AxionStrings modifiers) on boxes of 8
    te = np.abs(ic.normal(77, st.size).reshape(st.shape)) * 1e-3
    crit = np.array([1.5e-3, 2.0e-3, 1e-2, 1e-2])
    mask, counts = ref.tag("AxionStrings", st, te, 1.0, 0, dt, dx, te_crit=crit, max_grid=8)
    mask0, counts0 = ref.tag("AxionStrings", st, None, 1.0, 0, dt, dx, max_grid=8)
    np.savez_compressed(os.path.join(HERE, "ref_tag.npz"), state=st, te=te, te_crit=crit,
                        mask=mask, counts=counts, mask_user=mask0, counts_user=counts0, dt=dt,
                        dx=dx)
    print("ref_tag", int(mask.sum()), int(mask0.sum()))
    # average-down with truncation error: the reference kernel on one box
    fine = ic.normal(5, 4 * 16 ** 3).reshape(4, 16, 16, 16)
    crse = ic.normal(6, 4 * 8 ** 3).reshape(4, 8, 8, 8)
    tei = np.zeros_like(fine)
    c2, t2 = crse.copy(), tei.copy()
    import ctypes as C
    f = ref.lib.ref_avgdown_te_kernel
    f.restype = C.c_int
    f(4, 8, C.c_void_p(fine.ctypes.data), C.c_void_p(c2.ctypes.data), C.c_void_p(t2.ctypes.data))
    np.savez_compressed(os.path.join(HERE, "ref_avgdown_te.npz"), fine=fine, crse_in=crse,
                        crse_out=c2, te_out=t2)
    print("ref_avgdown_te")


def bubble_profile(nbins, inv_dx, radius, width, amplitude, velocity=0.0):
    """Tanh wall profile phi(r) = A/2 (1 - tanh((r - R)/w)) and its time
    derivative for a wall moving outwards at speed v (rows 0 and 1)."""
    r = np.arange(nbins) / inv_dx
    x = (r - radius) / width
    phi = 0.5 * amplitude * (1.0 - np.tanh(x))
    dphi = velocity * 0.5 * amplitude / width / np.cosh(x) ** 2
    return np.stack([phi, dphi])


def bubble_fixture():
    """The reference's AddBubble (FirstOrderPhaseTransition kernels_misc.h)
    on a 16^3 FOPT + GW state: three bubbles, one across the periodic
    corner, cut-off 5.3 with bins of 0.25."""
    import ctypes as C
    ref = Oracle(ref=True)
    N, dx = 16, 0.5
    st = np.stack([ic.gaussian_field(N, N * dx, 3.0, 90 + q) for q in range(14)]) * 0.1
    xyz = np.array([[3.1, 4.7, 2.2], [7.9, 0.3, 7.6], [0.0, 5.5, 4.0]])
    inv_dx, Lcut = 4.0, 5.3
    nbins = int(Lcut * inv_dx) + 2
    prof = bubble_profile(nbins, inv_dx, 2.5, 1.0, 1.2, velocity=0.4)
    out = np.ascontiguousarray(st.copy())
    f = ref.lib.ref_add_bubbles
    f.restype = C.c_int
    rc = f(N, 14, C.c_void_p(out.ctypes.data), 3, C.c_void_p(np.ascontiguousarray(xyz).ctypes.data),
           C.c_void_p(np.ascontiguousarray(prof).ctypes.data), nbins, C.c_double(inv_dx),
           C.c_double(Lcut), C.c_double(dx))
    assert rc == 0
    np.savez_compressed(os.path.join(HERE, "ref_bubbles.npz"), state_in=st, state_out=out,
                        xyz=xyz, profile=prof, inv_dx=inv_dx, Lcut=Lcut, dx=dx)
    print("ref_bubbles", float(np.abs(out - st).max()))


if __name__ == "__main__":
    args = [a for a in sys.argv[1:] if not a.startswith("--only=")]
    only = [x for a in sys.argv[1:] if a.startswith("--only=")
            for x in a.split("=", 1)[1].split(",")]
    ref_root = args[0] if args else (os.environ.get("SLEDGEHAMR_REF_ROOT") or
                                     os.path.join(os.path.dirname(ROOT), "reference"))
    subprocess.run(["sh", os.path.join(ROOT, "oracle", "build_ref.sh"), ref_root], check=True)
    if not only or "spectra" in only:
        spectra_fixtures(ref_root)
        hdf5_format_fixture(ref_root)
    if not only or "evolve" in only:
        evolve_fixtures()
    if not only or "bubbles" in only:
        bubble_fixture()
