"""Ensembles (sh_ensemble_*): batched periodic realisations in FP64 and in
FP32 with Kahan-compensated updates, against the oracle.

Tolerances: the FP64 ensemble within 1e-12 relative L2 of the oracle after
10 steps (the per-cell arithmetic is the projects' own, reordered); string
counts of one state bit-exact against the oracle's tags; GW spectra within
1e-10 per bin.  The FP32 forms are checked against the FP64 oracle with the
error bounds written at each test (FP32 rounding of the stencils, about
1e-6 relative per step, growing with the number of steps).
"""
import numpy as np
import pytest

import sledgehamr_gb300 as sh
from sledgehamr_gb300 import ic
from tests.conftest import rel_l2

pytestmark = pytest.mark.gpu

FIELD_TOL = 1e-12


def axion_state(N, L, seed):
    kmax = 0.5 * np.pi * N / L  # half the Nyquist wavenumber
    st = ic.axion_string_ic(N, L, kmax=kmax, seed=seed)
    st[2:] = 0.3 * ic.axion_string_ic(N, L, kmax=0.5 * kmax, seed=seed + 1)[:2]
    return st


def fopt_state(N, L, seed):
    s = np.zeros((14, N, N, N))
    kmax = 0.5 * np.pi * N / L
    s[0] = 0.5 + 0.3 * ic.gaussian_field(N, L, kmax, seed)
    s[1] = 0.1 * ic.gaussian_field(N, L, kmax, seed + 1)
    for q in range(12):
        s[2 + q] = 1e-3 * ic.gaussian_field(N, L, kmax, seed + 2 + q)
    return s


AX_CASES = [(sh.FAMILY_AXION_LAP1, "AxionStringsLap1"), (sh.FAMILY_AXION_LAP2, "AxionStringsLap2")]


@pytest.mark.parametrize("family,project", AX_CASES)
def test_axion_fp64_vs_oracle_uneven_batch(ctx, oracle, family, project):
    Ns = [16, 24, 8, 32]
    L = 4.0
    lam = [0.8, 1.5, 0.5, 3.0]
    cs = [0.3, 0.0, 0.56233, 0.1]
    dx = [L / n for n in Ns]
    params = np.array([[lam[r], cs[r], 0, 0] for r in range(len(Ns))]).ravel()
    states = [axion_state(n, L, 10 + r) for r, n in enumerate(Ns)]
    t0, dt, nsteps = 1.0, 0.0625 * L / 32, 10
    with sh.Ensemble(ctx, family, sh.PREC_FP64, Ns, dx, params) as E:
        for r, s in enumerate(states):
            E.write(r, s)
        E.set_time(t0)
        E.step(dt, nsteps)
        assert abs(E.time() - (t0 + nsteps * dt)) < 1e-12
        for r, s in enumerate(states):
            ref = oracle.evolve_periodic(project, sh.RKN4, s, t0=t0, dt=dt, dx=dx[r],
                                         nsteps=nsteps, params=[lam[r], cs[r]],
                                         nghost=1 if family == sh.FAMILY_AXION_LAP1 else 2)
            assert rel_l2(E.read(r), ref) <= FIELD_TOL, r


def test_fopt_fp64_vs_oracle(ctx, oracle):
    Ns = [16, 12]
    L = 6.0
    q = [(-0.2, 0.5, -0.6), (-0.1, 0.3, -0.25)]
    dx = [L / n for n in Ns]
    params = np.array([[*q[r], 0.0] for r in range(2)]).ravel()
    states = [fopt_state(n, L, 40 + 20 * r) for r, n in enumerate(Ns)]
    dt, nsteps = 0.05, 10
    with sh.Ensemble(ctx, sh.FAMILY_FOPT_GW, sh.PREC_FP64, Ns, dx, params) as E:
        for r, s in enumerate(states):
            E.write(r, s)
        E.set_time(0.0)
        E.step(dt, nsteps)
        for r, s in enumerate(states):
            ref = oracle.evolve_periodic("FirstOrderPhaseTransition", sh.LEAPFROG, s, t0=0.0,
                                         dt=dt, dx=dx[r], nsteps=nsteps,
                                         params=[0.0, *q[r], 0.0, 0.0, 0.0], with_gw=True,
                                         nghost=2)
            out = E.read(r)
            assert rel_l2(out, ref) <= FIELD_TOL
            assert rel_l2(out[2:], ref[2:]) <= FIELD_TOL


def test_write_read_roundtrip(ctx):
    for prec in (sh.PREC_FP64, sh.PREC_FP32_KAHAN, sh.PREC_FP32):
        s = fopt_state(8, 2.0, 3)
        with sh.Ensemble(ctx, sh.FAMILY_FOPT_GW, prec, [8], [0.25], [0, 0, 0, 0]) as E:
            E.write(0, s)
            back = E.read(0)
        if prec == sh.PREC_FP64:
            assert np.array_equal(back, s)
        else:
            assert np.array_equal(back, s.astype(np.float32).astype(np.float64))


def test_batch_equals_single_realisations_bitwise(ctx):
    Ns = [16, 8, 24]
    dx = [0.25, 0.5, 0.2]
    params = np.array([[1.0, 0.1, 0, 0], [2.0, 0.0, 0, 0], [0.7, 0.3, 0, 0]]).ravel()
    states = [axion_state(n, 4.0, 70 + r) for r, n in enumerate(Ns)]
    for prec in (sh.PREC_FP64, sh.PREC_FP32_KAHAN):
        with sh.Ensemble(ctx, sh.FAMILY_AXION_LAP2, prec, Ns, dx, params) as E:
            for r, s in enumerate(states):
                E.write(r, s)
            E.set_time(1.0)
            E.step(0.01, 5)
            batch = [E.read(r) for r in range(3)]
        for r in range(3):
            with sh.Ensemble(ctx, sh.FAMILY_AXION_LAP2, prec, [Ns[r]], [dx[r]],
                             params[4 * r: 4 * r + 4]) as E1:
                E1.write(0, states[r])
                E1.set_time(1.0)
                E1.step(0.01, 5)
                assert np.array_equal(E1.read(0), batch[r])


@pytest.mark.parametrize("family", [sh.FAMILY_AXION_LAP1, sh.FAMILY_FOPT_GW])
def test_graph_and_tuning_change_nothing(ctx, family):
    """Graph replay and any tile depth give bitwise the same state: the
    per-cell arithmetic does not depend on the tiling."""
    N = 32
    st = axion_state(N, 8.0, 5) if family != sh.FAMILY_FOPT_GW else fopt_state(N, 8.0, 5)
    params = [1.0, 0.0, 0, 0] if family != sh.FAMILY_FOPT_GW else [-0.2, 0.5, -0.6, 0]
    outs = []
    for mode in ("plain", "graph", "tuned", "nz4"):
        with sh.Ensemble(ctx, family, sh.PREC_FP32_KAHAN, [N], [0.25], params) as E:
            E.write(0, st)
            E.set_time(1.0)
            if mode == "graph":
                E.set_graph(True)
            if mode == "tuned":
                nz = E.tune(0.02)
                assert nz in (4, 8, 16, 32, 64)
                assert E.time() == 1.0
            if mode == "nz4":
                assert E.tune(0.02, tile_nz=4) == 4
            E.step(0.02, 7)
            outs.append(E.read(0))
            assert abs(E.time() - (1.0 + 7 * 0.02)) < 1e-12
    for o in outs[1:]:
        assert np.array_equal(o, outs[0])


def test_string_count_matches_oracle_tags(ctx, oracle):
    N = 32
    st = ic.axion_string_ic(N, 8.0, kmax=3.0, seed=5)
    with sh.Ensemble(ctx, sh.FAMILY_AXION_LAP1, sh.PREC_FP64, [N, N], [0.25, 0.25],
                     [1, 0, 0, 0, 1, 0, 0, 0]) as E:
        E.write(0, st)
        E.write(1, np.roll(st, 3, axis=1))
        counts = E.string_count()
    mask, _ = oracle.tag("AxionStringsLap1", st, None, 1.0, 0, 0.0625, 0.25)
    assert counts[0] == int(mask.sum()) > 0
    assert counts[1] == counts[0]


def test_energy_matches_numpy(ctx):
    N = 16
    dx = 0.3
    st = axion_state(N, N * dx, 9)
    lam, c, t = 1.3, 0.2, 1.7

    def grad2(f):
        g = 0.0
        for ax in (1, 2, 3):
            d = (np.roll(f, -1, axis=ax - 1) - np.roll(f, 1, axis=ax - 1)) / (2 * dx)
            g = g + d * d
        return g

    p1, p2, q1, q2 = st
    r2 = p1 * p1 + p2 * p2
    dens = (0.5 * (q1 * q1 + q2 * q2) + 0.5 * (grad2(p1) + grad2(p2)) +
            lam / 4 * t * t * (r2 - 1) ** 2 + lam * c / 2 * r2)
    ref = dens.sum() * dx ** 3
    for prec, tol in ((sh.PREC_FP64, 1e-12), (sh.PREC_FP32_KAHAN, 1e-6)):
        with sh.Ensemble(ctx, sh.FAMILY_AXION_LAP1, prec, [N], [dx], [lam, c, 0, 0]) as E:
            E.write(0, st)
            E.set_time(t)
            e = E.energy()[0]
        assert abs(e - ref) <= tol * abs(ref)


@pytest.mark.parametrize("unbinned", [True, False])
def test_gw_spectrum_vs_oracle(ctx, oracle, unbinned):
    N = 16
    s = fopt_state(N, 4.0, 11)
    for prec, tol in ((sh.PREC_FP64, 1e-10), (sh.PREC_FP32_KAHAN, 1e-5)):
        with sh.Ensemble(ctx, sh.FAMILY_FOPT_GW, prec, [8, N], [0.5, 0.25],
                         [0, 0, 0, 0, -0.2, 0.5, -0.6, 0]) as E:
            E.write(1, s)
            bins, ks = E.gw_spectrum(1, zero_padding=1, projection_type=2, unbinned=unbinned)
        src = s if prec == sh.PREC_FP64 else s.astype(np.float32).astype(np.float64)
        comps = [src[8 + d] for d in (0, 3, 4, 1, 5, 2)]
        rb, rks = oracle.gw_spectrum(np.stack(comps), zero_padding=1, projection_type=2,
                                     unbinned=unbinned)
        assert np.array_equal(ks, rks)
        scale = np.abs(rb).max()
        assert np.all(np.abs(bins - rb) <= tol * np.abs(rb) + 1e-14 * scale)


def test_fp32_kahan_error_vs_fp64_oracle(ctx, oracle):
    """The FP32+Kahan form tracks the FP64 evolution: relative L2 error of the
    fields below 2e-5 after 40 steps of the 2nd-order axion family, and the
    string count within 1% of the FP64 count."""
    N = 32
    L = 16.0
    st = axion_state(N, L, 21)
    dt, nsteps, t0 = 0.05, 40, 1.0
    ref = oracle.evolve_periodic("AxionStringsLap1", sh.RKN4, st, t0=t0, dt=dt, dx=L / N,
                                 nsteps=nsteps, params=[1.0, 0.0], nghost=1)
    errs = {}
    for prec in (sh.PREC_FP32_KAHAN, sh.PREC_FP32):
        with sh.Ensemble(ctx, sh.FAMILY_AXION_LAP1, prec, [N], [L / N], [1, 0, 0, 0]) as E:
            E.write(0, st)
            E.set_time(t0)
            E.step(dt, nsteps)
            errs[prec] = rel_l2(E.read(0), ref)
            cnt = E.string_count()[0]
    with sh.Ensemble(ctx, sh.FAMILY_AXION_LAP1, sh.PREC_FP64, [N], [L / N], [1, 0, 0, 0]) as E:
        E.write(0, ref)
        cref = E.string_count()[0]
    assert errs[sh.PREC_FP32_KAHAN] <= 2e-5
    assert errs[sh.PREC_FP32] <= 1e-4
    assert abs(cnt - cref) <= max(1, 0.01 * cref)


def test_bad_arguments_are_reported(ctx):
    with pytest.raises(sh.ShError):
        sh.Ensemble(ctx, 7, sh.PREC_FP64, [16], [0.25])
    with pytest.raises(sh.ShError):
        sh.Ensemble(ctx, sh.FAMILY_AXION_LAP1, sh.PREC_FP64, [4], [0.25])
    with sh.Ensemble(ctx, sh.FAMILY_AXION_LAP1, sh.PREC_FP64, [16], [0.25]) as E:
        with pytest.raises(sh.ShError):
            E.gw_spectrum(0)
        with pytest.raises(sh.ShError):
            E.step(-1.0)


def test_level_bubbles_bitwise_vs_golden(ctx):
    """sh_level_add_bubbles on a multi-box FOPT + GW level equals the
    reference's AddBubble bit for bit."""
    from tests.conftest import golden
    g = golden("ref_bubbles")
    N = g["state_in"].shape[-1]
    lv = sh.Level.periodic(ctx, "FirstOrderPhaseTransition", N, 2, max_grid=8, with_gw=True)
    lv.write(g["state_in"])
    lv.add_bubbles(g["xyz"], g["profile"], float(g["inv_dx"]), float(g["Lcut"]),
                   float(g["dx"]))
    assert np.array_equal(lv.read(), g["state_out"])
    lv.close()


def test_ensemble_bubbles_vs_golden(ctx):
    from tests.conftest import golden
    g = golden("ref_bubbles")
    N = g["state_in"].shape[-1]
    dx = float(g["dx"])
    for prec in (sh.PREC_FP64, sh.PREC_FP32_KAHAN):
        with sh.Ensemble(ctx, sh.FAMILY_FOPT_GW, prec, [8, N], [0.3, dx],
                         [0, 0, 0, 0, -1, 1.6, -1, 0]) as E:
            E.write(1, g["state_in"])
            E.add_bubbles(1, g["xyz"], g["profile"], float(g["inv_dx"]), float(g["Lcut"]))
            out = E.read(1)
        if prec == sh.PREC_FP64:
            assert np.array_equal(out, g["state_out"])
        else:
            # FP32 storage of the input; the compensated result carries the
            # FP64 sum of the stored input and the bubbles
            from tests.oracle_lib import oracle_add_bubbles
            s32 = g["state_in"].astype(np.float32).astype(np.float64)
            ref = oracle_add_bubbles(s32, g["xyz"], g["profile"], float(g["inv_dx"]),
                                     float(g["Lcut"]), dx)
            assert np.max(np.abs(out - ref)) <= 1e-14 * np.abs(ref).max()


def test_fp32_spectrum_transforms_against_fp64_transforms(ctx):
    """GW spectra of an FP32 + Kahan ensemble with FP32 transforms and TT
    projection (sh_ensemble_set_spectrum_precision) against the FP64 ones of
    the same state: total power within 1e-5, bins holding more than 1e-6 of
    the largest within 1e-3 (FP32 rounding of the transforms, relative to
    the field's norm)."""
    N = 64
    st = fopt_state(N, 16.0, 9)
    with sh.Ensemble(ctx, sh.FAMILY_FOPT_GW, sh.PREC_FP32_KAHAN, [N], [0.25],
                     [-0.2, 0.5, -0.6, 0]) as E:
        E.write(0, st)
        E.step(0.05, 4)
        for unbinned in (False, True):
            a, ka = E.gw_spectrum(0, unbinned=unbinned)
            E.set_spectrum_precision(sh.PREC_FP32)
            b, kb = E.gw_spectrum(0, unbinned=unbinned)
            E.set_spectrum_precision(sh.PREC_FP64)
            assert np.array_equal(ka, kb)
            assert abs(b.sum() - a.sum()) / a.sum() <= 1e-5
            sig = a > 1e-6 * a.max()
            assert np.max(np.abs(b - a)[sig] / a[sig]) <= 1e-3
