"""Pools and the serving loop: a run's result does not depend on what else
shares the pool or when it was admitted (bitwise, the per-cell arithmetic
of a member is independent of the batch), admission follows free memory,
and the FP32+Kahan serving results stay close to FP64."""
import numpy as np
import pytest

import sledgehamr_gb300 as sh
from sledgehamr_gb300 import ic

pytestmark = pytest.mark.gpu

Q = (-1.0, 1.6, -1.0, 0.0)


def wall_profile(inv_dx, Lcut, radius=2.0, width=1.0, gamma=1.5, amplitude=1.0):
    nb = int(Lcut * inv_dx) + 2
    r = np.arange(nb) / inv_dx
    x = (r - radius) * gamma / width
    v = np.sqrt(1.0 - 1.0 / gamma ** 2)
    return np.stack([0.5 * amplitude * (1 - np.tanh(x)),
                     0.5 * amplitude * v * gamma / width / np.cosh(x) ** 2])


def request(N, d, seed):
    """Two bubbles a distance d apart along x in a periodic box."""
    L = 2.0 * d + 8.0
    dx = L / N
    c = np.array([[L / 2 - d / 2, L / 2, L / 2], [L / 2 + d / 2, L / 2, L / 2]])
    c[:, 1:] += np.random.default_rng(seed).uniform(-0.5, 0.5, 2)
    inv_dx, Lcut = 8.0, 6.0
    return dict(N=N, dx=dx, dt=0.2 * dx, t_end=0.5 * d, params=Q, centres=c,
                profile=wall_profile(inv_dx, Lcut), inv_dx=inv_dx, Lcut=Lcut)


def run_alone(ctx, rq, prec=sh.PREC_FP32_KAHAN):
    """The request's run in a one-member fixed ensemble."""
    with sh.Ensemble(ctx, sh.FAMILY_FOPT_GW, prec, [rq["N"]], [rq["dx"]], list(rq["params"])) as E:
        E.add_bubbles(0, rq["centres"], rq["profile"], rq["inv_dx"], rq["Lcut"])
        nsteps = int(np.ceil(rq["t_end"] / rq["dt"] - 1e-9))
        E.step(rq["dt"], nsteps)
        return E.gw_spectrum(0, zero_padding=1, projection_type=2, unbinned=False), E.read(0)


def test_pool_members_match_fixed_ensemble_bitwise(ctx):
    P = sh.Ensemble.pool(ctx, sh.FAMILY_FOPT_GW, sh.PREC_FP32_KAHAN, capacity_cells=80000)
    reqs = [request(16, 6.0, 1), request(24, 8.0, 2), request(32, 5.0, 3)]
    slots = []
    for rq in reqs[:2]:
        s = P.admit(rq["N"], rq["dx"], rq["params"], rq["dt"])
        assert s is not None
        P.add_bubbles(s, rq["centres"], rq["profile"], rq["inv_dx"], rq["Lcut"])
        slots.append(s)
    P.step(0.0, 3)
    # the third joins late: run it for its own number of steps afterwards
    s3 = P.admit(reqs[2]["N"], reqs[2]["dx"], reqs[2]["params"], reqs[2]["dt"])
    assert s3 is not None
    P.add_bubbles(s3, reqs[2]["centres"], reqs[2]["profile"], reqs[2]["inv_dx"],
                  reqs[2]["Lcut"])
    P.step(0.0, 4)
    for s, rq, n in ((slots[0], reqs[0], 7), (slots[1], reqs[1], 7), (s3, reqs[2], 4)):
        with sh.Ensemble(ctx, sh.FAMILY_FOPT_GW, sh.PREC_FP32_KAHAN, [rq["N"]], [rq["dx"]],
                         list(rq["params"])) as E:
            E.add_bubbles(0, rq["centres"], rq["profile"], rq["inv_dx"], rq["Lcut"])
            E.step(rq["dt"], n)
            assert np.array_equal(P.read(s), E.read(0))
    P.close()


def test_pool_admission_follows_free_memory(ctx):
    P = sh.Ensemble.pool(ctx, sh.FAMILY_FOPT_GW, sh.PREC_FP32, capacity_cells=3 * 16 ** 3)
    a = P.admit(16, 0.5)
    b = P.admit(16, 0.5)
    c = P.admit(16, 0.5)
    assert None not in (a, b, c)
    assert P.admit(8, 0.5) is None  # full
    P.release(b)
    assert P.admit(24, 0.5) is None  # 24^3 > the freed extent
    d = P.admit(8, 0.5)
    assert d is not None
    P.release(d)
    P.release(a)  # a and b merge into one extent of 2 * 16^3 cells
    assert P.pool_info()["largest_free"] == 2 * 16 ** 3
    assert P.admit(20, 0.5) is not None
    P.close()


def serve_all(ctx, reqs, capacity, arrivals=None, prec=sh.PREC_FP32_KAHAN):
    """Submit reqs (at the given iteration numbers) and run until all are
    done; returns the spectra in submission order and the server info."""
    S = sh.Server(ctx, prec, capacity_cells=capacity)
    arrivals = arrivals or [0] * len(reqs)
    ids = [None] * len(reqs)
    it = 0
    while True:
        for q, rq in enumerate(reqs):
            if ids[q] is None and arrivals[q] <= it:
                ids[q] = S.submit(rq["N"], rq["dx"], rq["dt"], rq["t_end"], rq["params"],
                                  rq["centres"], rq["profile"], rq["inv_dx"], rq["Lcut"])
        running, queued, _ = S.step()
        it += 1
        if all(i is not None for i in ids) and running == 0 and queued == 0:
            break
        assert it < 100000
    out = [S.result(i) for i in ids]
    info = S.info()
    S.close()
    return out, info


def test_served_results_equal_alone_and_in_the_mix(ctx):
    reqs = [request(16, 6.0, 1), request(24, 8.0, 2), request(32, 5.0, 3), request(16, 9.0, 4),
            request(24, 4.0, 5)]
    alone = [run_alone(ctx, rq)[0] for rq in reqs]
    # everything at once with room for all
    mix, _ = serve_all(ctx, reqs, capacity=200000)
    # staggered arrivals into a pool that holds about two runs at a time
    stag, info = serve_all(ctx, reqs, capacity=2 * 32 ** 3, arrivals=[0, 3, 5, 9, 20])
    for (ba, ka), (bm, km), (bs, ks) in zip(alone, mix, stag):
        assert np.array_equal(ka, km) and np.array_equal(ka, ks)
        assert np.array_equal(ba, bm)
        assert np.array_equal(ba, bs)
    assert info["cell_updates"] > 0


def test_served_fp32_spectra_close_to_fp64(ctx):
    """FP32+Kahan against FP64 on the same requests: total GW power within
    1%, every bin holding at least 1e-3 of the peak within 5%."""
    reqs = [request(24, 8.0, 7), request(32, 10.0, 8)]
    s32, _ = serve_all(ctx, reqs, capacity=100000, prec=sh.PREC_FP32_KAHAN)
    s64, _ = serve_all(ctx, reqs, capacity=100000, prec=sh.PREC_FP64)
    for (b32, _), (b64, _) in zip(s32, s64):
        assert abs(b32.sum() - b64.sum()) <= 1e-2 * b64.sum()
        big = b64 >= 1e-3 * b64.max()
        assert np.all(np.abs(b32[big] - b64[big]) <= 5e-2 * b64[big])


def test_fp64_pool_member_matches_oracle(ctx):
    """A member of an FP64 pool (own N, dx and step) follows the drop-in
    FirstOrderPhaseTransition leapfrog of the oracle to 1e-12."""
    from tests.conftest import rel_l2
    from tests.oracle_lib import Oracle, oracle_add_bubbles
    P = sh.Ensemble.pool(ctx, sh.FAMILY_FOPT_GW, sh.PREC_FP64, capacity_cells=60000)
    runs = []
    for rq in (request(16, 6.0, 1), request(24, 8.0, 2)):
        s = P.admit(rq["N"], rq["dx"], rq["params"], rq["dt"])
        P.add_bubbles(s, rq["centres"], rq["profile"], rq["inv_dx"], rq["Lcut"])
        runs.append((s, rq))
    P.step(0.0, 6)
    orc = Oracle()
    for s, rq in runs:
        N = rq["N"]
        st = oracle_add_bubbles(np.zeros((14, N, N, N)), rq["centres"], rq["profile"],
                                rq["inv_dx"], rq["Lcut"], rq["dx"])
        q = rq["params"]
        ref = orc.evolve_periodic("FirstOrderPhaseTransition", sh.LEAPFROG, st, t0=0.0,
                                  dt=rq["dt"], dx=rq["dx"], nsteps=6,
                                  params=[0.0, q[0], q[1], q[2], 0.0, 0.0, 0.0], with_gw=True,
                                  nghost=2)
        out = P.read(s)
        assert rel_l2(out, ref) <= 1e-12
        assert rel_l2(out[2:], ref[2:]) <= 1e-12
    P.close()


def amr_request(N, d, seed, max_level=1):
    rq = request(N, d, seed)
    rq.update(max_level=max_level, te_crit=(1e-3, 1e-3), regrid_dt=0.0)
    return rq


def run_amr_alone(ctx, rq, precision=sh.PREC_FP64):
    """The AMR request's hierarchy built directly: FirstOrderPhaseTransition
    + GW, leapfrog, TruncationModifier maxima from level 0, bubbles on
    level 0 of a zero state, ceil(t_end / dt) coarse steps, spectrum of
    level 0; levels of the given precision (FP32 servers run FP32 + Kahan
    hierarchies)."""
    q = rq["params"]
    cfg = sh.amr_config("FirstOrderPhaseTransition", precision=precision, N0=rq["N"],
                        L=rq["N"] * rq["dx"],
                        cfl=rq["dt"] / rq["dx"], t_start=0.0, nghost=2,
                        max_level=rq["max_level"], blocking_factor=8, max_grid_size=32,
                        n_error_buf=1, regrid_dt=rq["regrid_dt"],
                        te_crit=list(rq["te_crit"]) + [1e300] * 12,
                        params=[0.0, q[0], q[1], q[2], 0.0, 0.0, 0.0], with_gw=1,
                        integrator=sh.LEAPFROG, params_mod_norm0=1)
    A = sh.Amr(ctx, cfg, None)
    A.level(0).add_bubbles(rq["centres"], rq["profile"], rq["inv_dx"], rq["Lcut"], rq["dx"])
    A.step(int(np.ceil(rq["t_end"] / rq["dt"] - 1e-9)))
    out = A.level(0).gw_spectrum(zero_padding=1, projection_type=2, unbinned=False)
    finest = A.info()["finest"]
    A.close()
    return out, finest


def submit_all(S, reqs):
    return [S.submit(rq["N"], rq["dx"], rq["dt"], rq["t_end"], rq["params"], rq["centres"],
                     rq["profile"], rq["inv_dx"], rq["Lcut"], max_level=rq.get("max_level", 0),
                     te_crit=rq.get("te_crit", (1e300, 1e300)),
                     regrid_dt=rq.get("regrid_dt", 0.0)) for rq in reqs]


@pytest.mark.parametrize("prec", [sh.PREC_FP32_KAHAN, sh.PREC_FP64])
def test_amr_requests_equal_alone_and_in_the_mix(ctx, prec):
    """A request with a refinement level runs as its own hierarchy, of the
    server's precision: its spectrum equals the hierarchy's run outside the
    server bitwise, alone and beside single-level requests in the same
    server."""
    ra = amr_request(32, 6.0, 11)
    alone, finest = run_amr_alone(ctx, ra, prec)
    assert finest >= 1  # the walls were refined
    mixes = ([ra], [request(16, 6.0, 1), ra, request(24, 8.0, 2)])
    for reqs in mixes:
        S = sh.Server(ctx, prec, capacity_cells=60000)
        ids = submit_all(S, reqs)
        it = 0
        while True:
            running, queued, _ = S.step()
            it += 1
            if running == 0 and queued == 0:
                break
            assert it < 10000
        b, k = S.result(ids[reqs.index(ra)])
        assert np.array_equal(b, alone[0]) and np.array_equal(k, alone[1])
        assert S.info()["cell_updates"] > 0
        S.close()
