"""CUDA path (through the C ABI) against the oracle and the golden fixtures.

Tolerances: fields within 1e-12 relative L2 after up to 10 steps, tag masks
and tag counts bit-exact, average-down and truncation errors bit-exact, GW
spectra within 1e-10 relative per bin.
"""
import numpy as np
import pytest

import sledgehamr_gb300 as sh
from sledgehamr_gb300 import ic
from tests.conftest import golden, rel_l2

pytestmark = pytest.mark.gpu

FIELD_TOL = 1e-12


def axion_state(N=16, L=4.0, seed=3):
    st = ic.axion_string_ic(N, L, kmax=6.0, seed=seed)
    st[2:] = 0.3 * ic.axion_string_ic(N, L, kmax=6.0, seed=seed + 1)[:2]
    return st


@pytest.mark.parametrize("project,integ,nghost", [
    ("AxionStringsLap1", sh.RKN4, 1),
    ("AxionStringsLap2", sh.RKN4, 2),
    ("AxionStringsLap3", sh.RKN4, 3),
    ("AxionStrings", sh.RKN4, 2),
    ("AxionStrings", sh.RKN5, 2),
    ("AxionStrings", sh.LSSSPRK3, 2),
    ("AxionStrings", sh.LEAPFROG, 2),
    ("NextToMinimalExample", sh.RKN4, 2),
    ("MinimalExample", sh.LSSSPRK3, 2),
])
@pytest.mark.parametrize("max_grid", [0, 8])
def test_evolve_vs_oracle(ctx, oracle, project, integ, nghost, max_grid):
    st = axion_state()
    params = [0.8, 0.3] if project.startswith("AxionStringsLap") else [0.8]
    kw = dict(t0=1.0, dt=0.0625, dx=0.25, nsteps=10, params=params, nghost=nghost,
              max_grid=max_grid)
    gpu = ctx.evolve_periodic(project, integ, st, **kw)
    ref = oracle.evolve_periodic(project, integ, st, **kw)
    assert rel_l2(gpu, ref) <= FIELD_TOL


@pytest.mark.parametrize("name", ["ref_axion_rkn4", "ref_axion_rkn5", "ref_minimal_ssprk3",
                                  "ref_axion_leapfrog"])
def test_evolve_vs_golden(ctx, name):
    g = golden(name)
    out = ctx.evolve_periodic(str(g["project"]), int(g["integrator"]), g["state_in"],
                              t0=float(g["t0"]), dt=float(g["dt"]), dx=float(g["dx"]),
                              nsteps=int(g["nsteps"]), nghost=int(g["nghost"]))
    assert rel_l2(out, g["state_out"]) <= FIELD_TOL


def test_fopt_gw_leapfrog_vs_golden(ctx):
    g = golden("ref_fopt_gw_leapfrog")
    out = ctx.evolve_periodic("FirstOrderPhaseTransition", sh.LEAPFROG, g["state_in"], t0=0.0,
                              dt=float(g["dt"]), dx=float(g["dx"]), nsteps=int(g["nsteps"]),
                              nghost=2, params=g["params"], gw_params=g["gw_params"],
                              with_gw=True)
    assert rel_l2(out, g["state_out"]) <= FIELD_TOL
    # the tensor block separately (it is much smaller than the scalar)
    assert rel_l2(out[2:], g["state_out"][2:]) <= FIELD_TOL


def test_fopt_gw_all_integrators_vs_oracle(ctx, oracle):
    g = golden("ref_fopt_gw_leapfrog")
    for integ in (sh.RKN4, sh.LSSSPRK3, sh.LEAPFROG):
        kw = dict(t0=0.0, dt=0.05, dx=0.25, nsteps=6, nghost=2, params=g["params"],
                  gw_params=g["gw_params"], with_gw=True, max_grid=6)
        a = ctx.evolve_periodic("FirstOrderPhaseTransition", integ, g["state_in"], **kw)
        b = oracle.evolve_periodic("FirstOrderPhaseTransition", integ, g["state_in"], **kw)
        assert rel_l2(a, b) <= FIELD_TOL
        assert rel_l2(a[2:], b[2:]) <= FIELD_TOL


def test_user_tableau_equals_rkn4(ctx):
    # RKN4 written as a user tableau: nodes, bbar, b, lower triangle
    tab = [0.0, 0.5, 1.0, 1 / 6, 1 / 3, 0.0, 1 / 6, 4 / 6, 1 / 6,
           0.0, 1 / 8, 0.0, 0.0, 0.5, 0.0]
    st = axion_state()
    kw = dict(t0=1.0, dt=0.0625, dx=0.25, nsteps=4, nghost=2)
    a = ctx.evolve_periodic("AxionStrings", sh.RKN_TABLEAU, st, tableau=tab, **kw)
    b = ctx.evolve_periodic("AxionStrings", sh.RKN4, st, **kw)
    assert np.array_equal(a, b)


def test_leapfrog_stale_momenta(ctx, oracle):
    """The second force evaluation reads the momenta the new time level held
    before the step; with a velocity-dependent Rhs that is observable."""
    st = axion_state()
    init_new = axion_state(seed=9)
    kw = dict(t0=1.0, dt=0.0625, dx=0.25, nsteps=3, nghost=2, init_new=init_new)
    a = ctx.evolve_periodic("AxionStrings", sh.LEAPFROG, st, **kw)
    b = oracle.evolve_periodic("AxionStrings", sh.LEAPFROG, st, **kw)
    assert rel_l2(a, b) <= FIELD_TOL


def test_rhs_gw_hook_and_dissipation_vs_golden(ctx):
    g = golden("ref_rhs")
    t, dt, dx = float(g["time"]), float(g["dt"]), float(g["dx"])
    N = g["state16"].shape[-1]
    lv = sh.Level.periodic(ctx, "AxionStrings", N, 3, with_gw=True)
    lv.write(g["state16"])
    lv.fill_patch()
    r = lv.rhs(t, 0, dt, dx).reshape(g["rhs_axion_gw"].shape)
    assert rel_l2(r, g["rhs_axion_gw"]) <= FIELD_TOL
    lv.close()
    lv = sh.Level.periodic(ctx, "MinimalExample", N, 3)
    lv.write(g["state4"])
    lv.fill_patch()
    for order, key in ((2, "rhs_ko2"), (3, "rhs_ko3")):
        r = lv.rhs(t, 0, dt, dx, ko_order=order, ko_strength=[0.1, 0.2, 0.3, 0.4])
        assert rel_l2(r.reshape(g[key].shape), g[key]) <= FIELD_TOL
    lv.close()


def boxes_to_canonical(flat, boxes, N):
    out = np.empty((N, N, N), dtype=flat.dtype)
    off = 0
    for lo, hi in boxes:
        nx, ny, nz = (hi[0] - lo[0] + 1, hi[1] - lo[1] + 1, hi[2] - lo[2] + 1)
        out[lo[2]:hi[2] + 1, lo[1]:hi[1] + 1, lo[0]:hi[0] + 1] = \
            flat[off:off + nx * ny * nz].reshape(nz, ny, nx)
        off += nx * ny * nz
    return out


@pytest.mark.parametrize("use_te", [True, False])
def test_tag_vs_golden(ctx, use_te):
    g = golden("ref_tag")
    st, te = g["state"], g["te"]
    N = st.shape[-1]
    lv = sh.Level.periodic(ctx, "AxionStrings", N, 2, max_grid=8)
    lv.write(st)
    lv.fill_patch()
    lv.write(te, which=sh.SH_OLD)
    mask, counts, lst = lv.tag(1.0, 0, float(g["dt"]), float(g["dx"]), use_te=use_te,
                               te_crit=g["te_crit"], want_list=True)
    m = boxes_to_canonical(mask, lv.boxes, N)
    if use_te:
        assert np.array_equal(m, g["mask"]) and np.array_equal(counts, g["counts"])
    else:
        assert np.array_equal(m, g["mask_user"])
        assert np.array_equal(counts[:2], g["counts_user"][:2])
    assert np.array_equal(lst, np.flatnonzero(mask))
    lv.close()


def test_tag_evolved_state_vs_oracle(ctx, oracle):
    """Tags of a state evolved on the GPU, computed by GPU and oracle on the
    same (GPU) field values."""
    N = 32
    st = ic.axion_string_ic(N, 8.0, kmax=3.0, seed=5)
    st = ctx.evolve_periodic("AxionStringsLap1", sh.RKN4, st, t0=0.5, dt=0.0625, dx=0.25,
                             nsteps=8, params=[1.0, 0.0], nghost=1)
    lv = sh.Level.periodic(ctx, "AxionStringsLap1", N, 1)
    lv.write(st)
    lv.fill_patch()
    mask, counts, _ = lv.tag(1.0, 0, 0.0625, 0.25)
    m2, c2 = oracle.tag("AxionStringsLap1", st, None, 1.0, 0, 0.0625, 0.25)
    assert mask.sum() > 0
    assert np.array_equal(mask.reshape(N, N, N), m2) and counts[0] == c2[0]
    lv.close()


def test_average_down_te_vs_oracle(ctx, oracle):
    g = golden("ref_avgdown_te")
    fine_lv = sh.Level.periodic(ctx, "AxionStrings", 16, 2)
    crse_lv = sh.Level.periodic(ctx, "AxionStrings", 8, 2)
    fine_lv.write(g["fine"])
    fine_lv.write(np.zeros_like(g["fine"]), which=sh.SH_OLD)
    crse_lv.write(g["crse_in"])
    sh.average_down_te(ctx, fine_lv, crse_lv)
    assert np.array_equal(crse_lv.read(), g["crse_out"])
    assert np.array_equal(fine_lv.read(sh.SH_OLD), g["te_out"])
    crse_lv.write(g["crse_in"])
    sh.average_down(ctx, fine_lv, crse_lv)
    assert np.array_equal(crse_lv.read(), oracle.average_down(g["fine"]))
    fine_lv.close()
    crse_lv.close()


@pytest.mark.parametrize("unbinned", [True, False])
@pytest.mark.parametrize("zp", [1, 2])
def test_gw_spectrum_vs_oracle(ctx, oracle, unbinned, zp):
    N = 16
    s = np.zeros((14, N, N, N))
    for q in range(12):
        s[2 + q] = ic.gaussian_field(N, 4.0, 8.0, 100 + q)
    lv = sh.Level.periodic(ctx, "FirstOrderPhaseTransition", N, 2, max_grid=8, with_gw=True)
    lv.write(s)
    bins, ks = lv.gw_spectrum(zero_padding=zp, projection_type=2, unbinned=unbinned)
    comps = [s[2 + 6 + d] for d in (0, 3, 4, 1, 5, 2)]  # du_xx du_xy du_xz du_yy du_yz du_zz
    rb, rks = oracle.gw_spectrum(np.stack(comps), zero_padding=zp, projection_type=2,
                                 unbinned=unbinned)
    assert np.array_equal(ks, rks)
    scale = np.abs(rb).max()
    assert np.all(np.abs(bins - rb) <= 1e-10 * np.abs(rb) + 1e-14 * scale)
    lv.close()


def test_runs_are_bitwise_deterministic(ctx):
    st = axion_state(32, 8.0)
    kw = dict(t0=1.0, dt=0.0625, dx=0.25, nsteps=3, nghost=2, max_grid=16)
    a = ctx.evolve_periodic("AxionStrings", sh.RKN4, st, **kw)
    b = ctx.evolve_periodic("AxionStrings", sh.RKN4, st, **kw)
    assert np.array_equal(a, b)


@pytest.mark.parametrize("project,integ,nghost,N", [
    ("AxionStringsLap1", sh.RKN4, 1, 16),
    ("AxionStringsLap2", sh.RKN5, 2, 16),
    ("AxionStringsLap3", sh.LSSSPRK3, 3, 16),
    ("AxionStrings", sh.LEAPFROG, 2, 16),
    ("AxionStringsLap2", sh.RKN4, 2, 20),  # tiles of 20 cells in x, 6 rows
    ("AxionStringsLap1", sh.RKN4, 1, 40),  # a ragged second tile in x
    ("AxionStringsLap3", sh.RKN4, 3, 6),   # ghost depth half the extent
])
def test_one_box_ghost_images_equal_the_fill(ctx, project, integ, nghost, N):
    """A level of one box covering the periodic domain has the stage kernels
    write the periodic images of their outputs into its ghost cells instead
    of a separate fill: the result equals the same level chopped into boxes
    (ghosts filled by copies) bit for bit, and the ghost cells after a step
    equal a fresh fill (the Rhs, which reads them as they are, is unchanged
    by an explicit FillPatch)."""
    L = N / 4.0
    st = axion_state(N, L)
    params = [0.8, 0.3] if project.startswith("AxionStringsLap") else [0.8]
    kw = dict(t0=1.0, dt=0.0625, dx=0.25, nsteps=3, params=params, nghost=nghost)
    one = ctx.evolve_periodic(project, integ, st, max_grid=0, **kw)
    chopped = ctx.evolve_periodic(project, integ, st, max_grid=N // 2, **kw)
    assert np.array_equal(one, chopped)
    lv = sh.Level.periodic(ctx, project, N, nghost)
    assert lv.nbox == 1
    lv.write(st)
    lv.set_time(1.0)
    lv.fill_patch()
    for _ in range(2):
        lv.advance(integ, 0.0625, 0.25, params)
    t = lv.time()[0]
    before = lv.rhs(t, 0, 0.0625, 0.25, params)
    lv.fill_patch()
    after = lv.rhs(t, 0, 0.0625, 0.25, params)
    assert np.array_equal(before, after)
    lv.close()


def test_full_size_translation_invariance(ctx):
    """128^3 (the single-level workload size): a periodic shift of the
    initial state shifts the result exactly."""
    N = 128
    st = ic.axion_string_ic(N, 32.0, kmax=1.0, seed=0)
    kw = dict(t0=0.1, dt=0.0625, dx=0.25, nsteps=4, params=[1.0, 0.0], nghost=1)
    a = ctx.evolve_periodic("AxionStringsLap1", sh.RKN4, st, **kw)
    sh_ = (3, 5, 7)
    b = ctx.evolve_periodic("AxionStringsLap1", sh.RKN4,
                            np.roll(st, sh_, axis=(1, 2, 3)), **kw)
    assert np.array_equal(np.roll(a, sh_, axis=(1, 2, 3)), b)


@pytest.mark.parametrize("precision,integ", [(sh.PREC_FP64, sh.LEAPFROG),
                                             (sh.PREC_FP32_KAHAN, sh.RKN4)])
def test_beyond_2_31_elements_translation_invariance(precision, integ):
    """A level whose buffers hold more than 2^31 elements (832^3 cells, four
    components, 64 boxes of 208^3: the element offsets of the later boxes,
    of their ghost copies and of the canonical-layout moves need 64 bits):
    a periodic shift of the initial state shifts the result of two steps
    exactly, on FP64 and on FP32 + Kahan storage.  The data are made and
    compared on the device (about 125 GB at the peak), so that no host
    array of that size exists; a context of its own returns the level
    memory when the test ends."""
    torch = pytest.importorskip("torch")
    N, mg = 832, 208
    # the device's memory pool keeps what earlier tests freed until a
    # context is destroyed: destroying a fresh one returns it
    sh.Context(0).close()
    torch.cuda.empty_cache()
    free, _ = torch.cuda.mem_get_info()
    if free < 160e9:
        pytest.skip("needs about 160 GB of free device memory")
    ctx = sh.Context(0)
    dx, dt = 0.25, 0.0625
    shift = (3, 5, 7)

    def run(state):
        lv = sh.Level.periodic(ctx, "AxionStringsLap1", N, 1, max_grid=mg,
                               precision=precision)
        assert lv.nbox == 64
        torch.cuda.synchronize()
        lv.write_device(state.data_ptr())
        lv.set_time(1.0)
        for _ in range(2):
            lv.advance(integ, dt, dx, [1.0, 0.0])
        out = torch.empty_like(state)
        lv.read_device(out.data_ptr())
        ctx.synchronize()
        lv.close()
        return out

    g = torch.Generator(device="cuda").manual_seed(5)
    st = 0.5 * torch.randn((4, N, N, N), dtype=torch.float64, device="cuda", generator=g)
    a = run(st)
    st = torch.roll(st, shift, dims=(1, 2, 3))
    b = run(st)
    del st
    ctx.close()
    finite = bool(torch.isfinite(a).all())
    shifted = bool(torch.equal(torch.roll(a, shift, dims=(1, 2, 3)), b))
    del a, b
    torch.cuda.empty_cache()
    assert finite and shifted


def test_full_size_linearity(ctx):
    """lambda = 0 makes the equations linear: doubling the state doubles the
    result exactly."""
    N = 128
    st = ic.axion_string_ic(N, 32.0, kmax=1.0, seed=1)
    kw = dict(t0=0.1, dt=0.0625, dx=0.25, nsteps=3, params=[0.0, 0.0], nghost=1)
    a = ctx.evolve_periodic("AxionStringsLap1", sh.RKN4, st, **kw)
    b = ctx.evolve_periodic("AxionStringsLap1", sh.RKN4, 2.0 * st, **kw)
    assert np.array_equal(2.0 * a, b)


def test_errors_are_reported_not_raised_on_device(ctx):
    st = axion_state()
    with pytest.raises(sh.ShError) as e:
        ctx.evolve_periodic("AxionStrings", sh.RKN4, st, t0=1.0, dt=0.06, dx=0.25, nsteps=1,
                            nghost=1)  # stencil reach 2 > nghost
    assert e.value.code == -1
    with pytest.raises(sh.ShError) as e:
        ctx.evolve_periodic("AxionStrings", 3, st, t0=1.0, dt=0.06, dx=0.25, nsteps=1)
    assert e.value.code == -5
    with pytest.raises(sh.ShError):
        sh.Level.periodic(ctx, "MinimalExample", 16, 2, with_gw=True)
    # the context is still usable
    out = ctx.evolve_periodic("AxionStrings", sh.RKN4, st, t0=1.0, dt=0.06, dx=0.25, nsteps=1)
    assert np.isfinite(out).all()


def test_level_errors_overlap_and_nesting(ctx):
    """Overlapping boxes are rejected at level creation, and a coarse level
    that does not cover the cells to interpolate is rejected by the fill and
    by the coarse link."""
    with pytest.raises(sh.ShError):
        sh.Level(ctx, "AxionStringsLap1", [((0, 0, 0), (15, 15, 15)), ((8, 8, 8), (23, 23, 23))],
                 (0, 0, 0), (31, 31, 31), 1)
    coarse = sh.Level(ctx, "AxionStringsLap1", [((0, 0, 0), (7, 7, 7))], (0, 0, 0),
                      (15, 15, 15), 1)
    fine = sh.Level(ctx, "AxionStringsLap1", [((16, 16, 16), (23, 23, 23))], (0, 0, 0),
                    (31, 31, 31), 1)
    import ctypes as C
    rc = ctx.lib.sh_level_fill_from(ctx.h, fine.h, sh.SH_NEW, None, sh.SH_NEW, coarse.h,
                                    C.c_double(0.0))
    assert rc != 0 and "nested" in ctx.lib.sh_ctx_last_error(ctx.h).decode()
    rc = ctx.lib.sh_level_set_coarse(ctx.h, fine.h, coarse.h)
    assert rc != 0 and "nested" in ctx.lib.sh_ctx_last_error(ctx.h).decode()
    fine.close()
    coarse.close()


def test_level_reduce_matches_numpy_and_is_reproducible(ctx):
    """sh_level_reduce over the valid cells of a multi-box level: norm0,
    min and max exact, sums within 1e-13 of numpy's, every result the same
    bit for bit on a second call."""
    N = 48
    st = np.random.default_rng(3).normal(size=(4, N, N, N)) * np.array([1., 1e-3, 10., 1.])[:, None, None, None]
    lv = sh.Level.periodic(ctx, "AxionStringsLap2", N, 2, max_grid=16)
    lv.write(st)
    ops = {sh.REDUCE_MAX_ABS: lambda a: np.abs(a).max(), sh.REDUCE_MIN: np.min,
           sh.REDUCE_MAX: np.max, sh.REDUCE_SUM: np.sum, sh.REDUCE_SUM_SQ: lambda a: (a * a).sum()}
    for c in range(4):
        for op, f in ops.items():
            got = lv.reduce(op, c)
            want = float(f(st[c]))
            if op in (sh.REDUCE_SUM, sh.REDUCE_SUM_SQ):
                assert abs(got - want) <= 1e-13 * float(np.abs(st[c]).sum() if op == sh.REDUCE_SUM
                                                        else want)
            else:
                assert got == want
            assert lv.reduce(op, c) == got
    lv.close()
