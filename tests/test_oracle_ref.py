"""The oracle's restatement against the reference's own code (oracle/_ref,
compiled from the sledgehamr sources): the per-cell headers, and the
integrators rkn.cpp, lsssprk3.cpp and leapfrog.cpp themselves (their
MultiFab Copy / Saxpy / LinComb sequences and FillIntermediatePatch calls
over an AMReX stand-in): bit-for-bit equality."""
import numpy as np
import pytest

from sledgehamr_gb300 import ic


@pytest.mark.parametrize("kind", [0, 1, 2, 3])
@pytest.mark.parametrize("order", [1, 2, 3])
def test_stencils_bitwise(oracle, ref, kind, order):
    f = ic.normal(kind * 10 + order, 12 ** 3).reshape(12, 12, 12)
    assert np.array_equal(oracle.stencil(kind, order, f, 0.3), ref.stencil(kind, order, f, 0.3))


def _axion_state(N=12, seed=1):
    st = ic.axion_string_ic(N, 3.0, kmax=6.0, seed=seed)
    st[2:] = 0.3 * ic.axion_string_ic(N, 3.0, kmax=6.0, seed=seed + 7)[:2]
    return st


@pytest.mark.parametrize("project", ["AxionStrings", "MinimalExample"])
@pytest.mark.parametrize("integ", [10, 11, 21, 22])
def test_evolve_bitwise(oracle, ref, project, integ):
    st = _axion_state()
    kw = dict(t0=1.0, dt=0.0625, dx=0.25, nsteps=3, nghost=2, max_grid=6)
    assert np.array_equal(oracle.evolve_periodic(project, integ, st, **kw),
                          ref.evolve_periodic(project, integ, st, **kw))


def test_next_to_minimal_matches_lap2_variant(oracle):
    """AxionStringsLap2 with (lambda, 0.56233) is NextToMinimalExample."""
    st = _axion_state()
    kw = dict(t0=1.0, dt=0.0625, dx=0.25, nsteps=2, nghost=2, params=[0.7, 0.56233])
    assert np.array_equal(oracle.evolve_periodic("NextToMinimalExample", 21, st, **kw),
                          oracle.evolve_periodic("AxionStringsLap2", 21, st, **kw))


def test_fopt_gw_leapfrog_bitwise(oracle, ref):
    from tests.golden.make_golden import fopt_params
    s = np.zeros((14, 10, 10, 10))
    s[0] = 0.8 * ic.gaussian_field(10, 2.5, 9.0, 1)
    s[2:8] = 0.05 * np.stack([ic.gaussian_field(10, 2.5, 9.0, 5 + q) for q in range(6)])
    kw = dict(t0=0.0, dt=0.05, dx=0.25, nsteps=3, nghost=2, params=fopt_params(),
              gw_params=[0.0, 1.0], with_gw=True)
    assert np.array_equal(oracle.evolve_periodic("FirstOrderPhaseTransition", 11, s, **kw),
                          ref.evolve_periodic("FirstOrderPhaseTransition", 11, s, **kw))


def test_rhs_gw_and_dissipation_bitwise(oracle, ref):
    st = _axion_state()
    s16 = np.zeros((16,) + st.shape[1:])
    s16[:4] = st
    s16[4:] = 0.1 * ic.normal(9, 12 * 12 ** 3).reshape((12,) + st.shape[1:])
    for proj, s, kw in (("AxionStrings", s16, dict(with_gw=True)),
                        ("MinimalExample", st, dict(ko_order=2, ko_strength=[.1, .2, .3, .4])),
                        ("MinimalExample", st, dict(ko_order=3, ko_strength=[.1, .2, .3, .4]))):
        a = oracle.fill_rhs(proj, s, 1.5, 0, 0.0625, 0.25, nghost=3, **kw)
        b = ref.fill_rhs(proj, s, 1.5, 0, 0.0625, 0.25, nghost=3, **kw)
        assert np.array_equal(a, b)


def test_tag_bitwise(oracle, ref):
    st = _axion_state(16, 3)
    te = np.abs(ic.normal(2, st.size).reshape(st.shape)) * 1e-3
    crit = np.array([1.5e-3, 2e-3, 1e-2, 1e-2])
    for t in (te, None):
        m1, c1 = oracle.tag("AxionStrings", st, t, 1.0, 0, 0.0625, 0.25, te_crit=crit,
                            max_grid=8)
        m2, c2 = ref.tag("AxionStrings", st, t, 1.0, 0, 0.0625, 0.25, te_crit=crit, max_grid=8)
        assert np.array_equal(m1, m2) and np.array_equal(c1, c2)
        assert m1.sum() > 0


def test_avgdown_te_bitwise(oracle, ref):
    import ctypes as C
    fine = ic.normal(5, 4 * 8 ** 3).reshape(4, 8, 8, 8)
    crse = ic.normal(6, 4 * 4 ** 3).reshape(4, 4, 4, 4)
    c1, t1 = oracle.avgdown_te(fine, crse, np.zeros_like(fine))
    c2, t2 = crse.copy(), np.zeros_like(fine)
    ref.lib.ref_avgdown_te_kernel(4, 4, C.c_void_p(fine.ctypes.data), C.c_void_p(c2.ctypes.data),
                                  C.c_void_p(t2.ctypes.data))
    assert np.array_equal(c1, c2) and np.array_equal(t1, t2)


@pytest.mark.parametrize("project,integ", [("AxionStrings", 21), ("AxionStrings", 22),
                                           ("AxionStrings", 11), ("AxionStrings", 10),
                                           ("MinimalExample", 10), ("MinimalExample", 21)])
def test_integrator_sequencing_equals_the_reference_integrators(oracle, project, integ):
    from tests.oracle_lib import ref_int_evolve, ref_integrators_available
    if not ref_integrators_available():
        pytest.skip("oracle/_ref/libshref_int.so not built (sledgehamr sources absent)")
    st = _axion_state()
    kw = dict(t0=1.0, dt=0.0625, dx=0.25, nsteps=4, nghost=2)
    assert np.array_equal(oracle.evolve_periodic(project, integ, st, **kw),
                          ref_int_evolve(project, integ, st, **kw))


@pytest.mark.parametrize("integ", [11, 21])
def test_integrator_sequencing_with_gw_tensor_equals_the_reference(oracle, integ):
    from tests.golden.make_golden import fopt_params
    from tests.oracle_lib import ref_int_evolve, ref_integrators_available
    if not ref_integrators_available():
        pytest.skip("oracle/_ref/libshref_int.so not built (sledgehamr sources absent)")
    s = np.zeros((14, 10, 10, 10))
    s[0] = 0.8 * ic.gaussian_field(10, 2.5, 9.0, 1)
    s[1] = 0.2 * ic.gaussian_field(10, 2.5, 9.0, 2)
    s[2:8] = 0.05 * np.stack([ic.gaussian_field(10, 2.5, 9.0, 5 + q) for q in range(6)])
    kw = dict(t0=0.0, dt=0.05, dx=0.25, nsteps=3, nghost=2, params=fopt_params(),
              gw_params=[0.0, 1.0], with_gw=True)
    assert np.array_equal(oracle.evolve_periodic("FirstOrderPhaseTransition", integ, s, **kw),
                          ref_int_evolve("FirstOrderPhaseTransition", integ, s, **kw))


@pytest.mark.parametrize("P,ptype", [(8, 2), (12, 1), (10, 3)])
def test_gw_lambda_equals_the_reference_header(oracle, P, ptype):
    """The oracle's Lambda_ijlm (gw_lambda) equals the reference's own
    gw_GetLambda / gw_GetProjection (source/gravitational_waves.h:101-133,
    compiled into oracle/_ref) on every k-cell and (i, j, l, m)."""
    import ctypes as C

    from tests.oracle_lib import ORACLE_SO, REF_INT_SO, ref_integrators_available
    if not ref_integrators_available():
        pytest.skip("oracle/_ref/libshref_int.so not built (sledgehamr sources absent)")
    n = 81 * (P // 2 + 1) * P * P
    a, b = np.empty(n), np.empty(n)
    itk = oracle.index_to_k(P, ptype)
    olib, rlib = C.CDLL(ORACLE_SO), C.CDLL(REF_INT_SO)
    assert olib.orc_gw_lambda_table(P, ptype, C.c_void_p(a.ctypes.data)) == 0
    assert rlib.ref_gw_lambda_table(P, C.c_void_p(itk.ctypes.data),
                                    C.c_void_p(b.ctypes.data)) == 0
    assert np.array_equal(a, b)
    assert np.abs(a).max() > 0.5
