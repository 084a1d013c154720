"""Tensor-copy (TMA) staging of the FP32 axion stage kernels
(csrc/sh_fast_tma.cuh) against the register-pipelined kernels and the FP64
oracle, and the bounded wait that guards its copies.

* Both stagings give the same FP32 arithmetic in the same order, so an
  ensemble of mixed sizes (32^3 .. 128^3, including sizes whose rows are
  not a multiple of 32 cells) evolves to bit-identical states, with and
  without compensation, with and without CUDA graphs, for the 7- and the
  13-point Laplacian;
* against the FP64 oracle the FP32 result stays within 5e-6 relative L2
  after 6 steps (FP32 rounding of the stencils);
* the autotuner's choice (staging and tile depth) leaves the results
  unchanged;
* a wait on an mbarrier that nothing completes ends at its limit with
  SH_ERR_TIMEOUT, and the device keeps working.
"""
import numpy as np
import pytest

import sledgehamr_gb300 as sh
from sledgehamr_gb300 import _lib, ic
from tests.conftest import rel_l2

pytestmark = pytest.mark.gpu

SIZES = [32, 48, 64, 96, 128, 32]


def _states(Ns, dx=0.25):
    out = []
    for r, N in enumerate(Ns):
        L = N * dx
        st = ic.axion_string_ic(N, L, kmax=1.5, seed=70 + r)
        st[2:] = 0.2 * ic.axion_string_ic(N, L, kmax=1.0, seed=170 + r)[:2]
        out.append(st)
    return out


def _run(ctx, family, prec, Ns, states, staging, steps=6, graph=False, tune=False,
         dt=0.0625):
    lam = [0.5 + 0.3 * r for r in range(len(Ns))]
    params = np.array([[l, 0.2, 0.0, 0.0] for l in lam]).ravel()
    E = sh.Ensemble(ctx, family, prec, Ns, [0.25] * len(Ns), params)
    for r, st in enumerate(states):
        E.write(r, st)
    E.set_time(0.7)
    if tune:
        E.tune(dt)
    else:
        E.tune(dt, tile_nz=16)
        E.set_staging(staging)
    assert tune or E.staging() == staging
    E.set_graph(graph)
    E.step(dt, steps)
    out = [E.read(r) for r in range(len(Ns))]
    chosen = E.staging()
    E.close()
    return out, chosen


@pytest.mark.parametrize("family", [sh.FAMILY_AXION_LAP1, sh.FAMILY_AXION_LAP2])
@pytest.mark.parametrize("prec", [sh.PREC_FP32, sh.PREC_FP32_KAHAN])
def test_tma_staging_equals_register_staging(ctx, family, prec):
    states = _states(SIZES)
    a, _ = _run(ctx, family, prec, SIZES, states, staging=0)
    b, _ = _run(ctx, family, prec, SIZES, states, staging=1)
    for r in range(len(SIZES)):
        assert np.array_equal(a[r], b[r]), (r, rel_l2(b[r], a[r]))


def test_tma_staging_with_graphs_and_against_the_oracle(ctx, oracle):
    Ns = [48, 64]
    states = _states(Ns)
    a, _ = _run(ctx, sh.FAMILY_AXION_LAP2, sh.PREC_FP32_KAHAN, Ns, states, staging=1,
                graph=True)
    b, _ = _run(ctx, sh.FAMILY_AXION_LAP2, sh.PREC_FP32_KAHAN, Ns, states, staging=1)
    for r in range(len(Ns)):
        assert np.array_equal(a[r], b[r])
        ref = oracle.evolve_periodic("AxionStringsLap2", sh.RKN4, states[r], t0=0.7,
                                     dt=0.0625, dx=0.25, nsteps=6,
                                     params=[0.5 + 0.3 * r, 0.2], nghost=2)
        assert rel_l2(a[r], ref) <= 5e-6


def test_tuned_choice_leaves_results_unchanged(ctx):
    states = _states(SIZES)
    a, _ = _run(ctx, sh.FAMILY_AXION_LAP1, sh.PREC_FP32_KAHAN, SIZES, states, staging=0)
    b, chosen = _run(ctx, sh.FAMILY_AXION_LAP1, sh.PREC_FP32_KAHAN, SIZES, states, staging=0,
                     tune=True)
    assert chosen in (0, 1)
    for r in range(len(SIZES)):
        assert np.array_equal(a[r], b[r])


def test_staging_unsupported_sizes_are_refused(ctx):
    E = sh.Ensemble(ctx, sh.FAMILY_AXION_LAP1, sh.PREC_FP32, [30], [0.25], [1, 0, 0, 0])
    with pytest.raises(sh.ShError) as e:
        E.set_staging(1)
    assert e.value.code == _lib.SH_ERR_UNSUPPORTED
    assert E.staging() == 0
    E.close()


def test_bounded_wait_times_out_and_the_device_keeps_working(ctx):
    import ctypes as C
    lib = _lib.load()
    st = C.c_int()
    assert lib.sh_probe_wait_timeout(0, C.byref(st)) == 0
    assert st.value == _lib.SH_ERR_TIMEOUT
    states = _states([32])
    out, _ = _run(ctx, sh.FAMILY_AXION_LAP1, sh.PREC_FP32, [32], states, staging=1, steps=2)
    assert np.all(np.isfinite(out[0]))
