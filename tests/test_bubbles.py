"""FirstOrderPhaseTransition bubble injection: the oracle's restatement
against the reference's own AddBubble (bitwise) and against the golden
fixture made from it."""
import numpy as np
import pytest

from tests.conftest import golden
from tests.oracle_lib import oracle_add_bubbles, ref_available


def test_oracle_bubbles_golden():
    g = golden("ref_bubbles")
    out = oracle_add_bubbles(g["state_in"], g["xyz"], g["profile"], float(g["inv_dx"]),
                             float(g["Lcut"]), float(g["dx"]))
    assert np.array_equal(out, g["state_out"])


@pytest.mark.skipif(not ref_available(), reason="oracle/_ref not built")
@pytest.mark.parametrize("seed", [0, 1])
def test_oracle_bubbles_bitwise_vs_reference(seed):
    rng = np.random.default_rng(seed)
    N, dx = 12, 0.7
    st = rng.normal(size=(14, N, N, N))
    xyz = rng.uniform(0, N * dx, size=(5, 3))
    inv_dx, Lcut = 3.0, 4.1
    nb = int(Lcut * inv_dx) + 2 + seed
    prof = rng.normal(size=(2, nb))
    a = oracle_add_bubbles(st, xyz, prof, inv_dx, Lcut, dx)
    b = oracle_add_bubbles(st, xyz, prof, inv_dx, Lcut, dx, ref=True)
    assert np.array_equal(a, b)
    assert not np.array_equal(a, st)
