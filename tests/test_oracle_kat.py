"""Known-answer tests of the oracle (the reference has no tests of its own):
stencil exactness on polynomials, RKN4/RKN5/SSPRK3 convergence orders on an
exactly solvable mode, vanishing truncation errors on smooth data, string
winding around a synthetic vortex line, and a single-mode GW spectrum."""
import numpy as np
import pytest

from sledgehamr_gb300 import ic


def test_laplacian_exact_on_trig_eigenfunction(oracle):
    """cos(2 pi m x / N) is an eigenfunction of every periodic stencil with
    eigenvalue -(sum_r c_r 2 sin^2(pi m r / N)) known in closed form."""
    N, dx, m = 16, 0.3, 3
    x = np.arange(N)
    f = np.cos(2 * np.pi * m * x / N)[None, None, :] * np.ones((N, N, N))
    th = 2 * np.pi * m / N
    eig = {1: (2 * np.cos(th) - 2) / dx ** 2,
           2: (-2 * np.cos(2 * th) + 32 * np.cos(th) - 30) / (12 * dx ** 2),
           3: (4 * np.cos(3 * th) - 54 * np.cos(2 * th) + 540 * np.cos(th) - 490) / (180 * dx ** 2)}
    for order in (1, 2, 3):
        lap = oracle.stencil(3, order, f, dx)
        assert np.allclose(lap, eig[order] * f, atol=1e-11)


def test_gradient_order_of_accuracy(oracle):
    for order, p in ((1, 2), (2, 4), (3, 6)):
        errs = []
        for N in (32, 64):
            dx = 2 * np.pi / N
            x = np.arange(N) * dx
            f = np.sin(x)[None, None, :] * np.ones((N, N, N))
            g = oracle.stencil(0, order, f, dx)
            errs.append(np.abs(g - np.cos(x)[None, None, :]).max())
        assert abs(np.log2(errs[0] / errs[1]) - p) < 0.3


def _mode_state(N, L, eta, kvec_n=(1, 0, 0)):
    """Psi1 = cos(k.x) sin(k_eff eta) / eta solves the lambda = 0 equations
    Psi'' + 2/eta Psi' = lap Psi on the lattice (k_eff^2 = -eigenvalue)."""
    dx = L / N
    n = np.array(kvec_n)
    x = np.arange(N) * dx
    phase = (2 * np.pi / L) * (n[0] * x[None, None, :] + n[1] * x[None, :, None] +
                               n[2] * x[:, None, None])
    keff2 = sum((4 / dx ** 2) * np.sin(np.pi * nn / N) ** 2 for nn in n)
    k = np.sqrt(keff2)
    s = np.zeros((4, N, N, N))
    s[0] = np.cos(phase) * np.sin(k * eta) / eta
    s[2] = np.cos(phase) * (k * np.cos(k * eta) * eta - np.sin(k * eta)) / eta ** 2
    return s, k


def _kg_state(N, L, t, m2=0.5, n=1):
    """Klein-Gordon mode Phi = cos(k x) cos(w t), w^2 = k_eff^2 + m^2, as the
    FirstOrderPhaseTransition Rhs with V'(Phi) = -m^2 Phi (no GW); k_eff^2 is
    minus the eigenvalue of the 13-point Laplacian that project uses."""
    dx = L / N
    x = np.arange(N) * dx
    th = 2 * np.pi * n / N
    keff2 = (2 * np.cos(2 * th) - 32 * np.cos(th) + 30) / (12 * dx ** 2)
    w = np.sqrt(keff2 + m2)
    c = np.cos(2 * np.pi * n * x / L)[None, None, :] * np.ones((N, N, N))
    return np.stack([c * np.cos(w * t), -w * c * np.sin(w * t)])


@pytest.mark.parametrize("integ,order", [(21, 4), (22, 5), (10, 3), (11, 2)])
def test_time_integrator_convergence(oracle, integ, order):
    """Convergence order on a velocity-independent force (y'' = f(t, y)),
    the class the reference's RKN tableaus are built for."""
    N, L, T, m2 = 8, 8.0, 1.0, 0.5
    s0 = _kg_state(N, L, 0.0, m2)
    exact = _kg_state(N, L, T, m2)
    params = [0.0, -m2, 0.0, 0.0, 0.0, 0.0, 0.0]
    errs = []
    for nsteps in (8, 16):
        out = oracle.evolve_periodic("FirstOrderPhaseTransition", integ, s0, t0=0.0,
                                     dt=T / nsteps, dx=L / N, nsteps=nsteps, params=params,
                                     nghost=2)
        errs.append(np.abs(out[0] - exact[0]).max())
    rate = np.log2(errs[0] / errs[1])
    assert rate > order - 0.5, (errs, rate)


def test_rkn_with_friction_is_first_order(oracle):
    """The reference's RKN stages keep y'0 for every stage (rkn.cpp:57-64), so
    with the velocity-dependent friction -2 Pi / eta the method is only first
    order; the restatement reproduces that."""
    N, L, eta0, T = 8, 8.0, 1.0, 0.5
    s0, k = _mode_state(N, L, eta0)
    exact, _ = _mode_state(N, L, eta0 + T)
    errs = []
    for nsteps in (8, 16):
        out = oracle.evolve_periodic("AxionStringsLap1", 21, s0, t0=eta0, dt=T / nsteps,
                                     dx=L / N, nsteps=nsteps, params=[0.0, 0.0], nghost=1)
        errs.append(np.abs(out[0] - exact[0]).max())
    assert abs(np.log2(errs[0] / errs[1]) - 1.0) < 0.2


def test_truncation_error_vanishes_for_linear_fields(oracle):
    Nc = 4
    z, y, x = np.meshgrid(np.arange(2 * Nc), np.arange(2 * Nc), np.arange(2 * Nc), indexing="ij")
    fine = np.stack([0.5 * x + 0.25 * y - 0.125 * z + 3.0] * 2).astype(float)
    # coarse cell i covers fine 2i, 2i+1: its exact average
    zc, yc, xc = np.meshgrid(np.arange(Nc), np.arange(Nc), np.arange(Nc), indexing="ij")
    crse = np.stack([0.5 * (2 * xc + 0.5) + 0.25 * (2 * yc + 0.5) - 0.125 * (2 * zc + 0.5) + 3.0] * 2)
    c, te = oracle.avgdown_te(fine, crse, np.full_like(fine, 7.0))
    assert np.allclose(c, crse, atol=1e-14)
    even = te[:, ::2, ::2, ::2]
    assert np.abs(even).max() < 1e-14
    te_odd = te.copy()
    te_odd[:, ::2, ::2, ::2] = 7.0
    assert np.all(te_odd == 7.0)  # only the even cells receive errors


def test_string_winding_around_vortex_line(oracle):
    """Psi = (x - x0) + i (y - y0): one string along z through (x0, y0);
    only the xy plaquettes around it are pierced."""
    N = 8
    x0, y0 = 3.5 + 0.1, 4.5 - 0.2
    z, y, x = np.meshgrid(np.arange(N), np.arange(N), np.arange(N), indexing="ij")
    s = np.zeros((4, N, N, N))
    # keep the periodic wrap away from the line: a smooth periodic profile
    s[0] = np.sin(2 * np.pi * (x - x0) / N)
    s[1] = np.sin(2 * np.pi * (y - y0) / N)
    mask, counts = oracle.tag("AxionStrings", s, None, 1.0, 0, 0.1, 1.0)
    tagged = np.argwhere(mask)
    assert len(tagged) > 0
    # every z plane carries the same pattern (the line is along z)
    assert all(np.array_equal(mask[0], mask[k]) for k in range(N))
    assert counts[0] == mask.sum() and counts[1] == mask.sum()


def test_gw_single_mode_lands_in_one_bin(oracle):
    """One transverse-traceless plane wave along x in du_yy = -du_zz puts all
    its power in the bin of |n| = m with the analytic weight."""
    N, m, A = 8, 2, 0.7
    x = np.arange(N)
    wave = A * np.cos(2 * np.pi * m * x / N)[None, None, :] * np.ones((N, N, N))
    zero = np.zeros((N, N, N))
    comps = np.stack([zero, zero, zero, wave, zero, -wave])  # xx xy xz yy yz zz
    bins, ks = oracle.gw_spectrum(comps, projection_type=2, unbinned=False)
    nz = np.flatnonzero(np.abs(bins) > 1e-14)
    assert list(nz) == [m]
    # |FFT|^2 of A cos: two peaks of (A N^3 / 2)^2; with multpl=2 for a>0 and
    # only the a=+m half stored: 2 * sum over the TT tensor (yy^2 + zz^2)
    expected = 2 * 2 * (A * N ** 3 / 2) ** 2 / N ** 6
    assert np.isclose(bins[m], expected, rtol=1e-12)
