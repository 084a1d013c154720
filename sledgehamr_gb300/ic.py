"""Seeded synthetic initial conditions (host side, numpy).

Random numbers come from SplitMix64 (Steele, Lea and Flood, "Fast splittable
pseudorandom number generators", OOPSLA 2014), turned into normal deviates
with the Box-Muller transform, so that the same seed gives the same field on
every host.

axion_string_ic: psi1 and psi2 are independent Gaussian random fields whose
Fourier amplitudes are i.i.d. complex normal with flat power for
|k| = 2 pi |n| / L <= kmax and zero above (Hermitian symmetry is implied by
building the field from its real-FFT half space), each rescaled to unit
real-space variance; Pi1 = Pi2 = 0.
"""
from __future__ import annotations

import numpy as np

_GOLDEN = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)


def splitmix64(seed: int, n: int) -> np.ndarray:
    """n successive outputs of SplitMix64 started at `seed`."""
    with np.errstate(over="ignore"):
        x = np.uint64(seed) + _GOLDEN * np.arange(1, n + 1, dtype=np.uint64)
        z = (x ^ (x >> np.uint64(30))) * _M1
        z = (z ^ (z >> np.uint64(27))) * _M2
        return z ^ (z >> np.uint64(31))


def uniform(seed: int, n: int) -> np.ndarray:
    """Uniform doubles in (0, 1] from the top 53 bits."""
    return ((splitmix64(seed, n) >> np.uint64(11)).astype(np.float64) + 1.0) * (2.0 ** -53)


def normal(seed: int, n: int) -> np.ndarray:
    m = (n + 1) // 2
    u = uniform(seed, 2 * m)
    r = np.sqrt(-2.0 * np.log(u[:m]))
    th = 2.0 * np.pi * u[m:]
    return np.concatenate([r * np.cos(th), r * np.sin(th)])[:n]


def gaussian_field(N: int, L: float, kmax: float, seed: int) -> np.ndarray:
    """Real N^3 field (z, y, x order, x fastest) with flat power up to kmax,
    zero mean and unit variance."""
    H = N // 2 + 1
    g = normal(seed, 2 * N * N * H).reshape(2, N, N, H)
    amp = g[0] + 1j * g[1]
    f = np.fft.fftfreq(N) * N
    fr = np.arange(H)
    n2 = f[:, None, None] ** 2 + f[None, :, None] ** 2 + fr[None, None, :] ** 2
    k = 2.0 * np.pi * np.sqrt(n2) / L
    amp = np.where(k <= kmax, amp, 0.0)
    amp[0, 0, 0] = 0.0
    field = np.fft.irfftn(amp, s=(N, N, N), axes=(0, 1, 2))
    std = field.std()
    if std == 0:
        raise ValueError("no modes below kmax: increase N, L or kmax")
    return np.ascontiguousarray((field - field.mean()) / std)


def axion_string_ic(N: int, L: float, kmax: float = 1.0, seed: int = 0) -> np.ndarray:
    """(Psi1, Psi2, Pi1, Pi2) in canonical layout (4, N, N, N)."""
    out = np.zeros((4, N, N, N))
    out[0] = gaussian_field(N, L, kmax, 2 * seed)
    out[1] = gaussian_field(N, L, kmax, 2 * seed + 1)
    return out
