"""GravitationalWaves::ComputeSpectrum restated with numpy (test
infrastructure): the oracle's gw_spectrum (oracle/oracle_core.h, after
source/gravitational_waves.cpp:202-304 and gravitational_waves.h:101-133)
vectorised over k-cells, with numpy's FFT, for grids where the oracle's own
transform would take too long (the GPU parity tests at 384^3).  Pinned to
the oracle on small grids by tests/test_gw_numpy.py.

The contraction sum_{ijlm} Lambda_ijlm (Re u_ij Re u_lm + Im u_ij Im u_lm),
Lambda_ijlm = P_il P_jm - P_ij P_lm / 2, equals
Re[sum_lm (P U P)_lm conj(U_lm)] - |sum_ij P_ij U_ij|^2 / 2 for the
symmetric U and P; it is zero at k = 0.
"""
from __future__ import annotations

import numpy as np


def gw_spectrum(comps6, zero_padding, projection_type, unbinned, index_to_k, unique_k2,
                chunk=16):
    """comps6: six (N, N, N) arrays (z, y, x) in the order xx, xy, xz, yy,
    yz, zz; index_to_k(P, type) and unique_k2(P) supply the k-map and the
    unbinned bin list (the oracle's).  Returns (bins, ks)."""
    c6 = [np.asarray(c, dtype=np.float64) for c in comps6]
    N = c6[0].shape[-1]
    P = N * zero_padding
    H = P // 2 + 1
    F = []
    for c in c6:
        if zero_padding == 1:
            F.append(np.fft.rfftn(c))
        else:
            pad = np.zeros((P, P, P))
            pad[:N, :N, :N] = c
            F.append(np.fft.rfftn(pad))
    itk = np.asarray(index_to_k(P, projection_type), dtype=np.float64)
    if unbinned:
        ks = np.asarray(unique_k2(P), dtype=np.int64)
    else:
        kmax = int(np.sqrt(3.0) / 2.0 * P + 0.5)
        ks = np.arange(kmax + 1, dtype=np.int64) ** 2
    out = np.zeros(ks.size)
    mat = ((0, 1, 2), (1, 3, 4), (2, 4, 5))
    a = np.arange(H)
    li = np.where(a >= P // 2, a - P, a)
    bj = np.arange(P)
    lj = np.where(bj >= P // 2, bj - P, bj)
    multpl = np.where((a == 0) | (a == P // 2), 1.0, 2.0)
    for c0 in range(0, P, chunk):
        c1 = min(P, c0 + chunk)
        cc = np.arange(c0, c1)
        lk = np.where(cc >= P // 2, cc - P, cc)
        # k-map components per cell (z, y, x) of the slab
        d = [np.broadcast_to(itk[a][None, None, :], (c1 - c0, P, H)),
             np.broadcast_to(itk[bj][None, :, None], (c1 - c0, P, H)),
             np.broadcast_to(itk[cc][:, None, None], (c1 - c0, P, H))]
        norm = d[0] ** 2 + d[1] ** 2 + d[2] ** 2
        zero = norm == 0.0
        safe = np.where(zero, 1.0, norm)
        Pm = [[(1.0 if i == j else 0.0) - d[i] * d[j] / safe for j in range(3)]
              for i in range(3)]
        U = [[F[mat[i][j]][c0:c1] for j in range(3)] for i in range(3)]
        PU = [[sum(Pm[i][k] * U[k][j] for k in range(3)) for j in range(3)] for i in range(3)]
        PUP = [[sum(PU[i][k] * Pm[k][j] for k in range(3)) for j in range(3)] for i in range(3)]
        first = sum((PUP[l][m] * np.conj(U[l][m])).real for l in range(3) for m in range(3))
        tr = sum(Pm[i][j] * U[i][j] for i in range(3) for j in range(3))
        val = first - 0.5 * (tr.real ** 2 + tr.imag ** 2)
        val = np.where(zero, 0.0, val) * multpl[None, None, :]
        sq = (li[None, None, :] ** 2 + lj[None, :, None] ** 2 + lk[:, None, None] ** 2)
        if unbinned:
            idx = np.searchsorted(ks, sq.ravel(), side="left")
        else:
            idx = (np.sqrt(sq.ravel().astype(np.float64)) + 0.5).astype(np.int64)
        out += np.bincount(idx, weights=val.ravel(), minlength=ks.size)[: ks.size]
    return out / float(P) ** 6, ks
