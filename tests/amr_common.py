"""Shared AMR test configuration: AxionStringsLap2 (4th-order Laplacian,
lambda = 1, plain quartic potential), 16^3 coarse grid with dx = 0.25, up to
two refinement levels, truncation-error and string-winding tags, global
regrids only unless a test asks for local ones (max_local_regrids)."""
import sledgehamr_gb300 as sh
from sledgehamr_gb300 import ic

N0, L = 16, 4.0


def config(**kw):
    base = dict(N0=N0, L=L, cfl=0.25, t_start=3.0, nghost=2, max_level=2, blocking_factor=8,
                max_grid_size=16, n_error_buf=1, regrid_dt=0.0, te_crit=[1e-2] * 4,
                params=[1.0, 0.0], string_width_threshold=2.0, record_regrids=1,
                max_local_regrids=0)
    base.update(kw)
    return sh.amr_config("AxionStringsLap2", **base)


def level0(seed=0):
    return ic.axion_string_ic(N0, L, kmax=3.0, seed=seed)


def boxes_layout_to_levelwise(flat, boxes, ncomp):
    """Split a boxes-layout array into per-box (ncomp, nz, ny, nx) blocks."""
    out, off = [], 0
    for lo, hi in boxes:
        n = (hi[0] - lo[0] + 1) * (hi[1] - lo[1] + 1) * (hi[2] - lo[2] + 1)
        out.append(flat[off:off + n * ncomp].reshape(ncomp, hi[2] - lo[2] + 1,
                                                     hi[1] - lo[1] + 1, hi[0] - lo[0] + 1))
        off += n * ncomp
    return out
