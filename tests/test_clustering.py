"""New-grid generation (shamr::make_boxes, shared by the GPU and oracle AMR
drivers): the boxes cover every tagged block, stay inside the allowed
(properly nested) blocks, do not overlap, respect max_grid_size, and the
Berger-Rigoutsos clusters reach the requested efficiency."""
import ctypes as C

import numpy as np
import pytest

from tests.oracle_lib import ORACLE_SO, build_oracle


def make_boxes(tags, allowed, clustering, grid_eff, w):
    build_oracle()
    lib = C.CDLL(ORACLE_SO)
    nb = tags.shape[0]
    cap = nb ** 3
    out = np.empty(6 * cap, dtype=np.int32)
    t = np.ascontiguousarray(tags, dtype=np.uint8)
    a = np.ascontiguousarray(allowed, dtype=np.uint8)
    n = lib.orc_make_boxes(C.c_void_p(t.ctypes.data), C.c_void_p(a.ctypes.data), nb, clustering,
                           C.c_double(grid_eff), w, C.c_void_p(out.ctypes.data), cap)
    assert n >= 0
    return out[: 6 * n].reshape(n, 6)


def blobs(nb, seed, nblob=6, r=3.0):
    rng = np.random.default_rng(seed)
    z, y, x = np.mgrid[0:nb, 0:nb, 0:nb]
    t = np.zeros((nb, nb, nb), dtype=bool)
    for _ in range(nblob):
        c = rng.uniform(0, nb, 3)
        rad = rng.uniform(1.0, r)
        t |= (x - c[0]) ** 2 + (y - c[1]) ** 2 + (z - c[2]) ** 2 <= rad ** 2
    # a thin string-like line as well
    t[nb // 3, nb // 2, :] = True
    return t


def cover_count(boxes, nb):
    cnt = np.zeros((nb, nb, nb), dtype=np.int32)
    for b in boxes:
        cnt[b[2]:b[5] + 1, b[1]:b[4] + 1, b[0]:b[3] + 1] += 1
    return cnt


@pytest.mark.parametrize("clustering", [0, 1, 2])
@pytest.mark.parametrize("seed", [0, 1, 2])
def test_boxes_cover_tags_inside_nesting(clustering, seed):
    nb, w, eff = 24, 4, 0.7
    tags = blobs(nb, seed)
    allowed = np.ones_like(tags)
    allowed[:, :, : nb // 4] = False  # a region outside the coarser level
    tags &= allowed
    boxes = make_boxes(tags, allowed, clustering, eff, w)
    cnt = cover_count(boxes, nb)
    assert cnt.max() <= 1  # disjoint
    assert np.all(cnt[tags] == 1)  # every tag covered
    assert not np.any(cnt[~allowed])  # nothing outside the nesting
    ext = boxes[:, 3:] - boxes[:, :3] + 1
    assert ext.min() >= 1 and ext.max() <= w
    if clustering == 1:
        assert np.array_equal(cnt.astype(bool), tags)  # windows: fully tagged boxes
    else:
        assert cnt.sum() <= tags.sum() / eff + 1e-9


def test_br_makes_fewer_boxes_than_windows():
    nb, w = 32, 4
    tags = blobs(nb, 7, nblob=10, r=5.0)
    allowed = np.ones_like(tags)
    br = make_boxes(tags, allowed, 0, 0.7, w)
    brw = make_boxes(tags, allowed, 2, 0.7, w)
    win = make_boxes(tags, allowed, 1, 0.7, w)
    assert len(br) < len(win) and len(brw) < len(win)


def test_full_and_empty_tag_sets():
    nb, w = 16, 4
    full = np.ones((nb, nb, nb), dtype=bool)
    b = make_boxes(full, full, 0, 0.7, w)
    assert len(b) == (nb // w) ** 3
    assert len(make_boxes(np.zeros_like(full), full, 0, 0.7, w)) == 0


def test_simplify_equals_plain_full_passes(tmp_path):
    """shamr::simplify (radix-sorted keys, merge-free directions skipped)
    gives the boxes of plain full passes of the same merging rule."""
    import os
    import shutil
    import subprocess
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    here = os.path.dirname(os.path.abspath(__file__))
    root = os.path.dirname(here)
    exe = str(tmp_path / "sc")
    r = subprocess.run([gxx, "-O2", "-std=c++17", "-fopenmp",
                        "-I" + os.path.join(root, "sledgehamr_gb300", "csrc"),
                        os.path.join(here, "cpp", "simplify_check.cpp"), "-o", exe],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0 and out.stdout.strip() == "ok", out.stdout


def test_cluster_tasks_equal_serial_recursion(tmp_path):
    """Berger-Rigoutsos with the large halves as OpenMP tasks
    (shamr::cluster_parallel) gives the serial recursion's clusters in the
    same order."""
    import os
    import shutil
    import subprocess
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    here = os.path.dirname(os.path.abspath(__file__))
    root = os.path.dirname(here)
    exe = str(tmp_path / "ctc")
    r = subprocess.run([gxx, "-O2", "-std=c++17", "-fopenmp",
                        "-I" + os.path.join(root, "sledgehamr_gb300", "csrc"),
                        os.path.join(here, "cpp", "cluster_tasks_check.cpp"), "-o", exe],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([exe], capture_output=True, text=True, timeout=300,
                         env=dict(os.environ, OMP_NUM_THREADS="4"))
    assert out.returncode == 0 and out.stdout.strip().endswith("ok"), out.stdout
