"""sh_tag_static: tagging that allocates no GPU memory, for callers whose
device memory is managed elsewhere or who cannot afford the synchronisation
of cudaMalloc/cudaFree mid-step.  Checked through the C ABI against sh_tag
on the same level, on two calls in a row (the working array keeps the
previous call's contents, so the second call also shows that nothing
leaks from the first).  Tag masks and counts are compared exactly, the
tolerance every tag test here uses."""
import ctypes as C

import numpy as np
import pytest

import sledgehamr_gb300 as sh
from sledgehamr_gb300 import _lib
from tests.conftest import golden

pytestmark = pytest.mark.gpu


def _call(ctx, fn, lv, use_te, te_crit, dt, dx):
    mask = np.empty(lv.nvalid, dtype=np.uint8)
    counts = np.zeros(2 + lv.ncomp, dtype=np.int64)
    lst = np.empty(lv.nvalid, dtype=np.int32)
    nt = C.c_longlong()
    crit = np.ascontiguousarray(te_crit, dtype=np.float64)
    rc = fn(ctx.h, lv.h, int(use_te), 1.0, 0, dt, dx, C.c_void_p(crit.ctypes.data), None, 0,
            None, 0, C.c_void_p(mask.ctypes.data), C.c_void_p(counts.ctypes.data),
            C.c_void_p(lst.ctypes.data), lv.nvalid, C.byref(nt))
    ctx.check(rc, fn.__name__)
    return mask, counts, lst[: nt.value].copy()


def _device_memory():
    """(free bytes of the device, bytes in use in its default memory pool),
    read through the CUDA driver: a cudaMalloc lowers the first, a
    cudaMallocAsync from the pool raises the second."""
    cu = C.CDLL("libcuda.so.1")
    free, total = C.c_size_t(), C.c_size_t()
    assert cu.cuMemGetInfo_v2(C.byref(free), C.byref(total)) == 0
    dev = C.c_int()
    assert cu.cuCtxGetDevice(C.byref(dev)) == 0
    pool = C.c_void_p()
    assert cu.cuDeviceGetDefaultMemPool(C.byref(pool), dev) == 0
    used = C.c_uint64()
    CU_MEMPOOL_ATTR_USED_MEM_CURRENT = 7
    assert cu.cuMemPoolGetAttribute(pool, CU_MEMPOOL_ATTR_USED_MEM_CURRENT, C.byref(used)) == 0
    return free.value, used.value


def test_tag_static_matches_tag_on_consecutive_calls(ctx):
    lib = _lib.load()
    g = golden("ref_tag")
    st, te, crit = g["state"], g["te"], g["te_crit"]
    dt, dx = float(g["dt"]), float(g["dx"])
    lv = sh.Level.periodic(ctx, "AxionStrings", st.shape[-1], 2, max_grid=8)
    lv.write(st)
    lv.fill_patch()
    lv.write(te, which=sh.SH_OLD)
    for q, use_te in enumerate((True, False)):  # two calls in a row, different results
        want = _call(ctx, lib.sh_tag, lv, use_te, crit, dt, dx)
        ctx.synchronize()
        before = _device_memory()
        got = _call(ctx, lib.sh_tag_static, lv, use_te, crit, dt, dx)
        ctx.synchronize()
        after = _device_memory()
        if q > 0:
            # the first call may load the library's device code lazily; from
            # the second on, the call takes no device memory of any kind
            assert after == before, (before, after)
        assert want[0].sum() > 0
        for w, h in zip(want, got):
            assert np.array_equal(w, h)
    lv.close()


def test_tag_static_rejects_levels_above_its_limit(ctx):
    lib = _lib.load()
    n = 1
    while n ** 3 <= _lib.SH_TAG_STATIC_MAX_CELLS:
        n += 8
    lv = sh.Level.periodic(ctx, "AxionStringsLap1", n, 1)
    mask = np.empty(lv.nvalid, dtype=np.uint8)
    rc = lib.sh_tag_static(ctx.h, lv.h, 0, 1.0, 0, 0.1, 0.25, None, None, 0, None, 0,
                           C.c_void_p(mask.ctypes.data), None, None, 0, None)
    assert rc == _lib.SH_ERR_ARG
    assert b"SH_TAG_STATIC_MAX_CELLS" in lib.sh_ctx_last_error(ctx.h)
    lv.close()
