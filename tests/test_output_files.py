"""Output files in sledgehamr's formats (no GPU).

* The HDF5 parser of the tests (tests/hdf5_read.py) is pinned on the
  reference's own HDF5 file data/spectra_ks.hdf5 (written by h5py), whose
  datasets must equal the spectrum bins and k maps the library generates.
* The library's HDF5 writer (sh_h5_*) round-trips datasets of every stored
  type and count through that parser, lays out the same structures and
  message sequence as the reference's file, and rejects bad names.
* The level and slice writers on host data (sh_output_*_host) equal the
  numpy restatement of LevelWriter::WriteSingleLevel and
  Slices::WriteSingleSlice (oracle/output_oracle.py) bit for bit, for both
  precisions, downsample factors 1, 2 and 4, and truncation errors.
"""
import os

import numpy as np
import pytest

from oracle import output_oracle as oo
from tests import hdf5_read
from tests.conftest import REF_ROOT

REF_DATA = os.path.join(REF_ROOT, "data", "spectra_ks.hdf5")


def _sh():
    import sledgehamr_gb300 as sh
    return sh


@pytest.mark.skipif(not os.path.exists(REF_DATA), reason="reference data file absent")
def test_reader_pinned_on_reference_file():
    sh = _sh()
    f = hdf5_read.File(REF_DATA)
    dims = sorted({int(k.split("_")[0]) for k in f.keys()})
    assert dims == [32, 64, 128, 256, 512]
    for N in dims:
        bins = f[f"{N}_bins"]
        assert bins.dtype == np.int64
        np.testing.assert_array_equal(bins, sh.spectrum_bins(N))
        assert f[f"{N}_nks"].tolist() == [bins.size]
        for p in (1, 2):
            k = f[f"{N}_k{p}"]
            assert k.dtype == np.float64 and k.shape == (N,)
            np.testing.assert_allclose(k, sh.index_to_k(N, p), rtol=0, atol=1e-15)


def _roundtrip(tmp_path, sets):
    from sledgehamr_gb300.output import H5File
    f = H5File()
    for name, a in sets.items():
        f.add(name, a)
    assert len(f) == len(sets)
    p = str(tmp_path / "x.hdf5")
    f.write(p)
    return hdf5_read.File(p)


@pytest.mark.parametrize("count", [0, 1, 7, 8, 9, 33, 300, 1200, 9000])
def test_writer_roundtrip(tmp_path, count):
    rng = np.random.default_rng(count)
    sets = {}
    for q in range(count):
        kind = q % 4
        n = int(rng.integers(0, 50)) if q % 7 else 0
        name = "d%0*d_%s" % (int(rng.integers(1, 6)), q, "x" * int(rng.integers(0, 12)))
        if kind == 0:
            sets[name] = rng.standard_normal(n).astype(np.float32)
        elif kind == 1:
            sets[name] = rng.standard_normal(n)
        elif kind == 2:
            sets[name] = rng.integers(-2**31, 2**31, n).astype(np.int32)
        else:
            sets[name] = rng.integers(-2**53, 2**53, n).astype(np.int64)
    r = _roundtrip(tmp_path, sets)
    assert r.keys() == sorted(sets)
    # symbol-table nodes hold 8 names and B-tree nodes 32 children: 9000
    # names need a B-tree of three levels
    assert len(r.btree_nodes) == (3 if count > 8 * 32 * 32 else 2 if count > 8 * 32 else 1)
    for name, a in sets.items():
        got = r[name]
        want_type = np.float32 if a.dtype == np.float32 else np.float64
        assert got.dtype == want_type and got.shape == a.shape
        np.testing.assert_array_equal(got, a.astype(want_type))


def test_writer_layout_matches_reference_file(tmp_path):
    r = _roundtrip(tmp_path, {"a": np.arange(5.0), "b": np.arange(3, dtype=np.float32)})
    assert (r.leaf_k, r.internal_k) == (4, 16)
    assert r.message_types("a") == [1, 3, 5, 8, 0] == r.message_types("b")
    if os.path.exists(REF_DATA):
        ref = hdf5_read.File(REF_DATA)
        assert (ref.leaf_k, ref.internal_k) == (r.leaf_k, r.internal_k)
        name = ref.keys()[0]
        assert ref.message_types(name) == r.message_types("a")
        # same dataspace, fill value and layout message forms
        for mtype in (1, 5):
            rm = [m for m in ref.datasets[name].messages if m.type == mtype][0]
            wm = [m for m in r.datasets["a"].messages if m.type == mtype][0]
            assert (rm.flags, rm.data[:4]) == (wm.flags, wm.data[:4])
        hdr_ref = ref.buf[ref.entries[name]:ref.entries[name] + 16]
        hdr_new = r.buf[r.entries["a"]:r.entries["a"] + 16]
        assert hdr_ref[:2] == hdr_new[:2] and hdr_ref[4:12] == hdr_new[4:12]
        # the F64 datatype message is byte for byte the one h5py wrote for
        # the reference's float64 k maps
        dt_ref = [m for m in ref.datasets["32_k1"].messages if m.type == 3][0]
        dt_new = [m for m in r.datasets["a"].messages if m.type == 3][0]
        assert (dt_ref.flags, dt_ref.data) == (dt_new.flags, dt_new.data)
        # superblock fields other than the end-of-file address are equal
        assert ref.buf[8:40] == r.buf[8:40] and ref.buf[48:56] == r.buf[48:56]


def test_writer_format_fields_equal_reference_fixture(tmp_path):
    """Format fields of the reference's h5py-written file (committed as
    tests/golden/hdf5_format.npz by tests/golden/make_golden.py) equal the
    writer's, byte for byte, without the reference present."""
    from tests.conftest import golden
    g = golden("hdf5_format")
    r = _roundtrip(tmp_path, {"a": np.arange(5.0)})
    u8 = lambda b: np.frombuffer(bytes(b), dtype=np.uint8)  # noqa: E731
    np.testing.assert_array_equal(u8(r.buf[8:40]), g["superblock_8_40"])
    np.testing.assert_array_equal(u8(r.buf[48:56]), g["superblock_48_56"])
    ds = r.datasets["a"]
    msg = {m.type: m for m in ds.messages}
    assert [m.type for m in ds.messages] == g["message_types"].tolist()
    assert [m.flags for m in ds.messages] == g["message_flags"].tolist()
    hdr = r.buf[r.entries["a"]:r.entries["a"] + 16]
    np.testing.assert_array_equal(u8(hdr[:2] + hdr[4:12]), g["header_prefix"])
    np.testing.assert_array_equal(u8(msg[1].data[:4]), g["dataspace_head"])
    np.testing.assert_array_equal(u8(msg[5].data), g["fill_value"])
    np.testing.assert_array_equal(u8(msg[3].data), g["datatype_f64"])
    np.testing.assert_array_equal(u8(msg[8].data[:2]), g["layout_head"])


def test_writer_rejects_bad_names(tmp_path):
    from sledgehamr_gb300.output import H5Error, H5File
    f = H5File()
    f.add("ok", np.zeros(2))
    for bad in ["", "a/b", "."]:
        with pytest.raises(H5Error):
            f.add(bad, np.zeros(2))
    with pytest.raises(H5Error):
        f.add("ok", np.zeros(2))
    assert len(f) == 1


def test_writer_reports_io_errors(tmp_path):
    from sledgehamr_gb300.output import H5Error, H5File
    f = H5File()
    f.add("a", np.ones(3))
    with pytest.raises(H5Error):
        f.write(str(tmp_path / "missing_dir" / "x.hdf5"))
    f.write(str(tmp_path / "x.hdf5"))
    assert hdf5_read.File(str(tmp_path / "x.hdf5"))["a"].tolist() == [1.0, 1.0, 1.0]


def test_comp_names():
    from sledgehamr_gb300.output import comp_names
    assert comp_names("AxionStrings") == ["Psi1", "Psi2", "Pi1", "Pi2"]
    names = comp_names("FirstOrderPhaseTransition", with_gw=True)
    assert names[:2] == ["Phi", "dPhi"]
    assert names[2:] == ["u_xx", "u_yy", "u_zz", "u_xy", "u_xz", "u_yz",
                         "du_xx", "du_yy", "du_zz", "du_xy", "du_xz", "du_yz"]


def _level(rng, N=32, bf=8, nbox=5):
    """Disjoint boxes aligned to the blocking factor inside an N^3 domain."""
    boxes = []
    taken = set()
    while len(boxes) < nbox:
        size = [int(rng.choice([bf, 2 * bf])) for _ in range(3)]
        lo = [int(rng.integers(0, (N - s) // bf + 1)) * bf for s in size]
        cells = {(x, y, z) for x in range(lo[0] // bf, (lo[0] + size[0]) // bf)
                 for y in range(lo[1] // bf, (lo[1] + size[1]) // bf)
                 for z in range(lo[2] // bf, (lo[2] + size[2]) // bf)}
        if cells & taken:
            continue
        taken |= cells
        boxes.append((tuple(lo), tuple(lo[d] + size[d] - 1 for d in range(3))))
    return boxes


def _compare(got_file, want):
    assert got_file.keys() == sorted(want)
    for name, a in want.items():
        g = got_file[name]
        assert g.dtype == a.dtype, name
        np.testing.assert_array_equal(g, a, err_msg=name)


@pytest.mark.parametrize("precision", [32, 64])
@pytest.mark.parametrize("downsample", [1, 2, 4])
@pytest.mark.parametrize("te", [False, True])
def test_level_datasets_match_oracle(tmp_path, precision, downsample, te):
    from sledgehamr_gb300.output import level_datasets_host
    rng = np.random.default_rng(100 * precision + 10 * downsample + te)
    boxes = _level(rng)
    names = ["Psi1", "Psi2", "Pi1"]
    nv = sum(np.prod([hi[d] - lo[d] + 1 for d in range(3)]) for lo, hi in boxes)
    cells = rng.standard_normal(nv * len(names)) * 10.0 ** rng.integers(-3, 4, nv * len(names))
    if te:
        cells = np.abs(cells)
    f = level_datasets_host(boxes, cells, names, 3.25, 1, 32, te, downsample, precision)
    p = str(tmp_path / "0.hdf5")
    f.write(p)
    want = oo.level_datasets(boxes, cells, names, 3.25, 1, 32, "te" if te else "data", te,
                             downsample, precision)
    _compare(hdf5_read.File(p), want)


@pytest.mark.parametrize("te", [False, True])
def test_slice_datasets_match_oracle(tmp_path, te):
    from sledgehamr_gb300.output import slices_datasets_host
    rng = np.random.default_rng(7 + te)
    boxes = _level(rng, nbox=7)
    names = ["Phi", "dPhi"]
    nv = sum(np.prod([hi[d] - lo[d] + 1 for d in range(3)]) for lo, hi in boxes)
    cells = rng.standard_normal(nv * len(names))
    for loc in [(0., 0., 0.), (0.3, 0.52, 0.9), (0.999, 0.25, 0.5), (1.0, 1.0, 1.0)]:
        f = slices_datasets_host(boxes, cells, names, 1.5, 2, 32, te, loc)
        p = str(tmp_path / "s.hdf5")
        f.write(p)
        want = oo.slices_datasets(boxes, cells, names, 1.5, 2, 32, te, loc)
        _compare(hdf5_read.File(p), want)


def test_level_writer_errors():
    from sledgehamr_gb300.output import H5Error, level_datasets_host
    boxes = [((0, 0, 0), (7, 7, 5))]
    cells = np.zeros(8 * 8 * 6)
    with pytest.raises(H5Error):  # 6 cells are not a multiple of 4
        level_datasets_host(boxes, cells, ["a"], 0., 0, 8, False, 4, 32)
    with pytest.raises(H5Error):  # not a power of 2
        level_datasets_host(boxes, cells, ["a"], 0., 0, 8, False, 3, 32)
    with pytest.raises(H5Error):
        level_datasets_host(boxes, cells, ["a"], 0., 0, 8, False, 1, 16)
    f = level_datasets_host(boxes, cells, ["a"], 0., 0, 8, False, 2, 64)
    assert len(f) == 1 + 1 + 6


def test_spectra_files(tmp_path):
    from sledgehamr_gb300 import output
    ks = np.array([0, 1, 2, 3, 4, 5, 6, 8])
    p = str(tmp_path / "spectra.hdf5")
    output.write_spectra(p, 2.5, 16, ks, {"phi": np.arange(8.0), "dphi": np.ones(8)})
    r = hdf5_read.File(p)
    assert r.keys() == ["Header", "dphi", "k_sq", "phi"]
    assert r["Header"].tolist() == [2.5, 16.0, 8.0]
    assert r["k_sq"].tolist() == ks.tolist()
    p = str(tmp_path / "gw.hdf5")
    output.write_gw_spectrum(p, 2.5, 16, 8.0, 2, True, ks, np.arange(8.0) ** 2)
    r = hdf5_read.File(p)
    assert r["Header"].tolist() == [2.5, 16.0, 8.0, 8.0, 2.0, 1.0]
    assert r["Spectrum"].tolist() == (np.arange(8.0) ** 2).tolist()
    p = str(tmp_path / "proj.hdf5")
    d = np.arange(16.0).reshape(4, 4)
    n = np.full((4, 4), 3, dtype=np.int32)
    output.write_projections(p, 1.0, 4, {"energy": (d, n)})
    r = hdf5_read.File(p)
    assert r.keys() == ["Header", "energy_data", "energy_n"]
    assert r["energy_data"].tolist() == d.reshape(-1).tolist()
    assert r["energy_n"].dtype == np.float64 and r["energy_n"].tolist() == [3.0] * 16


def _chop(N, mg):
    return [((x, y, z), (x + mg - 1, y + mg - 1, z + mg - 1))
            for z in range(0, N, mg) for y in range(0, N, mg) for x in range(0, N, mg)]


def _to_boxes_layout(field, boxes):
    """field[n, x, y, z] -> boxes layout (per box, per component, x fastest)."""
    out = []
    for lo, hi in boxes:
        blk = field[:, lo[0]:hi[0] + 1, lo[1]:hi[1] + 1, lo[2]:hi[2] + 1]
        out.append(blk.transpose(0, 3, 2, 1).reshape(-1))
    return np.concatenate(out)


@pytest.mark.parametrize("downsample", [1, 2])
def test_files_reassemble_as_pysledgehamr_reads_them(tmp_path, downsample):
    """pySledgehamr's Output reassembles a level from the per-box datasets
    and their bounds (Output.py __Read3dField / __Read2dField); done here on
    the written files, it gives back the level's field (block-averaged for
    downsample 2) and its planes."""
    from sledgehamr_gb300.output import level_datasets_host, slices_datasets_host
    rng = np.random.default_rng(5)
    N, names = 32, ["Phi", "dPhi"]
    field = rng.standard_normal((2, N, N, N))
    boxes = _chop(N, 16)
    rng.shuffle(boxes)
    cells = _to_boxes_layout(field, boxes)
    p = str(tmp_path / "0.hdf5")
    level_datasets_host(boxes, cells, names, 0.5, 0, N, False, downsample, 64).write(p)
    r = hdf5_read.File(p)
    for f, name in enumerate(names):
        d = N // downsample
        got = np.full((d, d, d), np.nan)
        lx, ly, lz = (r[f"le{a}_data"].astype(int) // downsample for a in "xyz")
        hx, hy, hz = (r[f"he{a}_data"].astype(int) // downsample for a in "xyz")
        for b in range(len(lx)):
            got[lx[b]:hx[b], ly[b]:hy[b], lz[b]:hz[b]] = r[f"{name}_data_{b + 1}"].reshape(
                hx[b] - lx[b], hy[b] - ly[b], hz[b] - lz[b])
        want = field[f].reshape(d, downsample, d, downsample, d, downsample).mean(axis=(1, 3, 5))
        np.testing.assert_allclose(got, want, rtol=0, atol=1e-14)
    loc = (0.25, 0.5, 0.75)
    p = str(tmp_path / "s.hdf5")
    slices_datasets_host(boxes, cells, names, 0.5, 0, N, False, loc).write(p)
    r = hdf5_read.File(p)
    for f, name in enumerate(names):
        for a, ax in enumerate("xyz"):
            got = np.full((N, N), np.nan, dtype=np.float32)
            le1, le2 = r[f"le1_{ax}"].astype(int), r[f"le2_{ax}"].astype(int)
            he1, he2 = r[f"he1_{ax}"].astype(int), r[f"he2_{ax}"].astype(int)
            for b in range(len(le1)):
                got[le1[b]:he1[b], le2[b]:he2[b]] = r[f"{name}_{ax}_{b + 1}"].reshape(
                    he1[b] - le1[b], he2[b] - le2[b])
            s = int(N * loc[a])
            s += s % 2
            want = np.take(field[f], s, axis=a).astype(np.float32)
            np.testing.assert_array_equal(got, want)


def test_output_abi_rejects_bad_arguments():
    import ctypes as C
    from sledgehamr_gb300 import _lib
    from sledgehamr_gb300._lib import ShBox
    lib = _lib.load()
    assert lib.sh_h5_create(None) < 0
    h = C.c_void_p()
    assert lib.sh_h5_create(C.byref(h)) == 0
    x = np.zeros(4)
    px = C.c_void_p(x.ctypes.data)
    assert lib.sh_h5_add(None, b"a", 8, px, 4) < 0
    assert lib.sh_h5_add(h, None, 8, px, 4) < 0
    assert lib.sh_h5_add(h, b"a", 8, None, 4) < 0
    assert lib.sh_h5_add(h, b"a", 8, px, -1) < 0
    assert lib.sh_h5_add(h, b"a", 3, px, 4) < 0
    assert lib.sh_h5_add(h, b"a", 8, None, 0) == 0  # an empty dataset
    assert lib.sh_h5_write(h, None) < 0
    assert lib.sh_h5_last_error(h)
    box = (ShBox * 1)()
    box[0].hi[:] = [7, 7, 7]
    names = (C.c_char_p * 1)(b"phi")
    cells = np.zeros(512)
    pc = C.c_void_p(cells.ctypes.data)
    loc = (C.c_double * 3)(0.5, 0.5, 0.5)
    assert lib.sh_output_level_host(box, 1, 1, pc, names, 0.0, 0, 8, 0, 1, 32, None) < 0
    assert lib.sh_output_level_host(box, 1, 1, None, names, 0.0, 0, 8, 0, 1, 32, h) < 0
    assert lib.sh_output_level_host(box, 1, 1, pc, None, 0.0, 0, 8, 0, 1, 32, h) < 0
    assert lib.sh_output_level_host(box, -1, 1, pc, names, 0.0, 0, 8, 0, 1, 32, h) < 0
    bad = (C.c_char_p * 1)(b"a/b")
    assert lib.sh_output_level_host(box, 1, 1, pc, bad, 0.0, 0, 8, 0, 1, 32, h) < 0
    assert lib.sh_output_slices_host(box, 1, 1, pc, names, 0.0, 0, 8, 0, None, h) < 0
    assert lib.sh_output_slices_host(box, 1, 1, pc, names, 0.0, 0, 8, 0, loc, h) == 0
    n = C.c_longlong()
    assert lib.sh_h5_count(h, C.byref(n)) == 0 and n.value == 1 + 3 * (1 + 1 + 4)
    assert lib.sh_output_level(None, None, 0, 0, 1, 32, h) < 0
    assert lib.sh_output_slices(None, None, 0, 0, loc, h) < 0
    s = C.c_char_p()
    assert lib.sh_project_comp_name(0, -1, C.byref(s)) < 0
    assert lib.sh_project_comp_name(0, 4, C.byref(s)) == 0 and s.value == b"u_xx"
    assert lib.sh_project_comp_name(0, 16, C.byref(s)) < 0
    assert lib.sh_project_comp_name(99, 0, C.byref(s)) < 0
    assert lib.sh_h5_destroy(h) == 0


def test_output_headers_build_without_cuda(tmp_path):
    """The HDF5 writer and the dataset assembly are plain C++ (g++, no CUDA
    headers)."""
    import shutil
    import subprocess
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    src = tmp_path / "t.cpp"
    src.write_text('#include "sh_output.h"\nint main() { sh::h5::Writer w; '
                   'return (int)w.size(); }\n')
    r = subprocess.run([gxx, "-std=c++17", "-fopenmp", "-Wall", "-Werror", "-fsyntax-only",
                        "-I" + os.path.join(root, "include"),
                        "-I" + os.path.join(root, "sledgehamr_gb300", "csrc"), str(src)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def _literal_level_loop(boxes, cells, names, ident, te, downsample, precision):
    """level_writer.h:88-148 as literal per-cell loops (k, j, i), small
    cases only: pins the vectorised oracle's order of operations."""
    T = np.float32 if precision == 32 else np.float64
    ndist = 2 if te else 1
    gd = downsample * ndist
    volfac = 1.0 / float(downsample) ** 3
    out = {}
    base = 0
    for b, (lo, hi) in enumerate(boxes):
        lx, ly, lz = lo
        hx, hy, hz = (hi[d] + 1 for d in range(3))
        dimx, dimy, dimz = (hx - lx) // gd, (hy - ly) // gd, (hz - lz) // gd
        vol = (hx - lx) * (hy - ly) * (hz - lz)
        for f, name in enumerate(names):
            arr = [T(0)] * (dimx * dimy * dimz)
            src = cells[base + f * vol: base + (f + 1) * vol]
            for k in range(lz, hz):
                for j in range(ly, hy):
                    for i in range(lx, hx):
                        if te and (i % 2 or j % 2 or k % 2):
                            continue
                        ind = (i - lx) // gd * dimy * dimz + (j - ly) // gd * dimz + (k - lz) // gd
                        v = float(src[(i - lx) + (hx - lx) * ((j - ly) + (hy - ly) * (k - lz))])
                        if te:
                            c = T(v)
                            arr[ind] = arr[ind] if c < arr[ind] else c
                        else:
                            arr[ind] = T(float(arr[ind]) + v * volfac)
            out[f"{name}_{ident}_{b + 1}"] = np.array(arr, dtype=T)
        base += vol * len(names)
    return out


@pytest.mark.parametrize("precision", [32, 64])
@pytest.mark.parametrize("downsample,te", [(1, False), (2, False), (4, False), (1, True),
                                           (2, True)])
def test_vectorised_level_oracle_equals_literal_loops(precision, downsample, te):
    rng = np.random.default_rng(3)
    boxes = [((0, 0, 0), (7, 7, 7)), ((8, 0, 0), (15, 7, 15))]
    names = ["a", "b"]
    nv = 8 ** 3 + 8 * 8 * 16
    cells = rng.standard_normal(nv * 2) * 10.0 ** rng.integers(-8, 9, nv * 2)
    cells[::17] = -0.0
    if te:
        cells = np.abs(cells)
    ident = "te" if te else "data"
    want = _literal_level_loop(boxes, cells, names, ident, te, downsample, precision)
    got = oo.level_datasets(boxes, cells, names, 0., 0, 16, ident, te, downsample, precision)
    for k, v in want.items():
        assert got[k].dtype == v.dtype
        np.testing.assert_array_equal(got[k].view(np.uint8), v.view(np.uint8), err_msg=k)


def _literal_slice_loop(boxes, cells, names, ident, d1, d2, d3, te, location, dim_n):
    """slices.cpp:61-128 as literal loops, small cases only."""
    ndist = 2 if te else 1
    s = int(float(dim_n) * location[d1])
    if s % 2 == 1:
        s += 1
    out, count, base = {}, 0, 0
    for lo, hi in boxes:
        ext = [hi[d] - lo[d] + 1 for d in range(3)]
        vol = ext[0] * ext[1] * ext[2]
        if lo[d1] <= s <= hi[d1]:
            count += 1
            l1, l2, h1, h2 = lo[d2], lo[d3], hi[d2] + 1, hi[d3] + 1
            dim2 = (h2 - l2) // ndist
            arr = np.zeros(((h1 - l1) // ndist) * dim2, dtype=np.float32)
            for f, name in enumerate(names):
                src = cells[base + f * vol: base + (f + 1) * vol]
                for j in range(l2, h2):
                    for i in range(l1, h1):
                        if te and (i % 2 or j % 2):
                            continue
                        c = [0, 0, 0]
                        c[d1], c[d2], c[d3] = s, i, j
                        at = (c[0] - lo[0]) + ext[0] * ((c[1] - lo[1]) + ext[1] * (c[2] - lo[2]))
                        arr[(i - l1) // ndist * dim2 + (j - l2) // ndist] = np.float32(src[at])
                out[f"{name}_{ident}_{count}"] = arr.copy()
        base += vol * len(names)
    return out


@pytest.mark.parametrize("te", [False, True])
def test_vectorised_slice_oracle_equals_literal_loops(te):
    rng = np.random.default_rng(4)
    boxes = [((0, 0, 0), (7, 7, 7)), ((8, 0, 0), (15, 7, 15)), ((0, 8, 0), (7, 15, 7))]
    names = ["a", "b"]
    nv = sum((hi[0] - lo[0] + 1) * (hi[1] - lo[1] + 1) * (hi[2] - lo[2] + 1) for lo, hi in boxes)
    cells = rng.standard_normal(nv * 2)
    for loc in [(0.0, 0.3, 0.9), (0.45, 0.5, 0.2)]:
        for ident, d1, d2, d3 in (("x", 0, 1, 2), ("y", 1, 0, 2), ("z", 2, 0, 1)):
            want = _literal_slice_loop(boxes, cells, names, ident, d1, d2, d3, te, loc, 16)
            got = oo.slice_datasets(boxes, cells, names, 0., 0, 16, ident, d1, d2, d3, te, loc)
            for k, v in want.items():
                np.testing.assert_array_equal(got[k].view(np.uint8), v.view(np.uint8), err_msg=k)
            assert sorted(k for k in got if not k.startswith(("Header", "le", "he"))) == \
                sorted(want)
