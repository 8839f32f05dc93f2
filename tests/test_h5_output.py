"""CPU checks of the library's HDF5 encoder (tag_h5_write), which writes the
solution files of SaveSolutionCallback
(src/callbacks_step/save_solution_2d_manifold_in_3d_cartesian.jl:44-118) with
no HDF5 library present.

The checker is tests/h5_reader.py, a strict reader written from the file
format specification.  The reader is pinned first on a file written by the
HDF5 library itself (a MATLAB 7.3 file that scipy ships as test data, whose
content scipy's own tests give as pi/4 * (0..8)); then the encoder's
messages are compared byte for byte with the ones the HDF5 library wrote
there, and written files are read back."""
import ctypes
import os
import struct

import numpy as np
import pytest

from h5_reader import H5File, H5FormatError


def _hdf5_library_file():
    sm = pytest.importorskip("scipy.io.matlab")
    p = os.path.join(os.path.dirname(sm.__file__), "tests", "data", "testhdf5_7.4_GLNX86.mat")
    if not os.path.exists(p):
        pytest.skip("scipy's HDF5 test file is not installed")
    return p


@pytest.fixture(scope="module")
def out(tg):
    import importlib
    tg._lib.load()
    return importlib.import_module("trixiatmo_gb300.output")


def test_reader_reads_a_file_written_by_the_hdf5_library():
    f = H5File(_hdf5_library_file())
    assert f.names == ["testdouble"]
    d = f.datasets["testdouble"]
    assert d.data.shape == (9, 1)
    assert np.array_equal(d.data.ravel(), np.pi / 4 * np.arange(9))
    assert d.attrs == {"MATLAB_class": "double"}
    # that file's heap holds a real free block (the reader walked its list)
    assert f.heap[24:40] == struct.pack("<QQ", 1, len(f.heap) - 24)


def _messages(d, mtype):
    return [body for t, _flags, body in d.messages if t == mtype]


def test_encodings_match_the_hdf5_library(out, tmp_path):
    ref = H5File(_hdf5_library_file())
    p = tmp_path / "a.h5"
    out.write_h5(p, {"s": "double"}, [("x", np.arange(3.0), "double")])
    ours = H5File(p)
    rd, od = ref.datasets["testdouble"], ours.datasets["x"]
    # IEEE binary64 little-endian datatype and the fill-value message
    assert _messages(od, 3)[0][:20] == _messages(rd, 3)[0][:20]
    assert _messages(od, 5) == _messages(rd, 5)
    # attribute: the same scalar dataspace; the string type differs only in
    # the character set (UTF-8 here, as HDF5.jl writes; ASCII there)
    ra, oa = _messages(rd, 12)[0], _messages(od, 12)[0]
    assert oa[8:8 + 8] == b"name\0\0\0\0"
    ref_name_pad = (struct.unpack_from("<H", ra, 2)[0] + 7) & ~7
    r_t = ra[8 + ref_name_pad:8 + ref_name_pad + 8]
    o_t = oa[16:24]
    assert r_t[0] == o_t[0] == 0x13 and r_t[2:] == o_t[2:] and (r_t[1], o_t[1]) == (0x00, 0x10)
    assert ra[8 + ref_name_pad + 8:8 + ref_name_pad + 16] == oa[24:32]   # scalar dataspace
    # superblock: the same version-0 fields and group K values
    rb, ob = ref.b[ref.sb:ref.sb + 20], ours.b[:20]
    assert rb[:20] == ob[:20]


def test_round_trip_values_bit_for_bit(out, tmp_path):
    rng = np.random.default_rng(7)
    special = np.array([0.0, -0.0, np.inf, -np.inf, 5e-324, -2.2250738585072014e-308,
                        1.7976931348623157e308])
    nan = np.frombuffer(struct.pack("<Q", 0x7FF8_0000_DEAD_BEEF), "<f8")
    sets = [(f"variables_{k}", rng.standard_normal(k * 7 + 1), f"v{k}") for k in range(1, 41)]
    sets += [("special", np.concatenate([special, nan]), None), ("empty", np.zeros(0), "e")]
    attrs = {"i_min": -2 ** 63, "i_max": 2 ** 63 - 1, "zero": 0, "pi": np.pi, "tiny": 5e-324,
             "utf8": "ρθ — Δ", "empty": "", "a" * 300: "long name"}
    p = tmp_path / "r.h5"
    out.write_h5(p, attrs, sets)
    f = H5File(p)
    assert f.names == sorted(n for n, _, _ in sets)          # strcmp order
    assert f.attrs == attrs
    assert type(f.attrs["i_max"]) is int and type(f.attrs["pi"]) is float
    for name, arr, var in sets:
        d = f.datasets[name]
        assert d.data.dtype == np.float64 and d.data.shape == (arr.size,)
        assert d.data.tobytes() == np.asarray(arr, np.float64).tobytes()
        assert d.attrs == ({} if var is None else {"name": var})
    # 42 entries: six symbol-table nodes of at most eight under one B-tree node
    tree = struct.unpack_from("<Q", _messages_root(f)[0], 0)[0]
    assert struct.unpack_from("<H", f.b, tree + 6)[0] == 6
    # the data are stored once, after the metadata
    assert len(f.b) - sum(8 * a.size for _, a, _ in sets) == min(
        struct.unpack_from("<Q", _messages(d, 8)[0], 2)[0]
        for d in f.datasets.values() if d.data.size)


def _messages_root(f):
    return [body for t, _flags, body in f.root_messages if t == 0x11]


def test_trixi_solution_layout(out, tmp_path):
    """The attributes and datasets of save_solution_2d_manifold_in_3d_cartesian.jl:72-115."""
    data = np.arange(12.0).reshape(3, 4)
    p = out.write_solution_file(tmp_path / "solution_000000010.h5", data, ("h", "h_vcon1", "h_vcon2"),
                                ndims=2, equations="CovariantShallowWaterEquations2D", polydeg=3,
                                n_elements=2, mesh_type="P4estMesh", mesh_file="mesh.h5",
                                time=0.25, dt=1e-3, timestep=10,
                                element_variables={"indicator": np.ones(2)},
                                node_variables={"vorticity_node": np.zeros(4)})
    f = H5File(p)
    assert f.attrs == {"ndims": 2, "equations": "CovariantShallowWaterEquations2D", "polydeg": 3,
                       "n_vars": 3, "n_elements": 2, "mesh_type": "P4estMesh",
                       "mesh_file": "mesh.h5", "time": 0.25, "dt": 1e-3, "timestep": 10}
    assert list(f.attrs) == ["ndims", "equations", "polydeg", "n_vars", "n_elements", "mesh_type",
                             "mesh_file", "time", "dt", "timestep"]
    for v, name in enumerate(("h", "h_vcon1", "h_vcon2")):
        d = f.datasets[f"variables_{v + 1}"]
        assert np.array_equal(d.data, data[v]) and d.attrs == {"name": name}
    assert f.datasets["element_variables_1"].attrs == {"name": "indicator"}
    assert f.datasets["node_variables_1"].attrs == {"name": "vorticity_node"}


def test_rejects_bad_input(out, tg, tmp_path):
    E = tg._lib.TagError
    with pytest.raises(E, match="duplicate dataset"):
        out.write_h5(tmp_path / "d.h5", {}, [("a", [1.0], None), ("a", [2.0], None)])
    with pytest.raises(E, match="name empty or with"):
        out.write_h5(tmp_path / "d.h5", {}, [("a/b", [1.0], None)])
    with pytest.raises(E, match="at most 256"):
        out.write_h5(tmp_path / "d.h5", {}, [(f"x{k}", [1.0], None) for k in range(257)])
    with pytest.raises(E) as ei:
        out.write_h5(tmp_path / "missing_dir" / "d.h5", {}, [("a", [1.0], None)])
    assert ei.value.code == tg._lib.TAG_E_IO
    # through the C ABI: a bad attribute type and a negative count
    L = tg._lib.load()
    a = tg._lib.H5Attribute(b"x", 7, 0, 0.0, None)
    assert L.tag_h5_write(str(tmp_path / "d.h5").encode(), ctypes.byref(a), 1, None, 0) == 1
    d = tg._lib.H5Dataset(b"x", None, -1, None)
    assert L.tag_h5_write(str(tmp_path / "d.h5").encode(), None, 0, ctypes.byref(d), 1) == 1
    # 256 is the limit and is written
    out.write_h5(tmp_path / "full.h5", {}, [(f"x{k:03d}", [float(k)], None) for k in range(256)])
    f = H5File(tmp_path / "full.h5")
    assert len(f.names) == 256 and f.datasets["x255"].data[0] == 255.0


def test_reader_is_strict(out, tmp_path):
    """The checker rejects what an HDF5 library would: a truncated file, a
    wrong end-of-file address, a broken B-tree key order."""
    p = tmp_path / "s.h5"
    out.write_h5(p, {"a": 1}, [(f"v{k}", [float(k)], None) for k in range(12)])
    b = bytearray(open(p, "rb").read())
    open(tmp_path / "t.h5", "wb").write(b[:-8])
    with pytest.raises(H5FormatError):
        H5File(tmp_path / "t.h5")
    f = H5File(p)
    tree = struct.unpack_from("<Q", _messages_root(f)[0], 0)[0]
    bad = bytearray(b)
    # key 1 (last name of the first node) swapped with key 2
    k1, k2 = tree + 24 + 16, tree + 24 + 32
    bad[k1:k1 + 8], bad[k2:k2 + 8] = b[k2:k2 + 8], b[k1:k1 + 8]
    open(tmp_path / "k.h5", "wb").write(bad)
    with pytest.raises(H5FormatError):
        H5File(tmp_path / "k.h5")
