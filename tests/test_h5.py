"""HDF5 files written and read without h5py (pyloki_gb300.h5), the
pruning result files on top of them (pyloki_gb300.results,
io/cands.py:106-411), and the periodogram's NetCDF file.

No HDF5 library is installed, so the format is pinned two ways:
- the encoder's datatype, dataspace and attribute bytes against those
  libhdf5 itself wrote into a MATLAB 7.3 file (the constants below were read
  from scipy's test file ``testhdf5_7.4_GLNX86.mat``, which the reader also
  opens when it is installed);
- round trips through the reader of every type, shape and group size the
  result files use, including groups larger than one B-tree node.
"""

from __future__ import annotations

import struct
import zlib
from pathlib import Path

import numpy as np
import pytest

from pyloki_gb300 import h5
from pyloki_gb300.results import (LEVEL_DTYPE, TIMER_DTYPE, PruneResultWriter,
                                  PruneStatsCollection, merge_prune_result_files,
                                  read_prune_results)

# datatype / dataspace message bytes as libhdf5 wrote them into the MATLAB
# file: IEEE float64 little-endian, a 6-byte null-terminated ASCII string, a
# (9, 1) simple dataspace (version 1, no maximum dimensions)
LIBHDF5_F64 = bytes.fromhex("11203f0008000000000040003" "40b0034ff030000")
LIBHDF5_S6 = bytes.fromhex("1300000006000000")
LIBHDF5_SPACE_9x1 = bytes.fromhex("0102000000000000" "0900000000000000" "0100000000000000")
MATLAB_FILE = Path(np.__file__).parents[1] / "scipy/io/matlab/tests/data/testhdf5_7.4_GLNX86.mat"


def test_bool_is_the_h5py_enum():
    """numpy bool is stored as h5py stores it: an int8 enumeration with
    FALSE = 0 and TRUE = 1, and read back as bool."""
    msg = h5._dtype_message(np.dtype(np.bool_))
    assert msg[0] == 0x18 and msg[1] == 2  # enumeration, version 1, two members
    assert h5._decode_dtype(msg, 0)[0]["np"] == np.dtype(np.bool_)


def test_encodings_match_libhdf5():
    assert h5._dtype_message(np.dtype("<f8")) == LIBHDF5_F64
    assert h5._dtype_message(np.dtype("S6")) == LIBHDF5_S6
    assert h5._Writer.dataspace((9, 1)) == LIBHDF5_SPACE_9x1
    # the decoder reads the libhdf5 bytes back to the same types
    assert h5._decode_dtype(LIBHDF5_F64, 0)[0]["np"] == np.dtype("<f8")
    assert h5._decode_dtype(LIBHDF5_S6, 0)[0]["np"] == np.dtype("S6")


@pytest.mark.skipif(not MATLAB_FILE.exists(), reason="scipy's HDF5 test file is absent")
def test_reads_a_libhdf5_file():
    """A file written by libhdf5 (MATLAB 7.3: 512-byte user block, symbol-
    table root group, layout message version 2, fixed-string attribute)."""
    f = h5.read_file(MATLAB_FILE)
    assert list(f) == ["testdouble"]
    ds = f["testdouble"]
    np.testing.assert_array_equal(ds.data[:, 0], np.arange(9) * np.pi / 4)
    assert ds.attrs["MATLAB_class"] == b"double"


def _sample_tree() -> h5.Group:
    rng = np.random.default_rng(5)
    root = h5.Group()
    root.attrs.update({"version": "0.1.0", "names": ["freq", "accel", "jerk", "ω"],
                       "n": np.int64(128), "x": 1.5, "arr": np.arange(6, dtype=np.int16)})
    for dt in ("i1", "i2", "i4", "i8", "u1", "u2", "u4", "u8", "f4", "f8", "f2"):
        root.create_dataset(f"types/{dt}", data=(rng.standard_normal((3, 5)) * 50).astype(dt))
    root.create_dataset("types/big_endian", data=np.arange(7, dtype=">f8"))
    root.create_dataset("types/bytes", data=np.array([b"ab", b"cde", b""]))
    root.create_dataset("types/strings", data=np.array(["x", "", "long string ✓"], dtype=object))
    root.create_dataset("types/scalar", data=np.float64(2.5))
    root.create_dataset("types/empty", data=np.zeros((0, 4), np.float32))
    stats = np.zeros(4, LEVEL_DTYPE)
    stats["level"] = np.arange(4)
    stats["threshold"] = [1.0, 1.5, 2.0, 2.5]
    root.create_dataset("types/compound", data=stats)
    root["types/compound"].attrs["unit"] = "sigma"
    from pyloki_gb300.thresholds import state_dtype  # float32 fields and a bool

    states = np.zeros((3, 4), state_dtype)
    states["threshold"] = rng.random((3, 4))
    states["is_empty"] = rng.random((3, 4)) < 0.5
    root.create_dataset("types/states", data=states)
    root.create_dataset("types/bool", data=np.array([True, False, True]))
    big = root.create_group("many")  # more names than one B-tree node holds
    for k in range(700):
        big.create_dataset(f"{k:04d}_00", data=np.full(k % 3 + 1, k, np.int32))
    root.create_group("deep/er/est").attrs["leaf"] = np.float32(3)
    root.create_group("empty")
    return root


def _assert_same(a, b, path="/"):
    assert type(a) is type(b), path
    assert set(a.attrs) == set(b.attrs), path
    for k, v in a.attrs.items():
        w = b.attrs[k]
        if isinstance(v, str):
            assert w == v, (path, k)
        else:
            np.testing.assert_array_equal(np.asarray(w), np.asarray(v), err_msg=f"{path}@{k}")
    if isinstance(a, h5.Dataset):
        assert a.data.shape == b.data.shape, path
        if a.data.dtype.kind in "OS" or a.data.dtype.names:
            assert a.data.dtype == b.data.dtype, path
        else:
            assert a.data.dtype.newbyteorder("<") == b.data.dtype, path
        np.testing.assert_array_equal(a.data, b.data, err_msg=path)
        return
    assert sorted(a.members) == sorted(b.members), path
    for k in a.members:
        _assert_same(a.members[k], b.members[k], f"{path}{k}/")


def test_round_trip(tmp_path):
    root = _sample_tree()
    path = tmp_path / "t.h5"
    h5.write_file(path, root)
    raw = path.read_bytes()
    assert raw[:8] == h5.SIGNATURE and raw[8] == 0  # superblock version 0
    back = h5.read_file(path)
    _assert_same(root, back)
    assert list(back["many"]) == sorted(root["many"].members)  # B-tree order
    # read and written again: the same tree, and from then on the same bytes
    h5.write_file(tmp_path / "u.h5", back)
    back2 = h5.read_file(tmp_path / "u.h5")
    _assert_same(root, back2)
    h5.write_file(tmp_path / "v.h5", back2)
    assert (tmp_path / "v.h5").read_bytes() == (tmp_path / "u.h5").read_bytes()


def test_group_btree_levels(tmp_path):
    """Groups of 0, 1, 8, 9, 256 and 257 names: one symbol-table node, two,
    a full B-tree node of 32 symbol-table nodes, and a second B-tree level."""
    for n in (0, 1, 8, 9, 256, 257, 2100):
        g = h5.Group()
        for k in range(n):
            g.create_dataset(f"n{k:05d}", data=np.int64(k))
        h5.write_file(tmp_path / "g.h5", g)
        back = h5.read_file(tmp_path / "g.h5")
        assert list(back) == [f"n{k:05d}" for k in range(n)]
        assert [int(back[k].data) for k in back] == list(range(n))


def test_file_modes_and_copy(tmp_path):
    p = tmp_path / "f.h5"
    with h5.File(p, "w") as f:
        f.attrs["a"] = 1
        f.create_dataset("x/y", data=np.arange(3))
    with pytest.raises(FileExistsError):
        h5.File(p, "w-")
    with h5.File(p, "a") as f:
        assert "x/y" in f
        f.create_dataset("z", data=np.ones(2))
        with pytest.raises(ValueError, match="already exists"):
            f.create_dataset("z", data=np.ones(2))
    with h5.File(p, "r") as f, h5.File(tmp_path / "g.h5", "w") as g:
        np.testing.assert_array_equal(f["x/y"][:], np.arange(3))
        assert set(f) == {"x", "z"}
        f.copy("x", g)
        f.copy("z", g, name="w")
    back = h5.read_file(tmp_path / "g.h5")
    np.testing.assert_array_equal(back["x/y"].data, np.arange(3))
    np.testing.assert_array_equal(back["w"].data, np.ones(2))
    with pytest.raises(ValueError, match="not an HDF5 file"):
        (tmp_path / "bad.h5").write_bytes(b"\0" * 64)
        h5.read_file(tmp_path / "bad.h5")


def _stats(n: int, seed: int):
    from pyloki_gb300.prune import PruneStats

    rng = np.random.default_rng(seed)
    return [PruneStats(level=i, seg_idx=int(rng.integers(64)), threshold=0.1 * i,
                       score_min=float(rng.random()), score_max=float(rng.random() + 1),
                       n_branches=int(rng.integers(1, 99)), n_leaves=int(rng.integers(1, 999)),
                       n_leaves_phy=int(rng.integers(1, 999)),
                       n_leaves_surv=int(rng.integers(1, 99))) for i in range(n)]


def test_prune_result_writer_layout(tmp_path):
    """The reference's result layout (io/cands.py:277-355): file attributes,
    threshold_scheme, and per run the six datasets with the compound
    level_stats / timer_stats records."""
    path = tmp_path / "r_results.h5"
    thr = np.linspace(0, 4, 15)
    with PruneResultWriter(path) as w:
        w.write_metadata(["freq", "accel"], 16, 2**18, thr)
    with PruneResultWriter(path, mode="a") as w, pytest.raises(ValueError, match="exists"):
        w.write_metadata(["freq", "accel"], 16, 2**18, thr)  # the dataset exists already
    rng = np.random.default_rng(1)
    runs = {}
    for ref in (3, 8):
        name = f"{ref:03d}_00"
        runs[name] = (np.arange(16), rng.standard_normal((5, 2, 2)),
                      rng.random(5).astype(np.float32), rng.random(5).astype(np.float32),
                      _stats(16, ref))
        with PruneResultWriter(path, mode="a") as w:
            w.write_run_results(name, *runs[name])
            with pytest.raises(ValueError, match="already exists"):
                w.write_run_results(name, *runs[name])
    res = read_prune_results(path)
    assert res["attrs"]["pruning_version"] == "0.1.0"
    assert list(res["attrs"]["param_names"]) == ["freq", "accel"]
    assert int(res["attrs"]["nsegments"]) == 16 and int(res["attrs"]["max_sugg"]) == 2**18
    np.testing.assert_array_equal(res["threshold_scheme"], thr)
    assert sorted(res["runs"]) == sorted(runs)
    for name, (scheme, params, scores, scores_ep, stats) in runs.items():
        got = res["runs"][name]
        assert sorted(got) == sorted(["scheme", "param_sets", "scores_ep", "scores",
                                      "level_stats", "timer_stats"])
        np.testing.assert_array_equal(got["scheme"], scheme)
        np.testing.assert_array_equal(got["param_sets"], params)
        np.testing.assert_array_equal(got["scores"], scores)
        np.testing.assert_array_equal(got["scores_ep"], scores_ep)
        assert got["level_stats"].dtype == LEVEL_DTYPE
        assert got["timer_stats"].dtype == TIMER_DTYPE and got["timer_stats"].shape == (1,)
        col = PruneStatsCollection.from_arrays(got["level_stats"], got["timer_stats"])
        assert [s.n_leaves for s in col.stats_list] == [s.n_leaves for s in stats]
        np.testing.assert_array_equal(col.to_array()[0], PruneStatsCollection(stats).to_array()[0])


def test_merge_prune_result_files(tmp_path):
    """Temporary per-run files merged in reference-segment order, runs
    already present skipped, temporaries deleted (io/cands.py:365-411)."""
    main = tmp_path / "main_results.h5"
    log = tmp_path / "main_log.txt"
    log.write_text("Pruning log\n")
    with PruneResultWriter(main) as w:
        w.write_metadata(["freq"], 8, 64, np.ones(7))
        w.write_run_results("005_00", np.arange(8), np.ones((1, 2, 2)), np.ones(1, np.float32),
                            np.ones(1, np.float32), _stats(8, 0))
    for ref in (12, 5, 7):
        with PruneResultWriter(tmp_path / f"tmp_{ref:03d}_00_results.h5") as w:
            w.write_run_results(f"{ref:03d}_00", np.arange(8), np.full((1, 2, 2), ref),
                                np.full(1, ref, np.float32), np.ones(1, np.float32),
                                _stats(8, ref))
        (tmp_path / f"tmp_{ref:03d}_00_log.txt").write_text(f"run {ref}\n")
    merge_prune_result_files(tmp_path, log, main)
    assert not list(tmp_path.glob("tmp_*"))
    assert log.read_text() == "Pruning log\nrun 5\nrun 7\nrun 12\n"
    res = read_prune_results(main)
    assert sorted(res["runs"]) == ["005_00", "007_00", "012_00"]
    np.testing.assert_array_equal(res["runs"]["005_00"]["param_sets"], np.ones((1, 2, 2)))
    np.testing.assert_array_equal(res["runs"]["012_00"]["scores"], [12.0])


def _chunked_dataset_file(path, data: np.ndarray, chunk: tuple) -> None:
    """A file whose one dataset is stored as the reference writes its
    datasets (h5py, compression="gzip"): chunked, with the shuffle and
    deflate filters, indexed by a version 1 B-tree of chunk keys. Laid out
    here by the specification: layout message version 3 class 2, filter
    pipeline version 1, B-tree node type 1 (chunk size, filter mask,
    element offsets)."""
    w = h5._Writer()
    esize = data.dtype.itemsize
    rank = data.ndim
    entries = []  # (key bytes, chunk address)
    for start in np.ndindex(*[-(-s // c) for s, c in zip(data.shape, chunk)]):
        off = tuple(i * c for i, c in zip(start, chunk))
        block = np.zeros(chunk, data.dtype)
        sl = tuple(slice(o, min(o + c, s)) for o, c, s in zip(off, chunk, data.shape))
        block[tuple(slice(0, x.stop - x.start) for x in sl)] = data[sl]
        raw = np.frombuffer(block.tobytes(), np.uint8).reshape(-1, esize).T.tobytes()  # shuffle
        comp = zlib.compress(raw, 9)  # deflate
        addr = w.alloc(comp)
        key = struct.pack("<II", len(comp), 0) + b"".join(struct.pack("<Q", o) for o in off)
        entries.append((key + struct.pack("<Q", 0), addr))
    last_key = struct.pack("<II", 0, 0) + b"".join(
        struct.pack("<Q", c) for c in chunk) + struct.pack("<Q", esize)
    node = b"TREE" + struct.pack("<BBHQQ", 1, 0, len(entries), h5.UNDEF, h5.UNDEF)
    for key, addr in entries:
        node += key + struct.pack("<Q", addr)
    btree = w.alloc(node + last_key)
    layout = struct.pack("<BBBQ", 3, 2, rank + 1, btree) + b"".join(
        struct.pack("<I", c) for c in (*chunk, esize))
    pipeline = struct.pack("<BB6x", 1, 2)
    pipeline += struct.pack("<HHHH", 2, 8, 1, 1) + b"shuffle\0" + struct.pack("<I4x", esize)
    pipeline += struct.pack("<HHHH", 1, 8, 1, 1) + b"deflate\0" + struct.pack("<I4x", 9)
    hdr = w.header([w.msg(0x01, w.dataspace(data.shape)),
                    w.msg(0x03, h5._dtype_message(data.dtype), flags=1),
                    w.msg(0x08, layout), w.msg(0x0B, pipeline)])
    heap = bytearray(8) + b"gz\0" + bytes(5)
    data_addr = w.alloc(bytes(heap))
    heap_addr = w.alloc(b"HEAP" + bytes(4) + struct.pack("<QQQ", len(heap), 1, data_addr))
    snod = w.alloc(b"SNOD" + struct.pack("<BBH", 1, 0, 1) + struct.pack("<QQI4x16x", 8, hdr, 0)
                   + bytes(40 * 7))
    root_btree = w.btree([(snod, 8)])
    root = w.header([w.msg(0x11, struct.pack("<QQ", root_btree, heap_addr))])
    Path(path).write_bytes(w.finish(root, root_btree, heap_addr))


def test_reads_chunked_deflate_shuffle(tmp_path):
    """Chunked storage with ragged edge chunks, shuffle and deflate (how the
    reference's gzip-9 datasets are stored) is read back exactly."""
    rng = np.random.default_rng(3)
    for data, chunk in ((rng.standard_normal((5, 7)).astype(np.float32), (2, 4)),
                        (np.arange(10, dtype=np.int64), (4,)),
                        (rng.standard_normal((3, 4, 2)), (2, 4, 2))):
        p = tmp_path / "gz.h5"
        _chunked_dataset_file(p, data, chunk)
        np.testing.assert_array_equal(h5.read_file(p)["gz"].data, data)


def test_rejects_damaged_files(tmp_path):
    """Truncated files, a B-tree node that points back to itself and a
    continuation block that points back to itself raise ValueError instead
    of looping or reading out of the file."""
    g = h5.Group()
    g.create_dataset("x", data=np.arange(5))
    h5.write_file(tmp_path / "ok.h5", g)
    raw = (tmp_path / "ok.h5").read_bytes()
    (tmp_path / "short.h5").write_bytes(raw[: len(raw) // 2])
    with pytest.raises(ValueError):
        h5.read_file(tmp_path / "short.h5")
    # the root group's B-tree: make its single child the node itself
    r = h5._FileReader(raw)
    btree, _ = struct.unpack_from("<QQ", dict(r.messages(r.root_addr))[0x11])
    bad = bytearray(raw)
    struct.pack_into("<BBH", bad, btree + 4, 0, 1, 1)  # level 1: children are nodes
    struct.pack_into("<Q", bad, btree + 24 + 8, btree)
    (tmp_path / "cycle.h5").write_bytes(bytes(bad))
    with pytest.raises(ValueError, match="twice"):
        h5.read_file(tmp_path / "cycle.h5")
    # an object header whose continuation message points at its own messages
    w = h5._Writer()
    hdr = w.header([w.msg(0x10, struct.pack("<QQ", 0, 8)), w.msg(0x01, w.dataspace((1,)))])
    struct.pack_into("<H", w.out, hdr + 2, 5)  # claim more messages than there are
    struct.pack_into("<Q", w.out, hdr + 16 + 8, hdr + 16)
    r2 = h5._FileReader(w.finish(hdr, 0, 0))
    with pytest.raises(ValueError, match="cycle"):
        r2.messages(hdr)



def test_periodogram_netcdf_round_trip(tmp_path):
    """Periodogram.save / load (periodogram.py:165-172) in xarray's NetCDF-3
    layout: coordinate variables per parameter, the unnamed DataArray's
    variable with ``tobs`` as a double attribute, int32 integer coordinates."""
    from scipy.io import netcdf_file

    from pyloki_gb300.search import Periodogram

    rng = np.random.default_rng(4)
    params = {"accel": np.linspace(-5, 5, 3), "freq": np.linspace(1, 2, 4) * 1.1,
              "width": np.array([1, 2, 4, 8])}
    p = Periodogram(params, rng.random((3, 4, 4)).astype(np.float32), 1234.5678901234)
    path = tmp_path / "pgram.nc"
    p.save(path)
    with netcdf_file(path, "r", mmap=False) as f:
        var = f.variables[Periodogram.DATA_VAR]
        assert var.dimensions == ("accel", "freq", "width")
        assert f.variables["width"].data.dtype == np.dtype(">i4")
        assert var._attributes["tobs"].dtype == np.float64
    q = Periodogram.load(path)
    assert q.param_names == p.param_names and q.tobs == p.tobs
    np.testing.assert_array_equal(q.snrs, p.snrs)
    for k in params:
        np.testing.assert_array_equal(q.params[k], params[k])
    assert q.find_best_params() == p.find_best_params()
    (tmp_path / "x.nc").write_bytes(b"\x89HDF\r\n\x1a\n" + bytes(64))
    with pytest.raises(ValueError, match="NetCDF-3"):
        Periodogram.load(tmp_path / "x.nc")
