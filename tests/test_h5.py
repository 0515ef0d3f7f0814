"""The library's HDF5 files without libhdf5 (csrc/h5lite.cpp, csrc/h5io.cu),
host side, no GPU: its reader on a file libhdf5 wrote and on the variants the
oracle's independent writer makes; its writers' files read back by the
oracle's independent reader; two gloo ranks writing one file; the reference
data_io.c readers it exports.

The pin: scipy ships testhdf5_7.4_GLNX86.mat, an HDF5 file written by
libhdf5 (MATLAB 7.3 format: a 512-byte user block, superblock 0, symbol-table
root group, layout message 2), and testdouble_7.4_GLNX86.mat, the same
variable in the version 5 format scipy reads; both readers must give scipy's
values.  Neither machine has libhdf5 or h5py to open the written files."""
import ctypes as C
import os
import socket
import sys

import numpy as np
import pytest

from oracle import h5ref

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


@pytest.fixture(scope="module")
def lib():
    from test_particle_gb300 import build
    build.build()
    import test_particle_gb300 as tp
    return tp.lib()


def _scipy_mat(name):
    sio = pytest.importorskip("scipy.io")
    d = os.path.join(os.path.dirname(sio.__file__), "matlab", "tests", "data", name)
    if not os.path.exists(d):
        pytest.skip("scipy's MATLAB test files are not installed")
    return d


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p)


def _info(lib, path, group, name):
    rank, cls, size = C.c_int(), C.c_int(), C.c_int()
    dims = (C.c_ulonglong * 32)()
    rc = lib.tp_h5_info(path.encode(), group.encode(), name.encode(), C.byref(rank), dims, C.byref(cls),
                        C.byref(size))
    return rc, [dims[i] for i in range(rank.value)], cls.value, size.value


def _read(lib, path, group, name, offset, count, elem=8):
    out = np.zeros(count, dtype=np.float64 if elem == 8 else np.float32)
    r = len(count)
    rc = lib.tp_h5_read(path.encode(), group.encode(), name.encode(), r, (C.c_ulonglong * max(r, 1))(*count),
                        (C.c_ulonglong * max(r, 1))(*offset), elem, _ptr(out))
    return rc, out


def _err(lib):
    e = lib.tp_last_error
    e.restype = C.c_char_p
    return e().decode()


def test_oracle_reader_reads_a_file_libhdf5_wrote():
    sio = pytest.importorskip("scipy.io")
    h5 = _scipy_mat("testhdf5_7.4_GLNX86.mat")
    v5 = sio.loadmat(_scipy_mat("testdouble_7.4_GLNX86.mat"))["testdouble"]
    got = h5ref.read(h5, "/testdouble")
    assert got.dtype == np.dtype("<f8") and got.shape == (9, 1)
    assert np.array_equal(got.T, v5)


def test_library_reader_reads_a_file_libhdf5_wrote(lib):
    sio = pytest.importorskip("scipy.io")
    h5 = _scipy_mat("testhdf5_7.4_GLNX86.mat")
    v5 = sio.loadmat(_scipy_mat("testdouble_7.4_GLNX86.mat"))["testdouble"]
    rc, dims, cls, size = _info(lib, h5, "/", "testdouble")
    assert (rc, dims, cls, size) == (0, [9, 1], 1, 8)
    rc, out = _read(lib, h5, "", "testdouble", [0, 0], [9, 1])
    assert rc == 0 and np.array_equal(out.T, v5)
    rc, out = _read(lib, h5, "/", "testdouble", [3, 0], [4, 1], elem=4)
    assert rc == 0 and np.array_equal(out.ravel(), v5.ravel()[3:7].astype(np.float32))


def _particles(n, seed):
    import test_particle_gb300 as tp
    rng = np.random.default_rng(seed)
    p = np.zeros(n, dtype=tp.PARTICLE_DTYPE)
    for k in p.dtype.names:
        p[k] = rng.normal(size=n) * 10.0 ** rng.integers(-300, 300, size=n)
    return p


@pytest.mark.parametrize("n", [0, 1, 70001, 300007])  # the last on several threads
def test_particles_fields_file_reads_back_exactly(lib, tmp_path, n):
    """The reference's file: /particles_fields/particles [ntot] of
    {x,y,z,qm,ux,uy,uz,t} and /particles_fields/fields [ntot] of
    {Bx,By,Bz,Ex,Ey,Ez}, big-endian doubles (src/particle_info.c:452-489,
    src/emfields.c:227-257); every value back bit for bit."""
    import test_particle_gb300 as tp
    p = _particles(n, 1)
    emf = np.random.default_rng(2).normal(size=(n, 6))
    fn = str(tmp_path / "particles_fields_init.h5")
    assert lib.tp_h5_write_particles_fields(fn.encode(), 1, C.c_ulonglong(n), C.c_ulonglong(0), n, _ptr(p),
                                            _ptr(emf)) == 0
    f = h5ref.File(fn)
    assert f.eof == os.path.getsize(fn)
    a = f.read("/particles_fields/particles")
    b = f.read("/particles_fields/fields")
    assert a.dtype.names == ("x", "y", "z", "qm", "ux", "uy", "uz", "t")
    assert b.dtype.names == ("Bx", "By", "Bz", "Ex", "Ey", "Ez")
    assert all(a.dtype[k] == np.dtype(">f8") for k in a.dtype.names) and a.dtype.itemsize == 64
    assert a.shape == b.shape == (n,)
    for k in a.dtype.names:
        assert np.array_equal(a[k].view(np.uint64), p[k].astype(">f8").view(np.uint64)), k
    assert np.array_equal(np.stack([b[k] for k in b.dtype.names], 1) if n else np.zeros((0, 6)), emf)
    q = np.zeros(n, dtype=tp.PARTICLE_DTYPE)
    q["xshift"], q["zshift"] = 3.0, -1.0
    assert lib.tp_read_particles(0, n, None, _ptr(q), fn.encode()) == 0
    for k in ("x", "y", "z", "qm", "ux", "uy", "uz", "t"):
        assert np.array_equal(q[k], p[k]), k
    assert np.all(q["xshift"] == 3.0) and np.all(q["yshift"] == 0.0) and np.all(q["zshift"] == -1.0)


def test_read_particles_takes_any_member_order_and_type(lib, tmp_path):
    """libhdf5 converts compound members by name: the reader too (a file of
    little-endian members in another order, floats and integers, and an
    extra member)."""
    import test_particle_gb300 as tp
    n = 37
    rng = np.random.default_rng(3)
    dt = np.dtype([("t", "<f4"), ("extra", "<i8"), ("uz", ">f8"), ("uy", "<f8"), ("ux", "<i4"), ("qm", ">f4"),
                   ("z", "<f8"), ("y", ">f8"), ("x", "<f8")])
    rec = np.zeros(n, dtype=dt)
    for k in dt.names:
        rec[k] = (rng.normal(size=n) * 100).astype(dt[k])
    fn = str(tmp_path / "p.h5")
    h5ref.write(fn, {"particles_fields": {"particles": rec}}, compound_version=3)
    q = np.zeros(n + 5, dtype=tp.PARTICLE_DTYPE)
    acc = np.array([5, n + 5], dtype=np.int32)
    assert lib.tp_read_particles(1, n, _ptr(acc), _ptr(q[5:]), fn.encode()) == -1  # records [5, 42) of 37
    assert "beyond" in _err(lib)
    acc = np.array([0, n], dtype=np.int32)
    assert lib.tp_read_particles(1, n, _ptr(acc), _ptr(q), fn.encode()) == 0
    for k in ("x", "y", "z", "qm", "ux", "uy", "uz", "t"):
        assert np.array_equal(q[k][:n], rec[k].astype(np.float64)), k



def test_read_particles_refuses_a_member_outside_the_record(lib, tmp_path):
    """A compound member whose offset puts it past the end of the record
    (here 2^32 - 4: offset + size wraps in 32 bits) is refused before any
    record is converted."""
    import struct
    import test_particle_gb300 as tp
    dt = np.dtype([("x", "<f8"), ("y", "<f8"), ("z", "<f8"), ("qm", "<f8"), ("ux", "<f8"), ("uy", "<f8"),
                   ("uz", "<f8"), ("t", "<f8")])
    rec = np.zeros(4, dtype=dt)
    fn = str(tmp_path / "m.h5")
    h5ref.write(fn, {"particles_fields": {"particles": rec}}, compound_version=1)
    b = bytearray(open(fn, "rb").read())
    at = b.index(b"ux" + b"\0" * 6 + struct.pack("<I", dt.fields["ux"][1])) + 8
    b[at:at + 4] = struct.pack("<I", 0xFFFFFFFC)
    open(fn, "wb").write(bytes(b))
    q = np.zeros(4, dtype=tp.PARTICLE_DTYPE)
    assert lib.tp_read_particles(0, 4, None, _ptr(q), fn.encode()) == -1
    assert "member ux lies outside the record" in _err(lib)
    lib.tp_clear_status()

def _write_ranks(lib, fn, p, emf, counts, order):
    acc = np.cumsum(counts).astype(np.int32)
    starts = np.concatenate([[0], acc[:-1]])
    for r in order:
        a, c = int(starts[r]), int(counts[r])
        assert lib.tp_h5_write_particles_fields(fn.encode(), int(a == 0), C.c_ulonglong(len(p)), C.c_ulonglong(a),
                                                c, _ptr(p[a:a + c]), _ptr(emf[a:a + c])) == 0


def test_ranks_write_disjoint_records_in_any_order(lib, tmp_path):
    """The layout depends only on the totals: ranks writing their records in
    any order (the metadata last, first, over an old longer file) give the
    same bytes as one writer."""
    n = 1000
    p = _particles(n, 4)
    emf = np.random.default_rng(5).normal(size=(n, 6))
    one = str(tmp_path / "one.h5")
    _write_ranks(lib, one, p, emf, [n], [0])
    ref = open(one, "rb").read()
    for order in ([2, 1, 0], [0, 2, 1]):
        fn = str(tmp_path / ("ranks%d.h5" % order[0]))
        with open(fn, "wb") as fh:
            fh.write(os.urandom(len(ref) + 4096))  # stale bytes of an earlier run
        _write_ranks(lib, fn, p, emf, [300, 0, 700], order)
        assert open(fn, "rb").read() == ref


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _gloo_rank(rank, world, port, fn):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import test_particle_gb300 as tp
    from test_particle_gb300 import shard
    dist.init_process_group("gloo", rank=rank, world_size=world)
    n = 5003
    p = _particles(n, 6)
    emf = np.random.default_rng(7).normal(size=(n, 6))
    a, b = shard.shard_range(n, rank, world)
    if rank == 0:
        dist.barrier()  # rank 1 writes first
    L = tp.lib()
    assert L.tp_h5_write_particles_fields(fn.encode(), int(a == 0), C.c_ulonglong(n), C.c_ulonglong(a), b - a,
                                          _ptr(p[a:b]), _ptr(emf[a:b])) == 0
    if rank == 1:
        dist.barrier()
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_write_one_file(lib, tmp_path):
    import torch.multiprocessing as mp
    pytest.importorskip("torch.distributed")
    fn = str(tmp_path / "particle_diagnostics.h5")
    mp.start_processes(_gloo_rank, args=(2, _free_port(), fn), nprocs=2, start_method="spawn", join=True)
    n = 5003
    p = _particles(n, 6)
    a = h5ref.read(fn, "/particles_fields/particles")
    for k in a.dtype.names:
        assert np.array_equal(a[k], p[k]), k
    e = h5ref.read(fn, "/particles_fields/fields")
    assert np.array_equal(np.stack([e[k] for k in e.dtype.names], 1), np.random.default_rng(7).normal(size=(n, 6)))


def test_poincare_file_from_two_ranks(lib, tmp_path, monkeypatch):
    """tp_poincare_save, poincare_map's default writer: data/poincare_map.h5,
    /poincare_map/{xpos,ypos,zpos} [points][ncross + 1] native doubles, each
    rank its rows (src/poincare_map.c:185-235)."""
    monkeypatch.chdir(tmp_path)
    (tmp_path / "data").mkdir()
    ntot, nc = 7, 4
    rng = np.random.default_rng(8)
    xyz = rng.normal(size=(3, ntot, nc + 1))
    fn = lib.tp_poincare_save
    fn.restype = None
    for rank, (s, m) in ((1, (3, 4)), (0, (0, 3))):
        part = [np.ascontiguousarray(a[s:s + m]) for a in xyz]
        fn(rank, 2, ntot, nc, s, m, _ptr(part[0]), _ptr(part[1]), _ptr(part[2]))
    f = h5ref.File("data/poincare_map.h5")
    for name, a in zip(("xpos", "ypos", "zpos"), xyz):
        got = f.read("/poincare_map/" + name)
        assert got.dtype == np.dtype("<f8") and np.array_equal(got, a)
    assert lib.tp_h5_write_poincare(b"data/x.h5", 2, 1, 1, 2, _ptr(xyz[0]), _ptr(xyz[1]), _ptr(xyz[2])) == -1


VARIANTS = {
    "contiguous_v3": dict(),
    "contiguous_v2_userblock_sb1": dict(layout_version=2, userblock=1024, superblock=1),
    "contiguous_v1_dataspace2": dict(layout_version=1, dataspace_version=2),
    "compact_v3": dict(layout="compact"),
    "compact_v2": dict(layout="compact", layout_version=2),
    "chunked_v3": dict(layout="chunked", chunks=(3, 5, 4)),
    "chunked_v2_split_header": dict(layout="chunked", chunks=(2, 3, 7), layout_version=2, split_header=True),
    "chunked_missing_with_fill": dict(layout="chunked", chunks=(4, 4, 4), drop_chunks={(1, 0, 1), (0, 1, 0)},
                                      fill=7.0),
    "chunked_two_level_btree": dict(layout="chunked", chunks=(1, 2, 3), chunk_leaf_entries=5),
    "split_header": dict(split_header=True, fill=1.0),
    "chunked_deflate": dict(layout="chunked", chunks=(3, 5, 4), filters=("deflate",)),
    "chunked_shuffle_deflate_fletcher32": dict(layout="chunked", chunks=(4, 4, 4),
                                               filters=("shuffle", "deflate", "fletcher32"),
                                               unfiltered_chunks={(0, 0, 0), (1, 1, 1)}),
}


@pytest.mark.parametrize("variant", sorted(VARIANTS))
@pytest.mark.parametrize("dtype", ["<f4", ">f4", "<f8", ">f8", "<i2", ">u4"])
def test_library_reader_variants(lib, tmp_path, variant, dtype):
    """Every storage variant of the earliest format the oracle writes, read
    whole and by random hyperslabs through tp_h5_read, equals numpy."""
    kw = dict(VARIANTS[variant])
    rng = np.random.default_rng(9)
    a = (np.abs(rng.normal(size=(7, 9, 10))) * 1000 - (0 if "u" in dtype else 500)).astype(dtype)
    b = (np.abs(rng.normal(size=(11,))) * 1000).astype(dtype)
    fn = str(tmp_path / "v.h5")
    chunks = kw.pop("chunks", None)
    if chunks is not None:
        kw["chunks"] = {"Timestep_3/sub/cbx": chunks, "top": (4,)}
    tree = {"top": b, "Timestep_3": {"sub": {"cbx": a}, "z": np.arange(3.0)}}
    h5ref.write(fn, tree, **kw)
    want = a.astype(np.float64)
    if "drop_chunks" in kw:
        for idx in kw["drop_chunks"]:
            want[tuple(slice(i * c, (i + 1) * c) for i, c in zip(idx, chunks))] = np.float64(
                np.asarray(kw["fill"], dtype=dtype))
    assert np.array_equal(h5ref.read(fn, "/Timestep_3/sub/cbx").astype(np.float64), want)
    rc, dims, cls, size = _info(lib, fn, "Timestep_3/sub", "cbx")
    assert (rc, dims, cls, size) == (0, [7, 9, 10], 0 if dtype[1] in "iu" else 1, np.dtype(dtype).itemsize)
    rc, out = _read(lib, fn, "/Timestep_3/sub", "cbx", [0, 0, 0], [7, 9, 10])
    assert rc == 0 and np.array_equal(out, want)
    rc, out = _read(lib, fn, "/Timestep_3/sub/", "cbx", [0, 0, 0], [7, 9, 10], elem=4)
    assert rc == 0 and np.array_equal(out, want.astype(np.float32))
    for _ in range(6):
        off = [int(rng.integers(0, s)) for s in a.shape]
        cnt = [int(rng.integers(1, s - o + 1)) for s, o in zip(a.shape, off)]
        rc, out = _read(lib, fn, "/Timestep_3/sub", "cbx", off, cnt)
        assert rc == 0
        assert np.array_equal(out, want[tuple(slice(o, o + c) for o, c in zip(off, cnt))])
    rc, out = _read(lib, fn, "/", "top", [2], [9])
    assert rc == 0 and np.array_equal(out, b[2:].astype(np.float64))


def test_reference_data_io_readers(lib, tmp_path):
    """read_data_serial_{float,double}_h5 / _binary under the reference's names
    (src/data_io.c:22-120): the 4-D hyperslab read of read_vfields_double_h5
    (src/velocity_field.c:165-245) and the binary reads of the .gda loaders."""
    rng = np.random.default_rng(10)
    u = rng.normal(size=(3, 4, 5, 6))
    fn = str(tmp_path / "u4d.h5")
    h5ref.write(fn, {"u4d": {"ux4d": u}})
    out = np.zeros((1, 4, 5, 6))
    cnt, off = (C.c_ulonglong * 4)(1, 4, 5, 6), (C.c_ulonglong * 4)(2, 0, 0, 0)
    f = lib.read_data_serial_double_h5
    f.restype = None
    f(4, cnt, off, fn.encode(), b"/u4d", b"ux4d", _ptr(out))
    assert np.array_equal(out[0], u[2])
    out32 = np.zeros((1, 4, 5, 6), dtype=np.float32)
    g = lib.read_data_serial_float_h5
    g.restype = None
    g(4, cnt, off, fn.encode(), b"/u4d", b"ux4d", _ptr(out32))
    assert np.array_equal(out32[0], u[2].astype(np.float32))
    raw = rng.normal(size=100).astype(np.float32)
    bn = str(tmp_path / "bx_0.gda")
    raw.tofile(bn)
    got = np.zeros(30, dtype=np.float32)
    h = lib.read_data_serial_float_binary
    h.restype = None
    h(bn.encode(), C.c_long(40), C.c_long(30), _ptr(got))
    assert np.array_equal(got, raw[40:70])
    raw64 = rng.normal(size=50)
    raw64.tofile(bn)
    got64 = np.zeros(10)
    k = lib.read_data_serial_double_binary
    k.restype = None
    k(bn.encode(), C.c_long(5), C.c_long(10), _ptr(got64))
    assert np.array_equal(got64, raw64[5:15])


def test_reader_refusals_name_the_reason(lib, tmp_path):
    fn = str(tmp_path / "a.h5")
    h5ref.write(fn, {"g": {"d": np.zeros((2, 3))}})
    assert _info(lib, fn, "g", "missing")[0] == -1 and "no object named 'missing'" in _err(lib)
    assert _info(lib, fn, "nogroup", "d")[0] == -1 and "no object named 'nogroup'" in _err(lib)
    rc, _ = _read(lib, fn, "g", "d", [1, 0], [2, 3])
    assert rc == -1 and "beyond the dataset's extent" in _err(lib)
    rc, _ = _read(lib, fn, "g", "d", [0], [2])
    assert rc == -1 and "rank 2" in _err(lib)
    assert _info(lib, str(tmp_path / "absent.h5"), "g", "d")[0] == -1 and "cannot open" in _err(lib)
    # a superblock of the newer format (version 2)
    b = bytearray(open(fn, "rb").read())
    b[8] = 2
    open(fn, "wb").write(bytes(b))
    assert _info(lib, fn, "g", "d")[0] == -1 and "superblock version 2" in _err(lib)
    with pytest.raises(h5ref.H5Error):
        h5ref.read(fn, "/g/d")
    # not an HDF5 file
    open(fn, "wb").write(b"\0" * 4096)
    assert _info(lib, fn, "g", "d")[0] == -1 and "no HDF5 superblock" in _err(lib)


def test_filtered_chunks_are_refused(lib, tmp_path):
    """Chunks that went through a filter (a chunk key's filter mask set, as
    deflate leaves it): the reader says so instead of returning the stored
    bytes."""
    fn = str(tmp_path / "f.h5")
    h5ref.write(fn, {"d": np.arange(24.0).reshape(4, 6)}, layout="chunked", chunks=(2, 3))
    b = bytearray(open(fn, "rb").read())
    f = h5ref.File(fn)
    _, _, layout, _, _ = f.info("/d")
    a = f._a(layout[1])
    used = int.from_bytes(b[a + 6:a + 8], "little")
    ks = 8 + 8 * 3
    for i in range(used):
        b[a + 24 + i * (ks + 8) + 4] = 1
    open(fn, "wb").write(bytes(b))
    rc, _ = _read(lib, fn, "/", "d", [0, 0], [4, 6])
    assert rc == -1 and "filtered chunk" in _err(lib)


_FUZZ_CHILD = r"""
import ctypes as C, os, sys
import numpy as np
sys.path.insert(0, sys.argv[1])
import test_particle_gb300 as tp
L = tp.lib()
src, work, seed, n = sys.argv[2], sys.argv[3], int(sys.argv[4]), int(sys.argv[5])
base = bytearray(open(src, "rb").read())
rng = np.random.default_rng(seed)
ok = err = 0
for it in range(n):
    b = bytearray(base)
    for _ in range(int(rng.integers(1, 4))):
        i = int(rng.integers(0, len(b)))
        b[i] = int(rng.integers(0, 256)) if rng.random() < 0.7 else b[i] ^ (1 << int(rng.integers(0, 8)))
    open(work, "wb").write(bytes(b))
    for grp, name in (("/Timestep_3/sub", "cbx"), ("/", "top")):
        rank, cls, size = C.c_int(), C.c_int(), C.c_int()
        dims = (C.c_ulonglong * 32)()
        if L.tp_h5_info(work.encode(), grp.encode(), name.encode(), C.byref(rank), dims, C.byref(cls),
                        C.byref(size)) != 0:
            err += 1
            continue
        r = rank.value
        cnt = [min(int(dims[d]), 16) for d in range(r)]
        out = np.zeros(max(int(np.prod(cnt)) if r else 1, 1))
        rc = L.tp_h5_read(work.encode(), grp.encode(), name.encode(), r, (C.c_ulonglong * max(r, 1))(*cnt),
                          (C.c_ulonglong * max(r, 1))(*([0] * r)), 8, out.ctypes.data_as(C.c_void_p))
        ok += rc == 0
        err += rc != 0
    q = np.zeros(4, dtype=tp.PARTICLE_DTYPE)
    L.tp_read_particles(0, 4, None, q.ctypes.data_as(C.c_void_p), work.encode())
print("FUZZ", ok, err)
"""


@pytest.mark.parametrize("layout", ["contiguous", "chunked"])
def test_corrupted_files_give_errors_not_crashes(lib, tmp_path, layout):
    """Random byte changes anywhere in a file: every call returns data or an
    error status (run in a child process, so a crash fails the test)."""
    import subprocess
    rng = np.random.default_rng(14)
    fn = str(tmp_path / "base.h5")
    kw = {"layout": "chunked", "chunks": {"Timestep_3/sub/cbx": (3, 4, 5), "top": (4,)}} if layout == "chunked" else {}
    h5ref.write(fn, {"top": rng.normal(size=11), "Timestep_3": {"sub": {"cbx": rng.normal(size=(7, 9, 10))}}}, **kw)
    r = subprocess.run([sys.executable, "-c", _FUZZ_CHILD, ROOT, fn, str(tmp_path / "work.h5"), "15", "600"],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    line = [ln for ln in r.stdout.splitlines() if ln.startswith("FUZZ")]
    assert line, r.stdout[-2000:]
    ok, err = (int(v) for v in line[0].split()[1:])
    assert ok > 0 and err > 0


def test_unknown_filters_are_refused(lib, tmp_path):
    """A chunk filter other than deflate, shuffle and Fletcher-32 (here the
    id of a third-party compressor): refused with its number."""
    fn = str(tmp_path / "u.h5")
    h5ref.write(fn, {"d": np.arange(24.0).reshape(4, 6)}, layout="chunked", chunks=(2, 3), filters=("deflate",))
    b = bytearray(open(fn, "rb").read())
    at = b.index(b"deflate\0") - 8  # the filter's id field
    assert int.from_bytes(b[at:at + 2], "little") == 1
    b[at:at + 2] = (32001).to_bytes(2, "little")
    open(fn, "wb").write(bytes(b))
    rc, _ = _read(lib, fn, "/", "d", [0, 0], [4, 6])
    assert rc == -1 and "filter 32001" in _err(lib)
    assert _info(lib, fn, "/", "d")[0] == 0  # the dataset's description still reads


def test_trajectory_diagnostics_rejects_what_it_cannot_do(lib):
    """More than one process (the reference gathers counts over MPI), an empty
    set or more trajectory particles than particles: errors before any GPU
    work."""
    import test_particle_gb300 as tp
    p = np.zeros(8, dtype=tp.PARTICLE_DTYPE)
    nst = np.zeros(8, dtype=np.int32)
    every = C.c_int(4)
    f = lib.tp_trajectory_diagnostics
    f.argtypes = [C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_int, C.c_int, C.c_void_p, C.c_void_p,
                  C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_int, C.c_int, C.c_void_p]
    for rank, size, n, ntraj in ((0, 2, 8, 2), (1, 1, 8, 2), (0, 1, 0, 1), (0, 1, 8, 9), (0, 1, 8, 0)):
        assert f(rank, size, n, 0.1, 1.0, ntraj, 4, _ptr(p), None, _ptr(nst), 10, 2, C.byref(every), 0, 0,
                 _ptr(p)) == -1
        assert "tp_trajectory_diagnostics" in _err(lib)
    lib.tp_clear_status()


def test_layouts_the_reader_cannot_index_are_refused(lib, tmp_path):
    """Layout messages that name no storage the reader knows: a version 2
    message of class 7 (classes are 0 compact, 1 contiguous, 2 chunked), and
    a chunked layout on a scalar dataspace (a chunk needs a rank).  Both are
    refused when the dataset is opened."""
    import struct
    fn = str(tmp_path / "c.h5")
    h5ref.write(fn, {"d": np.arange(12.0).reshape(3, 4)}, layout_version=2)
    b = bytearray(open(fn, "rb").read())
    at = b.index(bytes([2, 3, 1]) + b"\0" * 5)
    b[at + 2] = 7
    open(fn, "wb").write(bytes(b))
    assert _info(lib, fn, "/", "d")[0] == -1 and "layout class 7" in _err(lib)
    rc, _ = _read(lib, fn, "/", "d", [0, 0], [3, 4])
    assert rc == -1 and "layout class 7" in _err(lib)
    fn = str(tmp_path / "s.h5")
    h5ref.write(fn, {"s": np.float64(2.5)})
    assert h5ref.read(fn, "/s") == 2.5
    b = bytearray(open(fn, "rb").read())
    addr = h5ref.File(fn).info("/s")[2][1]
    at = b.index(bytes([3, 1]) + struct.pack("<QQ", addr, 8))
    # version 3, chunked, dimensionality 1 (the element size only), never written
    b[at:at + 15] = bytes([3, 2, 1]) + b"\xff" * 8 + struct.pack("<I", 8)
    open(fn, "wb").write(bytes(b))
    assert _info(lib, fn, "/", "s")[0] == -1 and "chunked layout of a scalar" in _err(lib)
    rc, _ = _read(lib, fn, "/", "s", [], [])
    assert rc == -1 and "chunked layout of a scalar" in _err(lib)
    lib.tp_clear_status()


def test_large_transfers_split_across_threads(lib, tmp_path):
    """Reads of 16 MiB or more run as slices on several threads: a 24 MB
    dataset read whole or from an offset comes back bit for bit (odd sizes, so
    the last slice is short), and so do 32 MB per coordinate written whole."""
    rng = np.random.default_rng(5)
    fn = str(tmp_path / "big.h5")
    v = rng.normal(size=3_000_001)
    h5ref.write(fn, {"d": v})
    rc, out = _read(lib, fn, "/", "d", [0], [len(v)])
    assert rc == 0 and np.array_equal(out, v)
    rc, out = _read(lib, fn, "/", "d", [17], [2_500_000])
    assert rc == 0 and np.array_equal(out, v[17:2_500_017])
    n, nc = 1_000_003, 3
    xyz = rng.normal(size=(3, n, nc + 1))
    fn = str(tmp_path / "p.h5")
    assert lib.tp_h5_write_poincare(fn.encode(), n, nc, 0, n, _ptr(xyz[0]), _ptr(xyz[1]), _ptr(xyz[2])) == 0
    f = h5ref.File(fn)
    for name, a in zip(("xpos", "ypos", "zpos"), xyz):
        assert np.array_equal(f.read("/poincare_map/" + name), a)


@pytest.mark.parametrize("layout", ["compact_v2", "chunked_shuffle_deflate"])
def test_reader_under_sanitizers(tmp_path, layout):
    """The reader built with AddressSanitizer and UndefinedBehaviorSanitizer
    (tests/h5lite_fuzz.cpp) on 4,000 files, each with one or two bytes changed
    outside the raw data: every open, description and read either succeeds or
    is refused, with no invalid access and no undefined behaviour."""
    import shutil
    import subprocess
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("no g++")
    exe = str(tmp_path / "fuzz")
    r = subprocess.run([gxx, "-O1", "-g", "-std=c++17", "-fsanitize=address,undefined",
                        "-fno-sanitize-recover=undefined", "-I", os.path.join(ROOT, "test_particle_gb300", "csrc"),
                        "-o", exe, os.path.join(ROOT, "tests", "h5lite_fuzz.cpp"), "-ldl"],
                       capture_output=True, text=True)
    if r.returncode != 0 and "asan" in r.stderr.lower():
        pytest.skip("sanitizer runtime not available")
    assert r.returncode == 0, r.stderr[-2000:]
    rng = np.random.default_rng(1)
    dt = np.dtype([(k, ">f8") for k in ("x", "y", "z", "qm", "ux", "uy", "uz", "t")])
    tree = {"top": rng.normal(size=7), "g": {"d": rng.normal(size=(4, 5, 3))},
            "particles_fields": {"particles": np.zeros(6, dtype=dt)}}
    kw = dict(layout="compact", layout_version=2) if layout == "compact_v2" else \
        dict(layout="chunked", chunks={"g/d": (2, 3, 2), "top": (3,)}, filters=("shuffle", "deflate"))
    fn = str(tmp_path / "base.h5")
    h5ref.write(fn, tree, compound_version=1, **kw)
    f = h5ref.File(fn)
    mask = np.ones(os.path.getsize(fn), bool)
    for path in ("/top", "/g/d", "/particles_fields/particles"):
        dims, dtype, lay = f.info(path)[:3]
        if lay[0] == "contiguous" and lay[1] != h5ref.UNDEF:
            a = lay[1] + f.base
            mask[a:a + int(np.prod(dims)) * dtype.itemsize] = False
    pos = str(tmp_path / "pos.bin")
    np.nonzero(mask)[0].astype(np.int64).tofile(pos)
    env = dict(os.environ, ASAN_OPTIONS="detect_leaks=0")
    r = subprocess.run([exe, fn, pos, str(tmp_path / "work.h5"), "4000", "11"], capture_output=True, text=True,
                       timeout=600, env=env)
    assert r.returncode == 0, (r.stdout[-500:], r.stderr[-3000:])
    ok, refused = (int(v) for v in r.stdout.split()[1:3])
    assert ok > 0 and refused > 0
