"""HDF5 files through the GPU: PIC field files read straight into device
memory (tp_read_pic_fields_h5) against the reference build's records, and
particles_fields files written with the fields from the GPU get_emf
(tp_save_particles_fields).

The PIC files hold the reference reader's input in C order ([nx][ny][nz],
src/magnetic_field.c:632-692): the records after the library's transpose must
equal the reference build's records for the same values
(tests/golden/fields.npz, made by the reference's binary readers, whose
scaling is the same data * B0 into float records)."""
import numpy as np
import pytest

import make_golden as mg
from oracle import h5ref
from oracle import pyoracle as po

pytestmark = pytest.mark.gpu
tp = pytest.importorskip("test_particle_gb300")
import test_gpu_fields as gf  # noqa: E402

NAMES = ("cbx", "cby", "cbz", "ex", "ey", "ez")


def _c_order(comp, nx, ny, nz):
    """A component in the reference's x-fastest order as the PIC file's [nx][ny][nz] array."""
    return np.ascontiguousarray(comp.reshape(nz, ny, nx).transpose(2, 1, 0))


@pytest.mark.parametrize("dtype,kw", [
    ("<f4", {}),
    (">f4", {"layout": "chunked", "chunks": (5, 3, 4)}),
    ("<f8", {"layout_version": 2}),
    (">f8", {"split_header": True}),
    ("<f4", {"pad": (3, 1, 2)}),
    ("<f4", {"layout": "compact"}),
    ("<f4", {"layout": "chunked", "chunks": (4, 4, 4), "filters": ("shuffle", "deflate")}),
])
def test_records_match_reference_reader(tmp_path, dtype, kw):
    f, ct, _, _ = gf.setup(tmp_path)
    nx, ny, nz = (int(v) for v in f["dims"][:3])
    kw = dict(kw)
    pad = kw.pop("pad", (0, 0, 0))
    grp = {}
    for c, name in enumerate(NAMES):
        a = _c_order(f["comps"][c], nx, ny, nz).astype(dtype)
        big = np.full((nx + pad[0], ny + pad[1], nz + pad[2]), 99.0, dtype=dtype)
        big[:nx, :ny, :nz] = a  # the reference reads the block at the origin
        grp[name] = big
    fn = str(tmp_path / ("fields_%d.h5" % ct))
    h5ref.write(fn, {"Timestep_%d" % ct: grp}, **kw)
    tp.read_pic_fields_h5(fn, "Timestep_%d" % ct)
    he, hb = tp.fetch_device_fields()
    assert np.array_equal(hb.ravel(), f["records_b"])
    assert np.array_equal(he.ravel(), f["records_e"])
    assert tp.device_status() == 0
    tp.release_device_fields()


def test_double_files_round_to_float_first(tmp_path):
    """The reference's float reader of a double file: H5Dread converts to
    float, then data * B0 into float records."""
    f, ct, _, _ = gf.setup(tmp_path)
    nx, ny, nz = (int(v) for v in f["dims"][:3])
    b0, e0 = (float(v) for v in f["scale"])
    rng = np.random.default_rng(11)
    grp = {n: rng.normal(size=(nx, ny, nz)) * 10.0 ** rng.integers(-3, 4, size=(nx, ny, nz)) for n in NAMES}
    fn = str(tmp_path / "d.h5")
    h5ref.write(fn, {"T": grp})
    tp.read_pic_fields_h5(fn, "/T")
    he, hb = tp.fetch_device_fields()
    for c, n in enumerate(NAMES):
        want = (grp[n].astype(np.float32).astype(np.float64) * (b0 if c < 3 else e0)).astype(np.float32)
        got = (hb if c < 3 else he)[:, c % 3].reshape(nz, ny, nx).transpose(2, 1, 0)
        assert np.array_equal(got, want), n
    tp.release_device_fields()


@pytest.mark.parametrize("b0", [0.75, 2.0])
def test_large_grid_streams_in_pieces_b_only(tmp_path, b0):
    """A 320 x 256 x 256 grid (84 MB per component: two staging pieces) and B
    only: E records zero; a power-of-two B0 takes the FP32 product, others the
    reference's double product, both giving the reference's floats."""
    nx, ny, nz = 320, 256, 256
    dom = tp.Domain()
    dom.xmax, dom.ymax, dom.zmax = nx - 1.0, ny - 1.0, nz - 1.0
    grd = tp.Grids()
    grd.nx, grd.ny, grd.nz, grd.nt = nx, ny, nz, 1
    grd.dx = grd.dy = grd.dz = 1.0
    tp.configure(system_type=tp.SYS_PIC, dom=dom, grd=grd)
    import ctypes as C
    L = tp.lib()
    L.set_variables_bfield(C.byref(grd), C.byref(dom), C.c_double(b0), C.c_int(0), C.c_int(4))
    rng = np.random.default_rng(12)
    grp = {n: rng.normal(size=(nx, ny, nz)).astype(np.float32) for n in NAMES[:3]}
    fn = str(tmp_path / "big.h5")
    h5ref.write(fn, {"Timestep_0": grp})
    tp.read_pic_fields_h5(fn, "Timestep_0", with_e=False)
    he, hb = tp.fetch_device_fields()
    assert not he.any()
    for c, n in enumerate(NAMES[:3]):
        want = (grp[n].astype(np.float64) * b0).astype(np.float32).transpose(2, 1, 0).ravel()
        assert np.array_equal(hb[:, c], want), n
    tp.release_device_fields()


def test_bad_files_are_errors(tmp_path):
    f, ct, _, _ = gf.setup(tmp_path)
    nx, ny, nz = (int(v) for v in f["dims"][:3])
    fn = str(tmp_path / "bad.h5")
    h5ref.write(fn, {"G": {"cbx": np.zeros((nx, ny, nz), np.float32), "cby": np.zeros((nx, ny), np.float32),
                           "cbz": np.zeros((nx - 1, ny, nz), np.float32)}})
    for group, msg in (("G", "cby is not an array"), ("H", "no object named 'H'")):
        with pytest.raises(RuntimeError, match=msg):
            tp.read_pic_fields_h5(fn, group, with_e=False)
    with pytest.raises(RuntimeError, match="no object named 'ex'"):
        h5ref.write(fn, {"G": {n: np.zeros((nx, ny, nz), np.float32) for n in NAMES[:3]}})
        tp.read_pic_fields_h5(fn, "G")
    with pytest.raises(RuntimeError, match="not floating point"):
        h5ref.write(fn, {"G": {n: np.zeros((nx, ny, nz), np.int32) for n in NAMES}})
        tp.read_pic_fields_h5(fn, "G")


def test_saved_fields_are_the_gpu_get_emf_and_the_oracle(tmp_path):
    """particles_fields_init.h5 of the gridded PIC scenario written by two
    ranks: the records as given, the fields equal tp.get_emf at (x, y, z, t)
    and the oracle's (the reference's get_emf restated, bit-exact for the
    gridded fields); read back by tp_read_particles."""
    s = mg.scenarios()["pic"]
    tp.configure(system_type=s["system_type"], charge_mass=s["charge_mass"], dom=s["dom"], grd=s["grd"],
                 mt=s["mt"], bgrid=s.get("bgrid"), egrid=s.get("egrid"))
    d = s["dom"]
    rng = np.random.default_rng(13)
    n = 4099
    p = np.zeros(n, dtype=tp.PARTICLE_DTYPE)
    p["x"] = rng.uniform(d.xmin, d.xmax, n)
    p["y"] = rng.uniform(d.ymin, d.ymax, n)
    p["z"] = rng.uniform(d.zmin, d.zmax, n)
    p["ux"], p["uy"], p["uz"] = rng.normal(size=(3, n))
    p["qm"] = -1.0
    fn = str(tmp_path / "particles_fields_init.h5")
    tp.save_particles_fields(fn, p[2000:], ntot=n, offset=2000)
    tp.save_particles_fields(fn, p[:2000], ntot=n)
    a = h5ref.read(fn, "/particles_fields/particles")
    for k in a.dtype.names:
        assert np.array_equal(a[k], p[k]), k
    e = h5ref.read(fn, "/particles_fields/fields")
    emf = np.stack([e[k] for k in ("Bx", "By", "Bz", "Ex", "Ey", "Ez")], 1)
    xyzt = np.stack([p["x"], p["y"], p["z"], p["t"]], 1)
    assert np.array_equal(emf, tp.get_emf(xyzt))
    f = mg.field_from(s)
    assert np.array_equal(emf, po.get_emf(f, xyzt))
    q = tp.read_particles(fn, n - 10, offset=10)
    for k in ("x", "y", "z", "qm", "ux", "uy", "uz", "t"):
        assert np.array_equal(q[k], p[k][10:]), k
    assert tp.device_status() == 0


@pytest.mark.parametrize("scale", [1.0, 0.25])
def test_saved_pic_file_round_trips(tmp_path, scale):
    """tp_save_pic_fields_h5 writes the device fields as the reference's PIC
    file: its datasets are the records reordered to C order and divided by
    B0 (E0); loading it back gives the same records (B0 and E0 powers of two);
    the oracle's restatement of the reference's reorder loop gives them too."""
    import ctypes as C
    nx, ny, nz = 40, 33, 17
    dom = tp.Domain()
    dom.xmax, dom.ymax, dom.zmax = nx - 1.0, ny - 1.0, nz - 1.0
    grd = tp.Grids()
    grd.nx, grd.ny, grd.nz, grd.nt = nx, ny, nz, 1
    grd.dx = grd.dy = grd.dz = 1.0
    tp.configure(system_type=tp.SYS_PIC, dom=dom, grd=grd)
    L = tp.lib()
    L.set_variables_bfield(C.byref(grd), C.byref(dom), C.c_double(scale), C.c_int(0), C.c_int(4))
    L.set_variables_efield(C.byref(grd), C.byref(dom), C.c_double(scale / 2), C.c_int(0), C.c_int(4))
    import test_particle_gb300.workloads as wl
    mb = wl.kolmogorov_modes(64, 1, 6, 0.5, 41)
    mv = wl.kolmogorov_modes(64, 1, 6, 0.1, 42)
    tp.synth_pic_fields(mb, mv, 1.0)
    he, hb = tp.fetch_device_fields()
    fn = str(tmp_path / "fields_0.h5")
    tp.save_pic_fields_h5(fn, "/Timestep_0")
    f = h5ref.File(fn)
    for c, n in enumerate(NAMES):
        got = f.read("/Timestep_0/" + n)
        assert got.dtype == np.dtype("<f4") and got.shape == (nx, ny, nz)
        rec = (hb if c < 3 else he)[:, c % 3]
        want = (rec.astype(np.float64) / (scale if c < 3 else scale / 2)).astype(np.float32)
        assert np.array_equal(got, want.reshape(nz, ny, nx).transpose(2, 1, 0)), n
        ref = np.zeros((nx * ny * nz, 3), np.float32)
        po.pic_records_from_c(got, scale if c < 3 else scale / 2, c % 3, ref)
        assert np.array_equal(ref[:, c % 3], rec), n
    tp.release_device_fields()
    tp.read_pic_fields_h5(fn, "Timestep_0")
    he2, hb2 = tp.fetch_device_fields()
    assert np.array_equal(he2, he) and np.array_equal(hb2, hb)
    tp.release_device_fields()
