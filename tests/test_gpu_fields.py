"""Field files read straight into device memory (tp_read_pic_fields_binary)
against the reference's binary readers (tests/golden/fields.npz, made by
read_bfields_binary / read_efields_binary of the reference build): the
records are bit-identical, and tracking on the loaded fields equals tracking
on the same arrays passed as host fields."""
import ctypes as C

import numpy as np
import pytest

import make_golden as mg

pytestmark = pytest.mark.gpu
tp = pytest.importorskip("test_particle_gb300")
import test_particle_gb300.workloads as wl  # noqa: E402


def setup(tmp_path):
    f = np.load("%s/fields.npz" % mg.HERE)
    nx, ny, nz, ct = (int(v) for v in f["dims"])
    b0, e0 = (float(v) for v in f["scale"])
    for c, name in enumerate(("bx", "by", "bz", "ex", "ey", "ez")):
        f["comps"][c].tofile(str(tmp_path / ("%s_%d.gda" % (name, ct))))
    dom = tp.Domain()
    dom.xmax, dom.ymax, dom.zmax = nx - 1.0, ny - 1.0, nz - 1.0
    dom.tmax = 40 * 0.05 + 0.025
    grd = tp.Grids()
    grd.nx, grd.ny, grd.nz, grd.nt = nx, ny, nz, 1
    grd.dx = grd.dy = grd.dz = 1.0
    tp.configure(system_type=tp.SYS_PIC, dom=dom, grd=grd)
    L = tp.lib()
    L.set_variables_bfield(C.byref(grd), C.byref(dom), C.c_double(b0), C.c_int(0), C.c_int(4))
    L.set_variables_efield(C.byref(grd), C.byref(dom), C.c_double(e0), C.c_int(0), C.c_int(4))
    return f, ct, dom, grd


def test_records_match_reference_reader(tmp_path):
    f, ct, _, _ = setup(tmp_path)
    tp.read_pic_fields_binary(str(tmp_path) + "/", ct)
    he, hb = tp.fetch_device_fields()
    assert np.array_equal(hb.ravel(), f["records_b"])
    assert np.array_equal(he.ravel(), f["records_e"])
    assert tp.device_status() == 0
    tp.release_device_fields()


def test_missing_file_is_an_error(tmp_path):
    f, ct, _, _ = setup(tmp_path)
    with pytest.raises(RuntimeError):
        tp.read_pic_fields_binary(str(tmp_path) + "/", ct + 1)


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_tracking_on_loaded_fields_equals_host_fields(tmp_path, prec):
    f, ct, dom, grd = setup(tmp_path)
    code = tp.PREC_FP64 if prec == "fp64" else tp.PREC_MIXED
    tp.set_spectrum(50, 1e-3, 1e1)
    p0 = wl.shell_particles(300, 0.5, (0, 0, 0), (dom.xmax, dom.ymax, dom.zmax), 4)
    tp.read_pic_fields_binary(str(tmp_path) + "/", ct)
    a = tp.track(p0, 0.05, 2, 50, precision=code)
    tp.release_device_fields()
    # the same records as host arrays (the reference's layout)
    eh = np.ascontiguousarray(f["records_e"])
    bh = np.ascontiguousarray(f["records_b"])
    tp.configure(system_type=tp.SYS_PIC, dom=dom, grd=grd, egrid=eh, bgrid=bh)
    tp.set_spectrum(50, 1e-3, 1e1)
    b = tp.track(p0, 0.05, 2, 50, precision=code)
    for k in ("x", "y", "z", "ux", "uy", "uz"):
        assert np.array_equal(a["ptl"][k], b["ptl"][k]), k
    assert np.array_equal(a["espect"], b["espect"])
    assert np.array_equal(a["dsum"], b["dsum"])
    assert tp.device_status() == 0
