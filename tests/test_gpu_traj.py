"""Trajectory diagnostics (particle_tracking_fixed_time_step with
traj_diagnose = 1, src/tracking.c:436-447): the GPU records each particle's
state every nsteps_output steps at its offset in ptl_time, against records
made by the reference's own build (tests/golden/traj.npz).  Record times are
exact; states agree to the ulp-level differences of CUDA's sin/cos from
glibc's, grown over the run."""
import ctypes as C

import numpy as np
import pytest

import make_golden as mg
from oracle import pyoracle as po

pytestmark = pytest.mark.gpu
tp = pytest.importorskip("test_particle_gb300")
SC = mg.scenarios()


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p)


@pytest.mark.parametrize("name", ["pic", "test"])
def test_trajectory_records_match_reference(name, tmp_path, monkeypatch):
    monkeypatch.chdir(tmp_path)  # the reference API writes under data/
    (tmp_path / "data").mkdir()
    g = np.load("%s/traj.npz" % mg.HERE)
    dt, steps, every, tmax = g[name + "_meta"]
    steps, every = int(steps), int(every)
    s = SC[name]
    d = po.Domain.from_buffer_copy(s["dom"])
    d.tmax = tmax
    tp.configure(system_type=s["system_type"], charge_mass=s["charge_mass"], dom=d, grd=s["grd"],
                 mt=s["mt"], bgrid=s.get("bgrid"), egrid=s.get("egrid"))
    tp.set_spectrum(20, 1e-3, 1e1)
    p0 = np.ascontiguousarray(g[name + "_ptl0"])
    acc = np.ascontiguousarray(g[name + "_acc"], dtype=np.int32)
    n = len(p0)
    ptl_time = np.zeros(int(acc[-1]), dtype=tp.PARTICLE_DTYPE)
    ptl_time[np.concatenate([[0], acc[:-1]])] = p0
    pp = p0.copy()
    pinit = p0.copy()
    nst = np.zeros(n, dtype=np.int32)
    nspec = 20 * 2
    esp, etot, ese = np.zeros(nspec), np.zeros(nspec), np.zeros(nspec)
    epriv, eepriv = np.zeros(257 * nspec), np.zeros(257 * nspec)
    L = tp.lib()
    L.particle_tracking_fixed_time_step(C.c_int(0), C.c_int(n), C.c_double(dt), C.c_int(20), C.c_int(2),
                                        C.c_int(1), C.c_int(every), C.c_double(1.0), _ptr(acc), _ptr(pinit),
                                        _ptr(nst), _ptr(pp), _ptr(esp), _ptr(etot), _ptr(ese), _ptr(epriv),
                                        _ptr(eepriv), _ptr(ptl_time))
    ref_time, ref_p = g[name + "_ptl_time"], g[name + "_ptl"]
    assert np.array_equal(ptl_time["t"], ref_time["t"])
    # the push calls sin/cos: ulp differences from glibc, grown over the run
    rtol = 1e-8 if name == "pic" else 1e-11
    for k in ("x", "y", "z", "ux", "uy", "uz", "xshift", "yshift", "zshift"):
        np.testing.assert_allclose(ptl_time[k], ref_time[k], rtol=rtol, atol=1e-12, err_msg=k)
        np.testing.assert_allclose(pp[k], ref_p[k], rtol=rtol, atol=1e-12, err_msg=k)
    assert np.array_equal(nst, np.full(n, steps + 1))
    assert tp.device_status() == 0
