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


def _hybrid(L, n, dt, nb, nt, every, acc, traj, p_init, nst, p, p_time):
    I, D, V = C.c_int, C.c_double, C.c_void_p
    L.particle_tracking_hybrid.argtypes = [I, I, D, I, I, I, I, D, V, I, I, V, V, V, V]
    L.particle_tracking_hybrid(0, n, dt, nb, nt, 0, every, 1.0, None if acc is None else _ptr(acc), 0, traj,
                               _ptr(p_init), _ptr(nst), _ptr(p), None if p_time is None else _ptr(p_time))


def test_trajectory_diagnostics_file(tmp_path, monkeypatch):
    """tp_trajectory_diagnostics (src/diagnostics.c:403-568, one process): the
    particles sorted by final energy, their initial states reloaded from
    data/particles_fields_init.h5, every interval-th chosen from the highest
    energy down, tracked again with records, written to
    data/particle_diagnostics.h5 -- the records equal a direct tracking of the
    same choice (the tracking itself is checked against the reference above),
    the fields the GPU get_emf at each record."""
    from oracle import h5ref
    monkeypatch.chdir(tmp_path)
    (tmp_path / "data").mkdir()
    s = SC["pic"]
    dt, steps, nb, nt, every = 0.05, 120, 20, 2, 8
    d = po.Domain.from_buffer_copy(s["dom"])
    d.tmax = steps * dt + 0.5 * dt
    tp.configure(system_type=s["system_type"], charge_mass=s["charge_mass"], dom=d, grd=s["grd"], mt=s["mt"],
                 bgrid=s.get("bgrid"), egrid=s.get("egrid"))
    tp.set_spectrum(nb, 1e-3, 1e1)
    n, ntraj_tot = 96, 8
    p0 = mg.particles_for(s, np.random.default_rng(3), n)
    tp.save_particles_fields("data/particles_fields_init.h5", p0)
    L = tp.lib()
    p = p0.copy()
    p_init = p0.copy()
    nst = np.zeros(n, dtype=np.int32)
    _hybrid(L, n, dt, nb, nt, every, None, 0, p_init, nst, p, None)
    # the expected choice, restated: stable energy order, init states, uniform interval from the top
    ene = np.sqrt(1.0 + p["ux"] ** 2 + p["uy"] ** 2 + p["uz"] ** 2) - 1.0
    idx = np.argsort(ene, kind="stable")
    q = np.zeros(n, dtype=tp.PARTICLE_DTYPE)
    for k in ("x", "y", "z", "qm", "ux", "uy", "uz", "t"):
        q[k] = p0[k][idx]
    nst_sorted = nst[idx].copy()
    interval = n // ntraj_tot
    chosen = [n - 1 - i * interval for i in range(ntraj_tot)]
    acc = np.cumsum([(nst_sorted[j] - 1) // every + 1 for j in chosen]).astype(np.int32)
    pt = np.ascontiguousarray(q[chosen])
    ptime = np.zeros(int(acc[-1]), dtype=tp.PARTICLE_DTYPE)
    ptime[np.concatenate([[0], acc[:-1]])] = pt
    nst_exp = nst_sorted.copy()
    _hybrid(L, ntraj_tot, dt, nb, nt, every, acc, 1, p_init.copy(), nst_exp, pt, ptime)
    # the library's one call, through the Python binding
    p2, nst2, every2 = p.copy(), nst.copy(), C.c_int(every)
    assert tp.trajectory_diagnostics(p2, nst2, p_init.copy(), dt, ntraj_tot, nb, nt, every,
                                     s["system_type"]) == every
    for k in ("x", "y", "z", "qm", "ux", "uy", "uz", "t"):
        assert np.array_equal(p2[k], q[k]), k
    assert np.array_equal(nst2, nst_exp)
    got = h5ref.read("data/particle_diagnostics.h5", "/particles_fields/particles")
    assert len(got) == len(ptime)
    for k in got.dtype.names:
        assert np.array_equal(got[k], ptime[k]), k
    e = h5ref.read("data/particle_diagnostics.h5", "/particles_fields/fields")
    xyzt = np.stack([ptime["x"], ptime["y"], ptime["z"], ptime["t"]], 1)
    assert np.array_equal(np.stack([e[k] for k in ("Bx", "By", "Bz", "Ex", "Ey", "Ez")], 1), tp.get_emf(xyzt))
    assert L.tp_trajectory_diagnostics(0, 2, n, dt, 1.0, ntraj_tot, s["system_type"], _ptr(p2), None, _ptr(nst2),
                                       nb, nt, C.byref(every2), 0, 0, _ptr(p_init.copy())) == -1
    L.tp_clear_status()
