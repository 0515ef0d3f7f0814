"""Batched adaptive Bulirsch-Stoer on the GPU against the reference's stepper
(golden vectors, one particle per fresh reference process) and the oracle."""
import numpy as np
import pytest

import make_golden as mg
from oracle import pyoracle as po

pytestmark = pytest.mark.gpu
tp = pytest.importorskip("test_particle_gb300")
import ctypes as C  # noqa: E402

import test_particle_gb300.workloads as wl  # noqa: E402

SC = mg.scenarios()


def configure_loop():
    s = SC["loop"]
    tp.configure(system_type=tp.SYS_WLCS, charge_mass=s["charge_mass"], bc_flag=2, dom=s["dom"],
                 wl=s["wl"], ibessel=0)


def bs_steps(y0, h0, nsteps, atol=1e-5, rtol=1e-14, kmaxx=8, uform=0):
    y = np.ascontiguousarray(y0, dtype=np.float64).copy()
    n = len(y)
    rec = np.zeros((n, nsteps, 8))
    tp.check(tp.lib().tp_bs_steps(C.c_int(n), tp._ptr(y), C.c_double(0.0), C.c_double(h0),
                                  C.c_int(nsteps), C.c_double(atol), C.c_double(rtol), C.c_int(kmaxx),
                                  C.c_int(uform), tp._ptr(rec)), "bs_steps")
    return rec


def test_bs_steps_vs_reference():
    """Reference tolerances (atol 1e-5, rtol 1e-14): steps before the
    reference's first non-finite value agree to 1e-8 relative."""
    bs = np.load("%s/bs.npz" % mg.HERE)
    configure_loop()
    rec = bs_steps(bs["y0"], float(bs["h0"][0]), bs["out"].shape[1])
    for i in range(len(bs["y0"])):
        ref = bs["out"][i]
        bad = np.where(~np.isfinite(ref).all(axis=1))[0]
        upto = bad[0] if len(bad) else len(ref)
        assert upto >= 10
        got = rec[i, :upto]
        assert np.isfinite(got).all()
        err = np.abs(got - ref[:upto]) / (np.abs(ref[:upto]).max(axis=0) + 1e-300)
        assert err.max() < 1e-8, (i, err.max())


def test_bs_steps_vs_oracle_tight_tolerance():
    configure_loop()
    y0 = wl.torus_particles(64, 1.0, 0.05, 0.3, 0.1, 0.9, 21)
    rec = bs_steps(y0, 1e-6, 60, atol=1e-10, rtol=1e-10)
    f = mg.field_from(SC["loop"], bc_flag=2)
    for i in range(0, 64, 8):
        ref = po.bs_integrate(f, y0[i], 0.0, 1e-6, 60, atol=1e-10, rtol=1e-10)
        err = np.abs(rec[i] - ref) / (np.abs(ref).max(axis=0) + 1e-300)
        # libm ulps shift the controller's step sizes; orbits then separate slowly
        assert err[:3].max() < 1e-9, (i, err[:3].max())
        assert err.max() < 1e-4, (i, err.max())


def test_bs_production_run():
    """Every particle reaches t_end through the frame times; beta-form |beta|
    is conserved in a static magnetic field to the integration tolerance."""
    configure_loop()
    n, t_end, nt_out, nbins = 4096, 0.01, 5, 100
    tp.set_spectrum(nbins, 1e-3, 1e1)
    y0 = wl.torus_particles(n, 1.0, 0.05, 0.3, 0.1, 0.9, 5)
    y = y0.copy()
    t = np.zeros(n)
    steps = np.zeros(n, dtype=np.int32)
    st = np.zeros(n, dtype=np.int32)
    esp = np.zeros(nt_out * nbins)
    dfr = np.zeros(8 * (nt_out + 1))
    info = tp.RunInfo()
    tp.check(tp.lib().tp_bs_run(C.c_int(n), tp._ptr(y), tp._ptr(t), C.c_double(t_end), C.c_int(nt_out),
                                C.c_int(nbins), C.c_double(1e-6), C.c_double(1e-10), C.c_double(1e-10),
                                C.c_int(8), C.c_int(0), C.c_int(1000000), tp._ptr(steps), tp._ptr(st),
                                tp._ptr(esp), tp._ptr(dfr), C.byref(info)), "bs_run")
    assert (st == 0).all(), np.unique(st, return_counts=True)
    assert np.all(t == t_end)
    assert (steps > 0).all() and steps.max() > steps.min()
    assert esp.reshape(nt_out, nbins).sum(axis=1).tolist() == [n] * nt_out
    b0 = np.linalg.norm(y0[:, 3:], axis=1)
    b1 = np.linalg.norm(y[:, 3:], axis=1)
    assert np.max(np.abs(b1 - b0) / b0) < 1e-6
    assert info.pushes == steps.sum()
