"""Known answers on the GPU: gyration in a uniform magnetic field (system 0,
B = z, E = 0) through the full tracking entry point, for the FP64 parity
path, the FP64 path with FMA and the mixed-precision path.  The Wirz step is
an exact rotation in a uniform field, so after N steps the momentum has
turned by N qm dt / gamma about z with |u| and u_z unchanged, and the
guiding centre x + (u x z) / qm has not moved.  Measured after 500 steps of
2048 particles (GB300): the FP64 paths stay within 3e-14 of the answer; the
mixed path drifts by about 5e-5 in |u|, 8e-5 rad in phase and 3e-5 in the
guiding centre (FP32 rotation with rsqrt-based norms), and its tolerances
are about three times that."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
tp = pytest.importorskip("test_particle_gb300")


@pytest.mark.parametrize("prec,tol_u,tol_phase,tol_x", [
    ("fp64", 1e-13, 1e-10, 1e-11),
    ("fp64fast", 1e-13, 1e-10, 1e-11),
    ("mixed", 2e-4, 3e-4, 1e-4),
])
def test_uniform_field_gyration(prec, tol_u, tol_phase, tol_x):
    code = {"fp64": tp.PREC_FP64, "fp64fast": tp.PREC_FP64_FAST, "mixed": tp.PREC_MIXED}[prec]
    n, steps, dt = 2048, 500, 0.01
    dom = tp.Domain()
    dom.xmax = dom.ymax = dom.zmax = 1.0
    dom.tmax = steps * dt + 0.5 * dt
    tp.configure(system_type=tp.SYS_TEST, charge_mass=1.0, bc_flag=0, dom=dom)
    tp.set_spectrum(200, 1e-3, 1e2)
    rng = np.random.default_rng(11)
    p0 = np.zeros(n, dtype=tp.PARTICLE_DTYPE)
    for c in ("x", "y", "z"):
        p0[c] = rng.uniform(0.0, 1.0, n)
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1)[:, None]
    u = 0.7 / np.sqrt(1 - 0.49) * d
    p0["ux"], p0["uy"], p0["uz"] = u[:, 0], u[:, 1], u[:, 2]
    p0["qm"] = 1.0
    r = tp.track(p0, dt, 1, 200, precision=code)
    assert r["estep"] == steps
    p = r["ptl"]
    assert np.all(r["nsteps"] == steps + 1)
    u0 = np.stack([p0["ux"], p0["uy"], p0["uz"]], 1)
    u1 = np.stack([p["ux"], p["uy"], p["uz"]], 1)
    gam = np.sqrt(1 + (u0 ** 2).sum(1))
    np.testing.assert_allclose(np.linalg.norm(u1, axis=1), np.linalg.norm(u0, axis=1), rtol=tol_u)
    np.testing.assert_allclose(u1[:, 2], u0[:, 2], rtol=tol_u, atol=tol_u)
    turn = np.angle((u1[:, 0] + 1j * u1[:, 1]) / (u0[:, 0] + 1j * u0[:, 1]))
    want = np.angle(np.exp(-1j * steps * dt / gam))
    err = np.angle(np.exp(1j * (turn - want)))
    assert np.abs(err).max() < tol_phase
    gc0 = np.stack([p0["x"] + p0["uy"], p0["y"] - p0["ux"]], 1)
    gc1 = np.stack([p["x"] + p["xshift"] + p["uy"], p["y"] + p["yshift"] - p["ux"]], 1)
    np.testing.assert_allclose(gc1, gc0, rtol=0, atol=tol_x)
    zz = p["z"] + p["zshift"]
    np.testing.assert_allclose(zz, p0["z"] + steps * dt * p0["uz"] / gam, rtol=0, atol=tol_x)
    assert tp.device_status() == 0


def test_spectra_beyond_32_bit_indexing_are_refused():
    """A run whose spectra [nt_out][nbins] hold more than 2^31 - 1 entries
    (the kernels index them with 32-bit integers) is refused before any
    launch."""
    dt = 0.01
    dom = tp.Domain()
    dom.xmax = dom.ymax = dom.zmax = 1.0
    dom.tmax = 70000 * dt + 0.5 * dt
    tp.configure(system_type=tp.SYS_TEST, charge_mass=1.0, bc_flag=0, dom=dom)
    tp.set_spectrum(40000, 1e-3, 1e2)
    p0 = np.zeros(4, dtype=tp.PARTICLE_DTYPE)
    p0["qm"], p0["ux"] = 1.0, 0.1
    s = tp.Session(4)
    s.load(p0)
    with pytest.raises(RuntimeError, match="60000 frames x 40000 bins: not supported"):
        s.track(dt, 60000, 40000, tp.PREC_MIXED)
    s.close()
    tp.lib().tp_clear_status()
