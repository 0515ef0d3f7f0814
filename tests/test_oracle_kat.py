"""Known-answer tests of the oracle against physics and mathematics, beside
the golden vectors of the reference build (test_oracle_golden.py): gyration
in a uniform field, the force-free property of the ABC field, the complete
elliptic integrals against the arithmetic-geometric mean, and trilinear
interpolation of a linear field (which documents the reference's x/z weight
exchange, src/interpolation.c:173-180)."""
import math

import numpy as np
import pytest

from oracle import pyoracle as po


def _particles(n, rng, speed, lo=0.2, hi=0.8):
    p = np.zeros(n, dtype=po.PARTICLE_DTYPE)
    for c in ("x", "y", "z"):
        p[c] = rng.uniform(lo, hi, n)
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1)[:, None]
    u = speed / math.sqrt(1.0 - speed ** 2)
    p["ux"], p["uy"], p["uz"] = (u * d).T
    p["qm"] = 1.0
    return p


def _domain(lo, hi):
    d = po.Domain()
    d.xmin, d.ymin, d.zmin = lo
    d.xmax, d.ymax, d.zmax = hi
    d.xmin_ptl, d.ymin_ptl, d.zmin_ptl = lo
    d.xmax_ptl, d.ymax_ptl, d.zmax_ptl = hi
    d.tmax = 1e30
    return d


def test_uniform_field_gyration():
    """B = z (system 0), E = 0: the Wirz step is an exact rotation, so after
    N steps the momentum has turned by N qm dt / gamma about z, |u| and u_z
    are unchanged and the guiding centre x + (u x z) / qm stays put."""
    rng = np.random.default_rng(1)
    p0 = _particles(64, rng, 0.5)
    p0["ux"] *= 0.2  # gyroradii well inside the box
    p0["uy"] *= 0.2
    f = po.make_field(system_type=0, charge_mass=1.0, bc_flag=2, dom=_domain((0, 0, 0), (1, 1, 1)))
    dt, n = 0.01, 500
    p, esc = po.wirz_steps(f, p0, dt, n)
    assert not esc.any()
    u0 = np.stack([p0["ux"], p0["uy"], p0["uz"]], 1)
    u1 = np.stack([p["ux"], p["uy"], p["uz"]], 1)
    gam = np.sqrt(1 + (u0 ** 2).sum(1))
    np.testing.assert_allclose(np.linalg.norm(u1, axis=1), np.linalg.norm(u0, axis=1), rtol=1e-13)
    np.testing.assert_allclose(u1[:, 2], u0[:, 2], rtol=1e-13)
    turn = np.angle((u1[:, 0] + 1j * u1[:, 1]) / (u0[:, 0] + 1j * u0[:, 1]))
    want = np.angle(np.exp(-1j * n * dt / gam))  # du/dt = qm u x z / gamma turns clockwise
    np.testing.assert_allclose(turn, want, atol=1e-10)
    gc0 = np.stack([p0["x"] + p0["uy"], p0["y"] - p0["ux"]], 1)
    gc1 = np.stack([p["x"] + p["xshift"] + p["uy"], p["y"] + p["yshift"] - p["ux"]], 1)
    np.testing.assert_allclose(gc1, gc0, atol=1e-11)
    np.testing.assert_allclose(p["z"] + p["zshift"], p0["z"] + n * dt * p0["uz"] / gam, atol=1e-11)


def test_abc_field_is_force_free():
    """A = B = C = 1: curl B = lambda B and div B = 0 (central differences)."""
    lam = 2 * np.pi
    f = po.make_field(system_type=2, abc=(1.0, 1.0, 1.0), B0=1.0, lambda0=lam,
                      dom=_domain((0, 0, 0), (1, 1, 1)))
    rng = np.random.default_rng(2)
    x = rng.uniform(0, 1, (50, 3))
    h = 1e-5

    def B(pts):
        xyzt = np.zeros((len(pts), 4))
        xyzt[:, :3] = pts
        return po.get_emf(f, xyzt)[:, :3]

    d = np.zeros((3, 3, len(x)))  # d[i][j] = dB_i / dx_j
    for j in range(3):
        e = np.zeros(3)
        e[j] = h
        d[:, j, :] = ((B(x + e) - B(x - e)) / (2 * h)).T
    curl = np.stack([d[2, 1] - d[1, 2], d[0, 2] - d[2, 0], d[1, 0] - d[0, 1]], 1)
    b = B(x)
    np.testing.assert_allclose(curl, lam * b, atol=1e-7 * lam * np.abs(b).max())
    assert np.abs(d[0, 0] + d[1, 1] + d[2, 2]).max() < 1e-7


def _agm_KE(k):
    """Complete elliptic integrals K(k), E(k) by the arithmetic-geometric mean
    (Gauss; E from the sum of the squared half-differences)."""
    a, b, c = 1.0, math.sqrt(1.0 - k * k), k
    s, p2 = 0.5 * c * c, 0.5
    for _ in range(40):  # quadratic convergence: a handful of rounds reach rounding level
        a, b, c = 0.5 * (a + b), math.sqrt(a * b), 0.5 * (a - b)
        p2 *= 2
        s += p2 * c * c
    K = math.pi / (2 * a)
    return K, K * (1 - s)


def test_elliptic_integrals_against_agm():
    """The corrected integrals follow the AGM values over the whole range of
    the modulus; the reference's own series (kept for parity) follows them
    while m = k^2 < 0.9 and departs above (its m >= 0.9 branch expands about
    the wrong point, src/wlcs.c:741-804)."""
    ks = np.concatenate([np.linspace(0.0, 0.94, 48), np.linspace(0.95, 0.999, 24)])
    E_c, K_c = po.ellint(ks, corrected=1)
    E_r, K_r = po.ellint(ks, corrected=0)
    want = np.array([_agm_KE(k) for k in ks])
    np.testing.assert_allclose(K_c, want[:, 0], rtol=1e-12)
    np.testing.assert_allclose(E_c, want[:, 1], rtol=1e-12)
    low = ks ** 2 < 0.9
    np.testing.assert_allclose(K_r[low], want[low, 0], rtol=1e-12)
    np.testing.assert_allclose(E_r[low], want[low, 1], rtol=1e-12)
    assert np.abs(K_r[~low] / want[~low, 0] - 1).max() > 1e-6


@pytest.mark.parametrize("corrected", [1, 0])
def test_trilinear_interpolation_of_a_linear_field(corrected):
    """Gridded B linear in x, y, z with dyadic coefficients (exact in FP32 at
    the nodes): the corrected weights reproduce it to FP32 rounding; the
    reference's weights reproduce it with the x and z cell fractions
    exchanged."""
    n, dx = 8, 0.5
    L = (n - 1) * dx
    dom = _domain((0, 0, 0), (L, L, L))
    grd = po.Grids()
    grd.nx = grd.ny = grd.nz = n
    grd.nt = 1
    grd.dx = grd.dy = grd.dz = dx
    coef = np.array([[1.0, 0.5, 0.25, 0.125], [-2.0, 0.25, -0.5, 1.0], [0.5, -0.125, 0.75, -0.25]])
    zz, yy, xx = np.meshgrid(np.arange(n) * dx, np.arange(n) * dx, np.arange(n) * dx, indexing="ij")
    bg = np.stack([c[0] + c[1] * xx + c[2] * yy + c[3] * zz for c in coef], -1).astype(np.float32)
    f = po.make_field(system_type=4, dom=dom, grd=grd, bgrid=bg.reshape(-1),
                      egrid=np.zeros(n ** 3 * 3, np.float32), interp_corrected=corrected)
    rng = np.random.default_rng(3)
    pts = rng.uniform(0.1, L - dx - 0.1, (200, 3))
    xyzt = np.zeros((len(pts), 4))
    xyzt[:, :3] = pts
    got = po.get_emf(f, xyzt)[:, :3]
    cell = np.floor(pts / dx)
    fr = pts / dx - cell
    if not corrected:
        fr = fr[:, ::-1]  # x and z fractions exchanged
    q = (cell + fr) * dx
    want = np.stack([c[0] + c[1] * q[:, 0] + c[2] * q[:, 1] + c[3] * q[:, 2] for c in coef], 1)
    # the interpolated values are returned in FP32 (src/magnetic_field.c:593-622)
    np.testing.assert_allclose(got, want, rtol=0, atol=1e-6)
    other = (cell + fr[:, ::-1]) * dx  # the other weight convention misses by O(dx)
    miss = np.stack([c[0] + c[1] * other[:, 0] + c[2] * other[:, 1] + c[3] * other[:, 2] for c in coef], 1)
    assert np.abs(got - miss).max() > 1e-2
