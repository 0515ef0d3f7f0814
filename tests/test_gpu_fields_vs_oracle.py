"""The field evaluations of both GPU paths against the FP64 oracle at points.

The turbulent plane-wave mode sum has no reference counterpart; its FP64
definition is the oracle's or_mode_sum (oracle/tp_oracle.c), and these tests
pin the GPU to it: the FP64 path (fields_fp64.cuh) within 1e-13, the
mixed path's FP32 sum (tp_mixed.cuh) within the error budget of its FP32
arithmetic, stated below.  The mixed path's gridded and ABC fields are checked
against the oracle's FP64 evaluation of the same inputs in the same way.

FP32 error budget of one plane wave, cos(2 pi n.x + phi) evaluated from the
top 32 bits of a 64-bit fixed-point position with __cosf:
  position quantised to 2^-32 of the box    |n| 2 pi 2^-32  <= 9.4e-8 rad (|n| <= 64)
  phase turned to an FP32 angle in [-pi, pi)  pi 2^-24       =  1.9e-7 rad
  __cosf on [-pi, pi]                         2^-21.41       =  3.6e-7
so |dc| <= 6.5e-7 per mode; with FP32 amplitudes (2^-24 relative) and an
FP32 running sum of M terms (at most M 2^-24 of the sum of |terms| in the
worst case), a component's error is at most
  (6.5e-7 + (M + 1) 2^-24) * sum_m |a_m|,
the bound asserted for every point.  Typical errors are random-walk sized,
far below it; the RMS error is asserted against 2e-6 of the RMS field.
"""
import numpy as np
import pytest

from oracle import pyoracle as po

pytestmark = pytest.mark.gpu
tp = pytest.importorskip("test_particle_gb300")
import test_particle_gb300.workloads as wl  # noqa: E402

EPS32 = 2.0 ** -24


def _points(n, seed, lo=-1.0, hi=2.0):
    """Points in the box and in its periodic images (lo..hi box lengths)."""
    rng = np.random.default_rng(seed)
    xyzt = np.zeros((n, 4))
    xyzt[:, :3] = rng.uniform(lo, hi, (n, 3))
    xyzt[: n // 2, :3] = rng.uniform(0.0, 1.0, (n // 2, 3))
    return xyzt


def _modesum_setup(nmodes=512, kmax=64, seed=13):
    """The analytic turbulence workload's table: 512 modes, |n| in [1, 64],
    dB/B0 = 1, B0 = 1 along z, E = -v_A k^ x dB with v_A = 0.1."""
    cfg = wl.config_modesum(nptl=1, steps=1)
    modes = wl.kolmogorov_modes(nmodes, cfg["kmin"], kmax, cfg["dB"], seed, va=cfg["va"])
    dom = tp.Domain()
    dom.xmax = dom.ymax = dom.zmax = 1.0
    tp.configure(system_type=tp.SYS_MODESUM, dom=dom, modes=modes, mode_B0=cfg["B0"])
    f = po.make_field(system_type=tp.SYS_MODESUM, dom=po.Domain.from_buffer_copy(dom), modes=modes,
                      B0=cfg["B0"])
    return modes, f


@pytest.mark.parametrize("nmodes,kmax", [(512, 64), (64, 8), (1, 1)])
def test_modesum_fp64_matches_oracle(nmodes, kmax):
    modes, f = _modesum_setup(nmodes, kmax)
    xyzt = _points(10000, 1)
    gpu = tp.get_emf(xyzt)
    ref = po.get_emf(f, xyzt)
    scale = np.abs(ref).max(axis=0)
    err = np.abs(gpu - ref)
    assert np.all(err <= 1e-13 * np.maximum(np.abs(ref), scale)), err.max(axis=0)
    assert tp.device_status() == 0


def test_modesum_fp64_is_periodic_and_has_the_stated_rms():
    """Shifting a point by whole box lengths leaves the field unchanged (the
    phases are exact in 64-bit fixed point), and the fluctuation has rms
    dB/B0 = 1 (sum of a^2 / 2 over modes = 1)."""
    modes, f = _modesum_setup()
    xyzt = _points(4096, 2, 0.0, 1.0)
    xyzt[:, :3] = np.floor(xyzt[:, :3] * 2.0 ** 30) / 2.0 ** 30  # dyadic: whole shifts are exact
    a = tp.get_emf(xyzt)
    sh = xyzt.copy()
    sh[:, :3] += np.array([3.0, -2.0, 5.0])
    b = tp.get_emf(sh)
    assert np.array_equal(a, b)
    assert abs(0.5 * np.sum(modes["amp_b"] ** 2) - 1.0) < 1e-12
    db = a[:, :3] - [0.0, 0.0, 1.0]
    assert 0.8 < np.sqrt(np.mean(np.sum(db ** 2, axis=1))) < 1.2


def _fp32_budget(amp, nterms, maxn):
    dc = maxn * 2 * np.pi * 2.0 ** -32 + np.pi * EPS32 + 2.0 ** -21.41
    return (dc + (nterms + 1) * EPS32) * np.abs(amp).sum(axis=0)


@pytest.mark.parametrize("nmodes,kmax", [(512, 64), (64, 8)])
def test_modesum_mixed_fp32_within_budget(nmodes, kmax):
    modes, f = _modesum_setup(nmodes, kmax)
    xyzt = _points(10000, 3)
    gpu = tp.get_emf_mixed(xyzt[:, :3]).astype(np.float64)
    ref = po.get_emf(f, xyzt)
    maxn = np.abs(modes["n"]).sum(axis=1).max()  # |n_x| + |n_y| + |n_z| bounds n . x per box
    amp = np.concatenate([modes["amp_b"], modes["amp_e"]], axis=1)
    bound = _fp32_budget(amp, nmodes, maxn)
    bound[2] += EPS32 * 1.0  # B0 added in FP32
    err = np.abs(gpu - ref)
    assert np.all(err <= bound), (err.max(axis=0), bound)
    rms_err = np.sqrt(np.mean(err ** 2, axis=0))
    rms_fld = np.sqrt(np.mean((ref - ref.mean(axis=0)) ** 2, axis=0))
    assert np.all(rms_err <= 2e-6 * rms_fld), rms_err / rms_fld


def test_pic_mixed_fp32_matches_oracle():
    """Trilinear interpolation of the node-interleaved FP32 grid (the mixed
    path) against the oracle's FP64 interpolation of the same FP32 grid, with
    the reference's weights: the FP32 weights come from a 32-bit fixed-point
    fraction, so each corner weight is within a few 2^-24 of the FP64 one and
    the result within 16 2^-24 of the sum of |corner values|."""
    n, dx = 24, 0.25
    L = (n - 1) * dx
    dom = tp.Domain()
    dom.xmax = dom.ymax = dom.zmax = L
    grd = tp.Grids()
    grd.nx = grd.ny = grd.nz = n
    grd.nt = 1
    grd.dx = grd.dy = grd.dz = dx
    tp.configure(system_type=tp.SYS_PIC, dom=dom, grd=grd)
    mb = wl.kolmogorov_modes(64, 1, 6, 0.5, 31)
    mv = wl.kolmogorov_modes(64, 1, 6, 0.1, 32)
    he, hb = tp.synth_pic_fields(mb, mv, 1.0, to_host=True)
    try:
        xyzt = _points(20000, 4, 0.0, 1.0)
        xyzt[:, :3] *= L
        gpu = tp.get_emf_mixed(xyzt[:, :3]).astype(np.float64)
    finally:
        tp.release_device_fields()
    f = po.make_field(system_type=4, dom=po.Domain.from_buffer_copy(dom),
                      grd=po.Grids.from_buffer_copy(grd), egrid=he, bgrid=hb)
    ref = po.get_emf(f, xyzt)
    cmax = np.concatenate([np.abs(hb).max(axis=0), np.abs(he).max(axis=0)])
    err = np.abs(gpu - ref)
    assert np.all(err <= 16 * EPS32 * 8 * cmax), (err.max(axis=0), cmax)
    assert tp.device_status() == 0


def test_abc_mixed_fp32_matches_oracle():
    """ABC field A = B = C = 1, lambda = 2 pi on the unit box: exact 32-bit
    phases, three __sincosf per point (|error| <= 2^-21.41 each), FP32 sums."""
    dom = tp.Domain()
    dom.xmax = dom.ymax = dom.zmax = 1.0
    tp.configure(system_type=tp.SYS_FORCEFREE, dom=dom, abc=(1.0, 1.0, 1.0), B0=1.0,
                 lambda0=2 * np.pi)
    f = po.make_field(system_type=2, dom=po.Domain.from_buffer_copy(dom), abc=(1.0, 1.0, 1.0),
                      B0=1.0, lambda0=2 * np.pi)
    xyzt = _points(20000, 5)
    gpu = tp.get_emf_mixed(xyzt[:, :3]).astype(np.float64)
    ref = po.get_emf(f, xyzt)
    dc = 2 * np.pi * 2.0 ** -32 + np.pi * EPS32 + 2.0 ** -21.41
    err = np.abs(gpu - ref)
    assert np.all(err[:, :3] <= 2 * (dc + 3 * EPS32)), err.max(axis=0)
    assert np.all(err[:, 3:] == 0.0)
