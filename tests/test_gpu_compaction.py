"""Open boundaries (bc_flag 1) in segments with the departed particles
compacted away (tp_set_compaction): the same particles, step counts,
spectra and remaining counts as one launch over the whole run, diffusion sums
equal to rounding (their summation order changes), in the FP64 parity path
and in the mixed path."""
import json

import numpy as np
import pytest

import make_golden as mg
from oracle import pyoracle as po

pytestmark = pytest.mark.gpu
tp = pytest.importorskip("test_particle_gb300")
import test_particle_gb300.workloads as wl  # noqa: E402

SC = mg.scenarios()
COMPONENTS = ("x", "y", "z", "ux", "uy", "uz", "t", "xshift", "yshift", "zshift", "qm")


@pytest.fixture(autouse=True)
def _restore_default():
    yield
    tp.set_compaction(-1)


def run(p0, dt, nt_out, nbins, precision, seg):
    tp.set_compaction(seg)
    r = tp.track(p0, dt, nt_out, nbins, precision=precision)
    assert tp.device_status() == 0
    return r


def same(a, b):
    for c in COMPONENTS:
        assert np.array_equal(a["ptl"][c], b["ptl"][c]), c
    for k in ("nsteps", "espect", "espect_escape", "remain"):
        assert np.array_equal(a[k], b[k]), k
    np.testing.assert_allclose(a["dsum"], b["dsum"], rtol=1e-12, atol=1e-300)


@pytest.mark.parametrize("seg", [100, 300, 1900])
def test_fp64_open_boundary_segments(seg):
    """The golden open-boundary run (force-free field with a velocity grid,
    48 particles, 2000 steps, 44 leave the box)."""
    tr = np.load("%s/track.npz" % mg.HERE)
    m = json.loads(str(tr["case5_meta"]))
    s = dict(SC[m["name"]])
    d = po.Domain.from_buffer_copy(s["dom"])
    d.tmax = m["tmax"]
    tp.configure(system_type=s["system_type"], charge_mass=s["charge_mass"], bc_flag=1, dom=d,
                 grd=s["grd"], mt=s["mt"],
                 abc=s.get("abc", (1.0, np.sqrt(2 / 3.0), np.sqrt(1 / 3.0))),
                 B0=s.get("B0", 1.0), lambda0=s.get("lambda0", 1.0), vgrid_d=s.get("vgrid_d"),
                 vgrid_f=s.get("vgrid_f"), bgrid=s.get("bgrid"), egrid=s.get("egrid"),
                 bgrid_ab=s.get("bgrid_ab", (None, None)), egrid_ab=s.get("egrid_ab", (None, None)),
                 wl=s.get("wl"), ibessel=s.get("ibessel", 0))
    tp.set_spectrum(m["nbins"], m["emin"], m["emax"])
    p0 = tr["case5_ptl0"]
    one = run(p0, m["dt"], m["nt_out"], m["nbins"], tp.PREC_FP64, 0)
    cut = run(p0, m["dt"], m["nt_out"], m["nbins"], tp.PREC_FP64, seg)
    assert one["info"].launches == 3
    assert cut["info"].launches > 3  # more than one segment ran
    same(cut, one)
    # and both are the reference's run
    assert np.array_equal(cut["nsteps"], tr["case5_nsteps"])
    assert np.array_equal(cut["remain"], tr["case5_remain"])
    assert cut["espect_escape"].sum() == tr["case5_espect_escape"].sum()


def _open_pic(n=4096, steps=600, ng=40):
    cfg = wl.config_grid(nptl=n, steps=steps, n=ng, dx=0.25)
    L = cfg["hi"][0]
    dom = tp.Domain()
    dom.xmax = dom.ymax = dom.zmax = L
    dom.xmax_ptl = dom.ymax_ptl = dom.zmax_ptl = L
    dom.tmax = steps * cfg["dt"] + 0.5 * cfg["dt"]
    grd = tp.Grids()
    grd.nx = grd.ny = grd.nz = ng
    grd.nt = 1
    grd.dx = grd.dy = grd.dz = 0.25
    tp.configure(system_type=tp.SYS_PIC, dom=dom, grd=grd, bc_flag=1)
    mb = wl.kolmogorov_modes(64, 1, 8, 0.5, 21)
    mv = wl.kolmogorov_modes(64, 1, 8, 0.1, 22)
    tp.synth_pic_fields(mb, mv, 1.0)
    tp.set_spectrum(200, 1e-3, 1e2)
    return cfg, wl.shell_particles(n, 0.7, cfg["lo"], cfg["hi"], 21)


@pytest.mark.parametrize("precision", ["fp64", "fp64fast", "mixed"])
def test_open_box_segments(precision):
    """Gridded field in a 10^3 open box: most particles leave within the run;
    every precision that segments resumes exactly where it stopped."""
    code = {"fp64": tp.PREC_FP64, "fp64fast": tp.PREC_FP64_FAST, "mixed": tp.PREC_MIXED}[precision]
    cfg, p0 = _open_pic()
    try:
        one = run(p0, cfg["dt"], 3, 200, code, 0)
        cut = run(p0, cfg["dt"], 3, 200, code, 100)
    finally:
        tp.release_device_fields()
    assert cut["info"].launches > 3
    same(cut, one)
    left = one["espect_escape"].sum()
    assert 0.2 * len(p0) < left < len(p0)
    # departures counted at the diffusion steps up to step 500
    assert len(p0) - left <= one["remain"][-1] < len(p0)


def test_every_particle_leaves():
    """Uniform field along z, open unit box, every particle drifting out
    through the z faces within about 400 of 800 steps: the segments stop once
    the box is empty, and the later diffusion rows and remaining counts come
    from the closed form alone."""
    rng = np.random.default_rng(8)
    n, dt, steps = 3000, 0.005, 800
    dom = tp.Domain()
    dom.xmax = dom.ymax = dom.zmax = 1.0
    dom.xmax_ptl = dom.ymax_ptl = dom.zmax_ptl = 1.0
    dom.tmax = steps * dt + 0.5 * dt
    tp.configure(system_type=tp.SYS_TEST, charge_mass=1.0, bc_flag=1, dom=dom)
    tp.set_spectrum(100, 1e-3, 1e1)
    p0 = np.zeros(n, dtype=tp.PARTICLE_DTYPE)
    p0["x"], p0["y"], p0["z"] = rng.uniform(0.3, 0.7, n), rng.uniform(0.3, 0.7, n), rng.uniform(0.0, 1.0, n)
    uz = rng.uniform(0.6, 1.5, n) * np.where(rng.random(n) < 0.5, -1.0, 1.0)
    p0["ux"], p0["uy"], p0["uz"] = 0.05 * rng.standard_normal(n), 0.05 * rng.standard_normal(n), uz
    p0["qm"] = 1.0
    for prec in (tp.PREC_FP64, tp.PREC_MIXED):
        one = run(p0, dt, 4, 100, prec, 0)
        cut = run(p0, dt, 4, 100, prec, 100)
        same(cut, one)
        assert one["espect_escape"].sum() == n  # everybody left
        assert one["remain"][-1] == 0 and one["espect"][-1].sum() == 0
        # 8 segments would take 8 + 7 x 3 + 2 = 31 launches; the box empties in the 4th
        assert 3 < cut["info"].launches < 31


@pytest.mark.parametrize("seg", [2 ** 31 - 1, 2 ** 31 - 100])
def test_segment_length_near_int_max_runs_one_launch(seg):
    """A segment length near INT_MAX must not wrap when it is rounded up to
    the 100-step diffusion interval: the run takes one tracking launch, the
    same launches as with compaction off."""
    cfg, p0 = _open_pic(n=1024, steps=300)
    try:
        one = run(p0, cfg["dt"], 3, 200, tp.PREC_MIXED, 0)
        big = run(p0, cfg["dt"], 3, 200, tp.PREC_MIXED, seg)
    finally:
        tp.release_device_fields()
    assert big["info"].launches == one["info"].launches
    same(big, one)
