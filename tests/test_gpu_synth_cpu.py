"""The CPU synthesis of the gridded workload field (the oracle's
or_synth_pic_fields, which the reference arm of the benchmark uses so that it
runs no GPU code) against the library's GPU synthesis (synth.cu) of the same
seeded modes.  The two form each node's cosine differently (a product of
per-axis unit complex numbers against the cosine of the summed exact phase),
so a double result can differ in its last bits and, rarely, round to the
neighbouring float: every value is within one FP32 ulp (or, for values near
zero, whose FP32 ulp is below the double sums' rounding, within 1e-15 of the
largest value) and almost all are identical."""
import numpy as np
import pytest

from oracle import pyoracle as po

pytestmark = pytest.mark.gpu
tp = pytest.importorskip("test_particle_gb300")
import test_particle_gb300.workloads as wl  # noqa: E402


@pytest.mark.parametrize("n,nmodes,kmax", [(48, 512, 64), (33, 64, 8)])
def test_cpu_synthesis_matches_gpu(n, nmodes, kmax):
    cfg = wl.config_grid(nptl=1, steps=1, n=n)
    dom = tp.Domain()
    dom.xmax = dom.ymax = dom.zmax = cfg["hi"][0]
    grd = tp.Grids()
    grd.nx = grd.ny = grd.nz = n
    grd.nt = 1
    grd.dx = grd.dy = grd.dz = cfg["dx"]
    tp.configure(system_type=tp.SYS_PIC, dom=dom, grd=grd)
    mb = wl.kolmogorov_modes(nmodes, 1, kmax, 0.5, cfg["seed"])
    mv = wl.kolmogorov_modes(nmodes, 1, kmax, 0.1, cfg["seed"] + 1000)
    try:
        ge, gb = tp.synth_pic_fields(mb, mv, 1.0, to_host=True)
    finally:
        tp.release_device_fields()
    ce, cb = po.synth_pic_fields(mb, mv, 1.0, n, n, n)
    for g, c in ((ge, ce), (gb, cb)):
        ulp = np.spacing(np.maximum(np.abs(g), np.abs(c)).astype(np.float32))
        allowed = np.maximum(ulp, 1e-15 * np.abs(g).max())
        assert np.all(np.abs(g - c) <= allowed), np.max(np.abs(g - c) / allowed)
        assert np.mean(g != c) <= 1e-4, np.mean(g != c)
