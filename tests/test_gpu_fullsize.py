"""The headline workload at its full size (512^3 gridded E, B = 4.3 GB
interleaved, 1,048,576 particles) over a short horizon, checked through
properties that do not depend on the size: every particle is pushed every
step, every spectrum frame counts every particle, positions stay in the box
with whole periods in the shifts, no kernel raises a status bit, and the
mixed path follows the FP64 path particle by particle before chaos has had
time to amplify FP32 rounding.  At this size node offsets exceed 2^31 bytes,
which is what the small parity cases cannot exercise."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
tp = pytest.importorskip("test_particle_gb300")
import test_particle_gb300.workloads as wl  # noqa: E402


def test_headline_size_short_horizon():
    steps = 50
    cfg = wl.config_grid(steps=steps)  # 512^3, 1,048,576 particles
    n, L = cfg["n"], cfg["hi"][0]
    dom = tp.Domain()
    dom.xmin, dom.ymin, dom.zmin = cfg["lo"]
    dom.xmax, dom.ymax, dom.zmax = cfg["hi"]
    dom.xmin_ptl, dom.ymin_ptl, dom.zmin_ptl = cfg["lo"]
    dom.xmax_ptl, dom.ymax_ptl, dom.zmax_ptl = cfg["hi"]
    dom.tmax = steps * cfg["dt"] + 0.5 * cfg["dt"]
    grd = tp.Grids()
    grd.nx = grd.ny = grd.nz = n
    grd.nt = 1
    grd.dx = grd.dy = grd.dz = cfg["dx"]
    tp.configure(system_type=tp.SYS_PIC, charge_mass=1.0, bc_flag=0, dom=dom, grd=grd, mt=0)
    mb = wl.kolmogorov_modes(cfg["nmodes"], cfg["kmin"], cfg["kmax"], cfg["dB"], cfg["seed"])
    mv = wl.kolmogorov_modes(cfg["nmodes"], cfg["kmin"], cfg["kmax"], cfg["v_rms"], cfg["seed"] + 1000)
    tp.synth_pic_fields(mb, mv, 1.0)
    tp.set_spectrum(cfg["nbins"], cfg["emin"], cfg["emax"])
    p0 = wl.shell_particles(cfg["nptl"], cfg["speed"], cfg["lo"], cfg["hi"], cfg["seed"])
    nt_out = 5
    try:
        mix = tp.track(p0, cfg["dt"], nt_out, cfg["nbins"], precision=tp.PREC_MIXED)
        assert tp.device_status() == 0
        ref = tp.track(p0, cfg["dt"], nt_out, cfg["nbins"], precision=tp.PREC_FP64)
        assert tp.device_status() == 0
    finally:
        tp.release_device_fields()
    N = cfg["nptl"]
    for r in (mix, ref):
        assert r["estep"] == steps
        assert np.all(r["nsteps"] == steps + 1)
        assert np.all(r["espect"].sum(axis=1) == N)
        assert r["espect_escape"].sum() == 0  # periodic box: nobody leaves
        p = r["ptl"]
        for c in ("x", "y", "z"):
            assert np.all((p[c] >= 0) & (p[c] <= L))
            per = p[c + "shift"] / L
            assert np.all(np.abs(per - np.round(per)) < 1e-9)
    # particle by particle: displacement error relative to the displacement
    for c in ("x", "y", "z"):
        a = mix["ptl"][c] + mix["ptl"][c + "shift"]
        b = ref["ptl"][c] + ref["ptl"][c + "shift"]
        disp = np.abs(b - p0[c]) + 1e-3 * cfg["dx"]
        rel = np.abs(a - b) / disp
        assert np.median(rel) < 1e-4, (c, np.median(rel))
        assert np.quantile(rel, 0.99) < 1e-2, (c, np.quantile(rel, 0.99))
    gm = np.sqrt(1 + mix["ptl"]["ux"] ** 2 + mix["ptl"]["uy"] ** 2 + mix["ptl"]["uz"] ** 2)
    gr = np.sqrt(1 + ref["ptl"]["ux"] ** 2 + ref["ptl"]["uy"] ** 2 + ref["ptl"]["uz"] ** 2)
    assert np.median(np.abs(gm / gr - 1)) < 1e-5
