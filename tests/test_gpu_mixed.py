"""Mixed-precision path (FP32 push and field, 64-bit fixed-point positions)
against the FP64 parity path on the same inputs.  Trajectories are chaotic,
so the comparison is per particle over a short horizon (before FP32 rounding
has grown) and statistical over a long one."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
tp = pytest.importorskip("test_particle_gb300")
import test_particle_gb300.workloads as wl  # noqa: E402


def setup(kind, steps, n=8192, seed=5):
    dom = tp.Domain()
    if kind == "abc":
        cfg = wl.config_abc(nptl=n, steps=steps)
        dom.xmax = dom.ymax = dom.zmax = 1.0
        dom.tmax = steps * cfg["dt"] + 0.5 * cfg["dt"]
        tp.configure(system_type=tp.SYS_FORCEFREE, dom=dom, abc=(1.0, 1.0, 1.0), B0=1.0,
                     lambda0=2 * np.pi)
    elif kind == "grid":
        cfg = wl.config_grid(nptl=n, steps=steps, n=48, dx=0.25)
        L = cfg["hi"][0]
        dom.xmax = dom.ymax = dom.zmax = L
        dom.tmax = steps * cfg["dt"] + 0.5 * cfg["dt"]
        grd = tp.Grids()
        grd.nx = grd.ny = grd.nz = 48
        grd.dx = grd.dy = grd.dz = 0.25
        tp.configure(system_type=tp.SYS_PIC, dom=dom, grd=grd)
        mb = wl.kolmogorov_modes(64, 1, 8, 0.5, seed)
        mv = wl.kolmogorov_modes(64, 1, 8, 0.1, seed + 1)
        tp.synth_pic_fields(mb, mv, 1.0)
    else:
        cfg = wl.config_modesum(nptl=n, steps=steps)
        dom.xmax = dom.ymax = dom.zmax = 1.0
        dom.tmax = steps * cfg["dt"] + 0.5 * cfg["dt"]
        # 512 modes: the mode table alone takes 20 KB of shared memory
        nm, kmax = (512, 64) if kind == "modesum512" else (128, 16)
        modes = wl.kolmogorov_modes(nm, 1, kmax, 1.0, seed, va=0.1)
        tp.configure(system_type=tp.SYS_MODESUM, dom=dom, modes=modes, mode_B0=1.0)
    tp.set_spectrum(200, 1e-3, 1e2)
    p0 = wl.shell_particles(n, 0.7, cfg["lo"], cfg["hi"], seed)
    return cfg, p0


@pytest.mark.parametrize("kind,steps,tol", [(k, s, t) for k in ("abc", "grid", "modesum")
                                            for s, t in ((1, 1e-5), (10, 1e-4))] +
                         [("modesum512", 1, 1e-5)])
def test_mixed_short_horizon_per_particle(kind, steps, tol):
    """Before chaos amplifies FP32 rounding (the mode-sum field decorrelates
    within a few tens of steps) each particle follows the FP64 path."""
    cfg, p0 = setup(kind, steps)
    a = tp.track(p0, cfg["dt"], 1, 200, precision=tp.PREC_FP64)
    b = tp.track(p0, cfg["dt"], 1, 200, precision=tp.PREC_MIXED)
    L = np.array(cfg["hi"]) - np.array(cfg["lo"])
    u_a = np.sqrt(a["ptl"]["ux"] ** 2 + a["ptl"]["uy"] ** 2 + a["ptl"]["uz"] ** 2)
    for k, ax in (("x", 0), ("y", 1), ("z", 2)):
        pa = a["ptl"][k] + a["ptl"][k + "shift"]
        pb = b["ptl"][k] + b["ptl"][k + "shift"]
        disp = np.abs(pa - p0[k]) + 1e-3 * L[ax]
        assert np.median(np.abs(pa - pb) / disp) < tol, k
        uk = "u" + k
        assert np.median(np.abs(a["ptl"][uk] - b["ptl"][uk]) / u_a) < tol, uk
    assert np.array_equal(a["ptl"]["t"], p0["t"] + steps * cfg["dt"]) or \
        np.allclose(b["ptl"]["t"], a["ptl"]["t"], rtol=1e-14)
    assert tp.device_status() == 0


@pytest.mark.parametrize("kind", ["abc", "grid", "modesum"])
def test_mixed_long_horizon_statistics(kind):
    cfg, p0 = setup(kind, 2000)
    a = tp.track(p0, cfg["dt"], 4, 200, precision=tp.PREC_FP64)
    b = tp.track(p0, cfg["dt"], 4, 200, precision=tp.PREC_MIXED)
    n = len(p0)
    sa, sb = a["espect"] / n, b["espect"] / n
    assert abs(sa.sum() - sb.sum()) < 1e-12
    l1 = np.abs(sa - sb).sum(axis=1)
    # statistical noise floor of two decorrelated ensembles of n particles
    assert np.all(l1 < 0.15), l1
    scale = np.abs(a["dsum"][:, 1:]).max(axis=1, keepdims=True)
    live = scale[:, 0] > 1e-12  # rows that are not rounding noise (dee with E = 0)
    rel = np.abs(b["dsum"][live, 1:] - a["dsum"][live, 1:]) / scale[live]
    assert np.median(rel) < 0.1
    assert tp.device_status() == 0


def test_fp64_fast_matches_parity_short():
    cfg, p0 = setup("grid", 100)
    a = tp.track(p0, cfg["dt"], 1, 200, precision=tp.PREC_FP64)
    b = tp.track(p0, cfg["dt"], 1, 200, precision=tp.PREC_FP64_FAST)
    for k in ("x", "y", "z", "ux", "uy", "uz"):
        assert np.max(np.abs(a["ptl"][k] - b["ptl"][k])) < 1e-9
