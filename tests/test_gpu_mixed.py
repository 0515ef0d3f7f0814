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


def _l1_frames(a, b, n):
    """L1 distance of two spectra per output frame, each normalised by n."""
    return np.abs(a / n - b / n).sum(axis=1)


def sigma_l1(n):
    """Standard deviation of the L1 distance of two independent n-particle
    histograms (normal approximation of Poisson bin counts: each bin adds
    |X - Y| with variance 2 lambda (1 - 2/pi), and the lambdas sum to n)."""
    return np.sqrt(2.0 * (1.0 - 2.0 / np.pi) / n)


def fp32_rounded(p0):
    p = p0.copy()
    for c in ("x", "y", "z", "ux", "uy", "uz"):
        p[c] = p[c].astype(np.float32).astype(np.float64)
    return p


def sampling_floor(frames):
    """Per frame, the expected L1 distance of two independent ensembles of
    this size drawn from the spectrum: sum over bins of sqrt(4 p (1-p) / (pi N))."""
    out = []
    for fb in frames:
        nb = fb.sum()
        q = fb / nb
        out.append(np.sqrt(4 * q * (1 - q) / (np.pi * nb)).sum())
    return np.array(out)


@pytest.mark.parametrize("kind", ["abc", "grid", "modesum"])
def test_mixed_long_horizon_statistics(kind):
    """Ensemble statistics over 2000 steps, 65,536 particles, against the FP64
    path from the same initial state.

    Spectra, per output frame: the mixed path's L1 distance to FP64 must stay
    within max(1.5 x the chaos floor, the sampling floor) + 3 sigma.  The chaos
    floor is the distance of the FP64 run started from the initial state
    rounded to FP32 (the mixed path keeps momenta in FP32); the mixed path,
    which rounds at every step rather than once, decorrelates from FP64 about
    one frame sooner, after which both sit at the sampling floor, the distance
    of two independent ensembles of this size from the same distribution.  A
    bias of the mixed path larger than that sampling noise fails the test.

    Diffusion coefficients, per coefficient, largest relative error over the
    rows: within max(1 %, 2 x the chaos floor's, 4 sigma), sigma = 2 / sqrt(N),
    the relative standard deviation of the difference of two independent
    ensemble means of squared Gaussian displacements (each sqrt(2 / N))."""
    n = 65536
    cfg, p0 = setup(kind, 2000, n=n)
    a = tp.track(p0, cfg["dt"], 4, 200, precision=tp.PREC_FP64)
    r = tp.track(fp32_rounded(p0), cfg["dt"], 4, 200, precision=tp.PREC_FP64)
    b = tp.track(p0, cfg["dt"], 4, 200, precision=tp.PREC_MIXED)
    assert b["espect"].sum() == a["espect"].sum() == 4 * n
    l1_mixed = _l1_frames(b["espect"], a["espect"], n)
    l1_chaos = _l1_frames(r["espect"], a["espect"], n)
    floor = sampling_floor(a["espect"])
    bound = np.maximum(1.5 * l1_chaos, floor) + 3 * sigma_l1(n)
    print("%s L1 mixed %s chaos %s sampling %s" % (kind, l1_mixed, l1_chaos, floor))
    assert np.all(l1_mixed <= bound), (l1_mixed, bound)
    ref = a["dsum"][:, 1:]
    scale = np.abs(ref).max(axis=1)
    live = scale > 1e-12 * np.abs(ref).max()  # dee with E = 0 is rounding noise in every path
    sig = 2.0 / np.sqrt(n)
    for c in np.nonzero(live)[0]:
        den = np.maximum(np.abs(ref[c]), 1e-300)
        em = np.max(np.abs(b["dsum"][c, 1:] - ref[c]) / den)
        ef = np.max(np.abs(r["dsum"][c, 1:] - ref[c]) / den)
        print("%s diffusion row %d: mixed %.3e chaos %.3e" % (kind, c, em, ef))
        assert np.isfinite(em) and em <= max(0.01, 2.0 * ef, 4 * sig), (c, em, ef)
    assert tp.device_status() == 0


def test_fp64_fast_matches_parity_short():
    cfg, p0 = setup("grid", 100)
    a = tp.track(p0, cfg["dt"], 1, 200, precision=tp.PREC_FP64)
    b = tp.track(p0, cfg["dt"], 1, 200, precision=tp.PREC_FP64_FAST)
    for k in ("x", "y", "z", "ux", "uy", "uz"):
        assert np.max(np.abs(a["ptl"][k] - b["ptl"][k])) < 1e-9
