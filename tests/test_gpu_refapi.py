"""The reference's tracking entry points (src/tracking.c), called through the C
ABI the way a C caller of the reference calls them, against the library's own
run call (tp_track_host) and the golden runs of the reference build:

- particle_tracking_fixed_time_step (src/tracking.c:90-190): particles, step
  counts and spectra equal the run call's; the diffusion file it writes,
  data/diff_coeffs.dat, holds the run's sums and the reference's remaining
  counts;
- particle_tracking_multi_steps_openmp + gather_particle_spectra_openmp
  (src/tracking.c:297-375, 475-493) with the particles split between two
  thread slots, the way the reference's `omp for` splits them;
- particle_tracking_single_step_openmp (src/tracking.c:376-470) driven step by
  step by the loop of src/tracking.c:313-373, one particle at a time;
- particle_tracking_hybrid (src/tracking.c:659-699), the caller's entry point,
  with the fixed step and with the adaptive stepper, and the spectrum files it
  writes.

Cases from the golden runs: 0 (uniform test field), 3 (PIC grids), 4 (MHD
grids) and 5 (force-free field with open boundaries, 44 particles escape).
"""
import ctypes as C
import json
import math

import numpy as np
import pytest

import make_golden as mg
from oracle import pyoracle as po

pytestmark = pytest.mark.gpu
tp = pytest.importorskip("test_particle_gb300")
import test_particle_gb300.workloads as wl  # noqa: E402

SC = mg.scenarios()
CASES = (0, 3, 4, 5)
DIFF_INTERVAL = 100  # tinterval_dcoeffs, src/tracking.c:17
COMPONENTS = ("x", "y", "z", "ux", "uy", "uz", "t", "xshift", "yshift", "zshift", "qm")

I, D, V = C.c_int, C.c_double, C.c_void_p
PI, PD = C.POINTER(C.c_int), C.POINTER(C.c_double)


def ptr(a):
    return None if a is None else V(a.ctypes.data)


def lib():
    L = tp.lib()
    L.particle_tracking_fixed_time_step.argtypes = [I, I, D, I, I, I, I, D, V, V, V, V, V, V, V, V,
                                                    V, V]
    L.particle_tracking_multi_steps_openmp.argtypes = ([I, D, I, I, I, I, I, I, I, I, D] + [V] * 8
                                                       + [V] + [V] * 8)
    L.particle_tracking_single_step_openmp.argtypes = ([I, I, D, I, I, I, I, I, I, D, V, I, PI, V,
                                                        PI, PI, PI, V, V, V, V] + [PD] * 8)
    L.gather_particle_spectra_openmp.argtypes = [I, I, I, V, V, V, V]
    L.particle_bc.argtypes = [V, PI]
    return L


def setup(case):
    tr = np.load("%s/track.npz" % mg.HERE)
    key = "case%d_" % case
    m = json.loads(str(tr[key + "meta"]))
    s = dict(SC[m["name"]])
    d = po.Domain.from_buffer_copy(s["dom"])
    d.tmax = m["tmax"]
    tp.configure(system_type=s["system_type"], charge_mass=s["charge_mass"], bc_flag=m["bc"],
                 dom=d, grd=s["grd"], mt=s["mt"],
                 abc=s.get("abc", (1.0, np.sqrt(2 / 3.0), np.sqrt(1 / 3.0))),
                 B0=s.get("B0", 1.0), lambda0=s.get("lambda0", 1.0), vgrid_d=s.get("vgrid_d"),
                 vgrid_f=s.get("vgrid_f"), bgrid=s.get("bgrid"), egrid=s.get("egrid"),
                 bgrid_ab=s.get("bgrid_ab", (None, None)), egrid_ab=s.get("egrid_ab", (None, None)),
                 wl=s.get("wl"), ibessel=s.get("ibessel", 0))
    tp.set_spectrum(m["nbins"], m["emin"], m["emax"])
    estep = int(m["tmax"] / m["dt"])  # src/tracking.c:103-104
    m.update(estep=estep, einterval=estep // m["nt_out"], nsdc=estep // DIFF_INTERVAL + 1)
    return tr, key, m


def same_particles(a, b):
    for c in COMPONENTS:
        assert np.array_equal(a[c], b[c]), c


def read_diff_file(path):
    rows = open(path).read().splitlines()
    assert rows[0].split() == ["drr", "dxx", "dyy", "dzz", "dpp", "duu", "daa", "dee", "nptl"]
    vals = np.array([[float(x) for x in r.split()[:8]] for r in rows[1:]])
    nrem = np.array([int(r.split()[8]) for r in rows[1:]])
    return vals.T, nrem


@pytest.mark.parametrize("case", CASES)
def test_fixed_time_step(case, tmp_path, monkeypatch):
    tr, key, m = setup(case)
    p0 = tr[key + "ptl0"]
    n, nb, nt = len(p0), m["nbins"], m["nt_out"]
    run = tp.track(p0, m["dt"], nt, nb, precision=tp.PREC_FP64)
    monkeypatch.chdir(tmp_path)
    (tmp_path / "data").mkdir()
    pi, p = p0.copy(), p0.copy()
    nst = np.zeros(n, np.int32)
    esp, etot, ese = np.zeros(nt * nb), np.zeros(nt * nb), np.zeros(nt * nb)
    lib().particle_tracking_fixed_time_step(0, n, m["dt"], nb, nt, 0, 1, 1.0, None, ptr(pi),
                                            ptr(nst), ptr(p), ptr(esp), ptr(etot), ptr(ese), None,
                                            None, None)
    assert tp.device_status() == 0
    same_particles(p, run["ptl"])
    same_particles(pi, p0)  # the initial state is read only
    assert np.array_equal(nst, run["nsteps"])
    assert np.array_equal(nst, tr[key + "nsteps"])
    assert np.array_equal(esp.reshape(nt, nb), run["espect"])
    # escape spectra are kept only with open boundaries (src/tracking.c:482-487)
    want_ese = run["espect_escape"] if m["bc"] == 1 else np.zeros((nt, nb))
    assert np.array_equal(ese.reshape(nt, nb), want_ese)
    if m["bc"] == 1:
        assert ese.sum() == tr[key + "espect_escape"].sum() > 0
    dsum, nrem = read_diff_file(tmp_path / "data" / "diff_coeffs.dat")
    assert dsum.shape == (8, m["nsdc"])
    assert np.array_equal(nrem, tr[key + "remain"])
    # the file holds 5 significant digits
    np.testing.assert_allclose(dsum, run["dsum"], rtol=6e-5, atol=1e-30)
    np.testing.assert_allclose(dsum[:, 1:6], tr[key + "dsum"][:, 1:6], rtol=1e-4, atol=1e-20)


@pytest.mark.parametrize("case", CASES)
def test_multi_steps_split_over_two_threads(case):
    """src/tracking.c:139-172 with two threads: each multi-step call takes a
    contiguous half of the particles and its own private spectrum row; the
    gather sums the rows."""
    tr, key, m = setup(case)
    p0 = tr[key + "ptl0"]
    n, nb, nt, nsdc = len(p0), m["nbins"], m["nt_out"], m["nsdc"]
    run = tp.track(p0, m["dt"], nt, nb, precision=tp.PREC_FP64)
    L = lib()
    pi, p = p0.copy(), p0.copy()
    nst = np.ones(n, np.int32)  # src/tracking.c:127-129
    remain = np.full(nsdc, n, np.int32)
    d = np.zeros((8, nsdc))
    ep, eep = np.zeros((2, nt * nb)), np.zeros((2, nt * nb))
    half = n // 2
    for tid, (lo, hi) in enumerate(((0, half), (half, n))):
        rec = p0.itemsize * lo
        L.particle_tracking_multi_steps_openmp(
            hi - lo, m["dt"], tid, 1, m["estep"], nb, nt, m["einterval"], 0, 1, 1.0, None,
            V(pi.ctypes.data + rec), None, V(p.ctypes.data + rec), V(nst.ctypes.data + 4 * lo),
            ptr(ep), ptr(eep), None, ptr(remain), *[ptr(d[c]) for c in range(8)])
    assert tp.device_status() == 0
    assert ep[0].sum() > 0 and ep[1].sum() > 0
    esp, ese = np.zeros(nt * nb), np.zeros(nt * nb)
    L.gather_particle_spectra_openmp(2, nb, nt, ptr(esp), ptr(ep), ptr(ese), ptr(eep))
    same_particles(p, run["ptl"])
    assert np.array_equal(nst, run["nsteps"])
    assert np.array_equal(esp.reshape(nt, nb), run["espect"])
    if m["bc"] == 1:
        assert np.array_equal(ese.reshape(nt, nb), run["espect_escape"])
    assert np.array_equal(remain, run["remain"])
    np.testing.assert_allclose(d, run["dsum"], rtol=1e-12, atol=1e-30)


@pytest.mark.parametrize("case", (4, 5))
def test_single_step_loop(case):
    """The per-particle loop of src/tracking.c:313-373 around
    particle_tracking_single_step_openmp, one particle and one step per call."""
    tr, key, m = setup(case)
    p0 = tr[key + "ptl0"]
    n, nb, nt, nsdc = len(p0), m["nbins"], m["nt_out"], m["nsdc"]
    dt, estep, einterval = m["dt"], m["estep"], m["einterval"]
    run = tp.track(p0, dt, nt, nb, precision=tp.PREC_FP64)
    L = lib()
    pi, p = p0.copy(), p0.copy()
    nst = np.ones(n, np.int32)
    remain = np.full(nsdc, n, np.int32)
    d = np.zeros((8, nsdc))
    ep, eep = np.zeros(nt * nb), np.zeros(nt * nb)
    pre, after, ntp, npts = I(), I(), I(), I(1)
    single = [D(0.0) for _ in range(8)]
    refs = [C.byref(s) for s in single]
    pi_p, p_p, nst_p, ep_p, eep_p = ptr(pi), ptr(p), ptr(nst), ptr(ep), ptr(eep)
    step = L.particle_tracking_single_step_openmp
    for i in range(n):
        pre.value = 0
        L.particle_bc(V(p.ctypes.data + p.itemsize * i), C.byref(pre))
        after.value = pre.value
        ntp.value = math.floor(1 / einterval)
        for s in single:  # per-particle diffusion samples start from zero
            s.value = 0.0
        tstep = 1
        if pre.value:
            remain[tstep] -= 1
        for j in range(1, estep + 1):
            single[0].value = single[4].value = single[5].value = 0.0  # drr, dpp, duu
            step(i, j, dt, 0, einterval, 0, nb, nt, 1, 1.0, pi_p, 0, ntp, p_p, pre, after, npts,
                 nst_p, ep_p, eep_p, None, *refs)
            if j % DIFF_INTERVAL == 0:
                for c in range(8):
                    d[c, tstep] += single[c].value
                tstep += 1
            if after.value and j % DIFF_INTERVAL == 0 and tstep < nsdc:
                remain[tstep] -= 1
            pre.value = after.value
    assert tp.device_status() == 0
    same_particles(p, run["ptl"])
    assert np.array_equal(nst, run["nsteps"])
    assert np.array_equal(ep.reshape(nt, nb), run["espect"])
    if m["bc"] == 1:
        assert eep.sum() > 0
        assert np.array_equal(eep.reshape(nt, nb), run["espect_escape"])
    assert np.array_equal(remain, run["remain"])
    np.testing.assert_allclose(d, run["dsum"], rtol=1e-10, atol=1e-30)


def spectrum_file(path, nbins, nt_out):
    rows = open(path).read().splitlines()
    assert len(rows) == nt_out
    vals = np.array([[float(x) for x in r.split()] for r in rows])
    assert vals.shape == (nt_out, nbins)
    return vals


def bin_widths(nbins):
    """The bin widths collect_espectrum divides by (src/diagnostics.c:221-248)."""
    L = tp.lib()
    emin = C.c_double.in_dll(L, "emin").value
    logemin = C.c_double.in_dll(L, "logemin").value
    logde = C.c_double.in_dll(L, "logde").value
    w = np.empty(nbins)
    w[0] = emin
    for i in range(1, nbins):
        w[i] = 10 ** logemin * (10 ** (logde * i) - 10 ** (logde * (i - 1)))
    return w


def hybrid(n, dt, nb, nt, bc, method, pi, nst, p):
    L = lib()
    L.particle_tracking_hybrid.argtypes = [I, I, D, I, I, I, I, D, V, I, I, V, V, V, V]
    L.particle_tracking_hybrid(0, n, dt, nb, nt, bc, 1, 1.0, None, method, 0, ptr(pi), ptr(nst),
                               ptr(p), None)


@pytest.mark.parametrize("case", (0, 5))
def test_tracking_hybrid_fixed_step(case, tmp_path, monkeypatch):
    """src/tracking.c:659-699 with tracking_method 0: the run, then
    data/espectrum.dat (and data/espect_escape.dat with open boundaries) as
    counts per unit energy, and data/diff_coeffs.dat."""
    tr, key, m = setup(case)
    p0 = tr[key + "ptl0"]
    n, nb, nt = len(p0), m["nbins"], m["nt_out"]
    run = tp.track(p0, m["dt"], nt, nb, precision=tp.PREC_FP64)
    monkeypatch.chdir(tmp_path)
    (tmp_path / "data").mkdir()
    pi, p = p0.copy(), p0.copy()
    nst = np.zeros(n, np.int32)
    hybrid(n, m["dt"], nb, nt, m["bc"], 0, pi, nst, p)
    assert tp.device_status() == 0
    same_particles(p, run["ptl"])
    assert np.array_equal(nst, run["nsteps"])
    w = bin_widths(nb)
    got = spectrum_file(tmp_path / "data" / "espectrum.dat", nb, nt)
    np.testing.assert_allclose(got, run["espect"] / w, rtol=6e-5, atol=0)
    assert (tmp_path / "data" / "diff_coeffs.dat").exists()
    esc = tmp_path / "data" / "espect_escape.dat"
    if m["bc"] == 1:
        got = spectrum_file(esc, nb, nt)
        np.testing.assert_allclose(got, run["espect_escape"] / w, rtol=6e-5, atol=0)
        assert got.sum() > 0
    else:
        assert not esc.exists()


def test_tracking_hybrid_adaptive(tmp_path, monkeypatch):
    """tracking_method 1 runs the adaptive Bulirsch-Stoer stepper in the
    wire-loop field (the reference leaves this branch empty,
    src/tracking.c:681-684): the same particles, step counts and spectrum as a
    direct call of the batched stepper with u-form derivatives."""
    s = SC["loop"]
    n, nb, nt, h0, tmax = 512, 50, 4, 1e-6, 0.004
    d = po.Domain.from_buffer_copy(s["dom"])
    d.tmax = tmax
    tp.configure(system_type=tp.SYS_WLCS, charge_mass=s["charge_mass"], bc_flag=2, dom=d,
                 wl=s["wl"], ibessel=0)
    tp.set_spectrum(nb, 1e-3, 1e1)
    y0 = wl.torus_particles(n, 1.0, 0.05, 0.3, 0.1, 0.9, 11)
    gam = 1.0 / np.sqrt(1.0 - (y0[:, 3:] ** 2).sum(axis=1))
    p0 = np.zeros(n, dtype=tp.PARTICLE_DTYPE)
    for k, c in enumerate(("x", "y", "z")):
        p0[c] = y0[:, k]
        p0["u" + c] = gam * y0[:, 3 + k]
    p0["qm"] = s["charge_mass"]
    monkeypatch.chdir(tmp_path)
    (tmp_path / "data").mkdir()
    pi, p = p0.copy(), p0.copy()
    nst = np.zeros(n, np.int32)
    hybrid(n, h0, nb, nt, 2, 1, pi, nst, p)
    assert tp.device_status() == 0
    y = np.stack([p0["x"], p0["y"], p0["z"], p0["ux"], p0["uy"], p0["uz"]], 1).copy()
    t = np.zeros(n)
    steps, st = np.zeros(n, np.int32), np.zeros(n, np.int32)
    esp, dfr = np.zeros(nt * nb), np.zeros(8 * (nt + 1))
    tp.check(tp.lib().tp_bs_run(C.c_int(n), tp._ptr(y), tp._ptr(t), C.c_double(tmax), C.c_int(nt),
                                C.c_int(nb), C.c_double(h0), C.c_double(1e-10), C.c_double(1e-10),
                                C.c_int(8), C.c_int(1), C.c_int(10000000), tp._ptr(steps),
                                tp._ptr(st), tp._ptr(esp), tp._ptr(dfr), None), "bs_run")
    assert (st == 0).all()
    assert np.all(t == tmax) and np.all(p["t"] == tmax)
    for k, c in enumerate(("x", "y", "z", "ux", "uy", "uz")):
        assert np.array_equal(p[c], y[:, k]), c
    assert np.array_equal(nst, steps) and (steps > 0).all()
    got = spectrum_file(tmp_path / "data" / "espectrum.dat", nb, nt)
    np.testing.assert_allclose(got, esp.reshape(nt, nb) / bin_widths(nb), rtol=6e-5, atol=0)
    assert esp.reshape(nt, nb).sum(axis=1).tolist() == [n] * nt
