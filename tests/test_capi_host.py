"""C ABI without a GPU: the library builds, loads and exports every function
include/tp_gpu.h declares; host-only logic (exact bin edges, init.dat parsers,
scalar helpers) runs without touching CUDA."""
import ctypes as C
import os
import re

import numpy as np
import pytest

import make_golden as mg

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    from test_particle_gb300 import build
    build.build()
    import test_particle_gb300 as tp
    return tp.lib()


def declared_functions():
    names = []
    for fn in sorted(os.listdir(os.path.join(ROOT, "include"))):
        if not fn.endswith(".h"):
            continue
        src = open(os.path.join(ROOT, "include", fn)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"^[A-Za-z_][\w \*]*?\b([a-z_][a-z0-9_]*)\s*\(", src, flags=re.M):
            if not src[m.start():].lstrip().startswith(("typedef", "#")):
                names.append(m.group(1))
    return sorted(set(names))


def test_exports_every_declared_function(lib):
    names = declared_functions()
    assert len(names) > 60
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_exports_reference_globals(lib):
    for name in ("simul_grid", "simul_domain", "system_type", "multi_tframe", "bc_flag",
                 "charge_mass", "param", "config", "nwlcs", "iBessel", "magc_float",
                 "efc_float", "vc_double", "emin", "logemin", "logde"):
        C.c_int.in_dll(lib, name)


def test_bin_edges_reproduce_reference_bins(lib):
    """Bins from the host-derived edges equal the reference's glibc formula."""
    import test_particle_gb300 as tp
    eb = np.load(os.path.join(mg.HERE, "ebins.npz"))
    nb = int(eb["nbins"])
    tp.set_spectrum(nb, float(eb["emin"]), float(eb["emax"]))
    thr = tp.energy_thresholds(nb)
    assert np.all(np.diff(thr) > 0)
    p = eb["ptl"]
    e = np.sqrt(1.0 + p["ux"] ** 2 + p["uy"] ** 2 + p["uz"] ** 2) - 1.0
    bins = np.searchsorted(thr, e, side="right")
    bins[~np.isfinite(e)] = 0
    assert np.array_equal(bins, eb["bins"])


def test_bin_edges_are_tight(lib):
    """Each edge is the smallest double of its bin under the reference formula."""
    import test_particle_gb300 as tp
    from oracle import pyoracle as po
    for nb, e0, e1 in ((50, 1e-4, 10.0), (200, 1e-3, 1e2), (162, 1e-5, 1e3)):
        tp.set_spectrum(nb, e0, e1)
        thr = tp.energy_thresholds(nb)
        s = po.spectrum(nb, e0, e1)
        ob = po.oracle().or_energy_bin_e
        for b, t in enumerate(thr, start=1):
            assert ob(C.byref(s), C.c_double(t)) >= b
            assert ob(C.byref(s), C.c_double(np.nextafter(t, 0))) < b


def test_parsers(lib, tmp_path):
    init = tmp_path / "init.dat"
    init.write_text(
        "--------------------------------- System info --------------------------------\n"
        "0: test, 1: wlcs, 2: forcefree 3: MHD+test particle 4: PIC fields+test particle\n"
        "Flag for the system to use: 1\n"
        "Number of WLCSs: 2\n"
        "Configuration file name: %s\n"
        "------------------------------ Force-free field ------------------------------\n"
        "Normalized B(Gauss): 2.5\n"
        "1/Length scale (lambda): 6.25\n"
        "------------------------------ Particle tracking -----------------------------\n"
        "Total tracking time (s): 100.0\n"
        "0 for fixed step, 1 for adaptive\n"
        "Tracking method to use: 0\n"
        "Tracking time step (for electrons): 1E-2\n" % (tmp_path / "wl.dat"))
    (tmp_path / "wl.dat").write_text(
        "== header ==\n"
        "1.0 0.5 0.5 0.5 0.3 0.7 0.0 2.0 1.0 0.4 0.6 0.5 0.1 0.2\n"
        "0.5 0.1 0.2 0.3 0.0 0.0 1.0 1.0 0.5 0.5 0.5 0.5 0.0 0.0\n"
        "0\n0.002\n0.25\n")
    lib.get_tracking_time_interval.restype = C.c_double
    assert lib.get_tracking_time_interval(0, str(init).encode(), C.c_double(2.0)) == 2e-2
    lib.get_param_ff(0, str(init).encode())
    import test_particle_gb300 as tp
    prm = tp.ParamFF.in_dll(lib, "param")
    assert (prm.B0, prm.lambda0) == (2.5, 6.25)
    lib.read_wlcs(0, str(init).encode())
    assert C.c_int.in_dll(lib, "nwlcs").value == 2
    cfg = C.cast(C.c_void_p.in_dll(lib, "config").value, C.POINTER(tp.Wlcs))
    assert cfg[0].cur_wr == 0.25 and cfg[0].cur_lp == 0.5 and cfg[1].omega == 0.002
    assert abs(cfg[0].costheta_wr - np.cos(0.3)) < 1e-15 and abs(cfg[0].sinbeta_lp - np.sin(0.2)) < 1e-15
    dt = C.c_double(1.0)
    lib.adjust_dt_normI(C.byref(dt))
    assert abs(dt.value - 1.0 / 0.25 / 2.0) < 1e-15
    lib.free_config()


def test_scalar_helpers(lib):
    assert lib.getgamma(C.c_double(3.0), C.c_double(0.0), C.c_double(4.0)) == np.sqrt(26.0)
    assert lib.modulus(C.c_double(3.0), C.c_double(4.0), C.c_double(12.0)) == 13.0
    cx, cy, cz = C.c_double(), C.c_double(), C.c_double()
    lib.cross_product(C.c_double(1), C.c_double(0), C.c_double(0), C.c_double(0), C.c_double(1),
                      C.c_double(0), C.byref(cx), C.byref(cy), C.byref(cz))
    assert (cx.value, cy.value, cz.value) == (0.0, 0.0, 1.0)


def test_gather_particle_spectra(lib):
    """src/tracking.c:475-493: the per-thread rows add into the spectra; the
    escape spectra only with open boundaries (bc_flag 1)."""
    rng = np.random.default_rng(5)
    nth, nb, nt = 3, 7, 4
    ep = rng.integers(0, 9, (nth, nt * nb)).astype(np.float64)
    eep = rng.integers(0, 9, (nth, nt * nb)).astype(np.float64)
    bc = C.c_int.in_dll(lib, "bc_flag")
    old = bc.value
    try:
        for flag in (1, 0, 2):
            bc.value = flag
            esp, ese = np.full(nt * nb, 0.5), np.full(nt * nb, 0.25)
            lib.gather_particle_spectra_openmp(C.c_int(nth), C.c_int(nb), C.c_int(nt),
                                               esp.ctypes.data_as(C.c_void_p),
                                               ep.ctypes.data_as(C.c_void_p),
                                               ese.ctypes.data_as(C.c_void_p),
                                               eep.ctypes.data_as(C.c_void_p))
            assert np.array_equal(esp, 0.5 + ep.sum(0))
            assert np.array_equal(ese, 0.25 + eep.sum(0) if flag == 1 else np.full(nt * nb, 0.25))
    finally:
        bc.value = old


def test_diff_coeff_file_format(lib, tmp_path):
    """The single-rank collect_diff_coeffs writes the reference's table
    (src/diagnostics.c:723-782): a header line, then per sample the eight
    sums as %10.4e and the remaining particle count."""
    ns = 3
    cols = [np.arange(ns) * (c + 1) * 1.25e-3 for c in range(8)]
    rem = np.array([10, 9, 7], dtype=np.int32)
    fname = str(tmp_path / "dc.dat").encode()
    lib.collect_diff_coeffs(C.c_int(0), C.c_int(ns), *[c.ctypes.data_as(C.c_void_p) for c in cols],
                            C.c_char_p(fname), rem.ctypes.data_as(C.c_void_p))
    lines = (tmp_path / "dc.dat").read_text().splitlines()
    assert lines[0] == "drr        dxx        dyy        dzz        dpp        duu        daa        dee        nptl"
    for i in range(ns):
        want = " ".join("%10.4e" % c[i] for c in cols) + " %d" % rem[i]
        assert lines[1 + i] == want
    # rank > 0 writes nothing
    lib.collect_diff_coeffs(C.c_int(1), C.c_int(ns), *[c.ctypes.data_as(C.c_void_p) for c in cols],
                            C.c_char_p(str(tmp_path / "none.dat").encode()),
                            rem.ctypes.data_as(C.c_void_p))
    assert not (tmp_path / "none.dat").exists()


def test_no_gpu_is_an_error_not_a_fallback(lib):
    """Without a device the compute entry points fail loudly."""
    import test_particle_gb300 as tp
    try:
        import torch
        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = False
    if has_gpu:
        pytest.skip("a GPU is present")
    with pytest.raises(RuntimeError, match="no CUDA device"):
        tp.get_emf(np.zeros((1, 4)))



def test_empty_learned_field_batch_is_a_no_op(lib):
    """An empty (or negative) batch of learned-field evaluations returns at
    once, before any device work or host allocation."""
    assert lib.tp_mlp_eval(0, None, None) == 0
    assert lib.tp_mlp_eval(-5, None, None) == 0


def test_poincare_arguments_are_checked_before_any_device_work(lib):
    """tp_poincare_trace refuses a bad face, step, length or crossing count
    (more than 2^24 crossings per seed: rows indexed with 32-bit counts)
    before it touches the GPU."""
    st = C.c_int.in_dll(lib, "system_type")
    keep = st.value
    st.value = 4
    f = lib.tp_poincare_trace
    f.argtypes = [C.c_int, C.c_void_p, C.c_int, C.c_double, C.c_double, C.c_int, C.c_void_p, C.c_void_p,
                  C.c_void_p, C.c_void_p]
    e = lib.tp_last_error
    e.restype = C.c_char_p
    try:
        for args in ((1, 3, 0.5, 10.0, 4), (1, 2, 0.0, 10.0, 4), (1, 2, 0.5, -1.0, 4), (1, 2, 0.5, 10.0, 0),
                     (1, 2, 0.5, 10.0, (1 << 24) + 1), (-1, 2, 0.5, 10.0, 4)):
            n, face, step, length, nc = args
            assert f(n, None, face, step, length, nc, None, None, None, None) == -1
            assert b"bad Poincare map arguments" in e()
    finally:
        st.value = keep
        lib.tp_clear_status()

@pytest.mark.parametrize("case", ["no_step_label", "no_ff_label", "no_file", "no_wlcs_config"])
def test_config_errors_exit_like_the_reference(tmp_path, case):
    """Malformed or missing configuration: a message on stdout and exit(1), as
    the reference's readers do (src/tracking.c:1226-1255, src/force_free.c:99-125);
    adjust_dt_normI without a wire-loop configuration exits instead of
    dereferencing NULL (src/wlcs.c:266-269).  Run in a child process."""
    import subprocess
    import sys
    init = tmp_path / "init.dat"
    init.write_text(
        "------------------------------ Force-free field ------------------------------\n"
        "Normalized B(Gauss): 2.5\n"
        "------------------------------ Particle tracking -----------------------------\n"
        "Tracking method to use: 0\n")
    call = {
        "no_step_label": "L.get_tracking_time_interval(0, %r, C.c_double(1.0))" % str(init).encode(),
        "no_ff_label": "L.get_param_ff(0, %r)" % str(init).encode(),
        "no_file": "L.get_param_ff(0, %r)" % str(tmp_path / "missing.dat").encode(),
        "no_wlcs_config": "L.free_config(); d = C.c_double(1.0); L.adjust_dt_normI(C.byref(d))",
    }[case]
    code = ("import ctypes as C, test_particle_gb300 as tp\n"
            "L = tp.lib()\nL.get_tracking_time_interval.restype = C.c_double\n" + call + "\n"
            "print('RETURNED')\n")
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=120,
                       cwd=ROOT)
    assert r.returncode == 1, (r.returncode, r.stdout, r.stderr)
    assert "RETURNED" not in r.stdout
    assert r.stdout.strip(), "no message"
