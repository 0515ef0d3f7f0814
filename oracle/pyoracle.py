"""ctypes bindings for the oracle (oracle/tp_oracle.c) and for the pinning
build of the reference (oracle/_ref/libtpref.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, by the smoke check and by the
CPU-baseline leg of bench.py.  The product package never imports this module.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
BUILD = os.path.join(HERE, "_build")
LIB_ORACLE = os.path.join(BUILD, "liboracle.so")
LIB_REF = os.path.join(HERE, "_ref", "libtpref.so")

# particles record, include/particle_info.h:6-12 (88 bytes)
PARTICLE_DTYPE = np.dtype([(n, "<f8") for n in
                           ("x", "y", "z", "qm", "ux", "uy", "uz", "t",
                            "xshift", "yshift", "zshift")])


class Domain(C.Structure):
    _fields_ = [(n, C.c_double) for n in
                ("xmin_ptl", "xmax_ptl", "ymin_ptl", "ymax_ptl", "zmin_ptl", "zmax_ptl",
                 "xmin", "xmax", "ymin", "ymax", "zmin", "zmax", "tmin", "tmax")]


class Grids(C.Structure):
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int), ("nt", C.c_int),
                ("dx", C.c_double), ("dy", C.c_double), ("dz", C.c_double), ("dt", C.c_double)]


class Wlcs(C.Structure):
    _fields_ = [(n, C.c_double) for n in
                ("x_wr", "y_wr", "z_wr", "costheta_wr", "cosphi_wr", "sintheta_wr",
                 "sinphi_wr", "cur_wr", "t0", "x_lp", "y_lp", "z_lp", "r_lp",
                 "cosalpha_lp", "cosbeta_lp", "sinalpha_lp", "sinbeta_lp", "cur_lp", "omega")]


class Mode(C.Structure):
    _fields_ = [("n", C.c_int * 3), ("pad", C.c_int), ("amp_b", C.c_double * 3),
                ("amp_e", C.c_double * 3), ("phase", C.c_double), ("pad2", C.c_double)]


MODE_DTYPE = np.dtype([("n", "<i4", 3), ("pad", "<i4"), ("amp_b", "<f8", 3),
                       ("amp_e", "<f8", 3), ("phase", "<f8"), ("pad2", "<f8")])
assert MODE_DTYPE.itemsize == C.sizeof(Mode)


class OrField(C.Structure):
    _fields_ = [("system_type", C.c_int), ("charge_mass", C.c_double), ("bc_flag", C.c_int),
                ("dom", Domain), ("grd", Grids), ("multi_tframe", C.c_int),
                ("interp_corrected", C.c_int), ("ellint_corrected", C.c_int),
                ("ffA", C.c_double), ("ffB", C.c_double), ("ffC", C.c_double),
                ("B0", C.c_double), ("lambda0", C.c_double),
                ("vc_d", C.c_void_p), ("va_d", C.c_void_p), ("vb_d", C.c_void_p),
                ("vc_f", C.c_void_p), ("va_f", C.c_void_p), ("vb_f", C.c_void_p),
                ("bc_f", C.c_void_p), ("ba_f", C.c_void_p), ("bb_f", C.c_void_p),
                ("ec_f", C.c_void_p), ("ea_f", C.c_void_p), ("eb_f", C.c_void_p),
                ("nwlcs", C.c_int), ("iBessel", C.c_int), ("cfg", C.c_void_p),
                ("nmodes", C.c_int), ("modes", C.c_void_p)]


class OrSpectrum(C.Structure):
    _fields_ = [("nbins", C.c_int), ("emin", C.c_double), ("emax", C.c_double),
                ("logemin", C.c_double), ("logemax", C.c_double), ("logde", C.c_double)]


class OrBsCfg(C.Structure):
    _fields_ = [("atol", C.c_double), ("rtol", C.c_double), ("kmaxx", C.c_int),
                ("max_rejects", C.c_int)]


def build_oracle(force=False):
    """Compile oracle/tp_oracle.c into oracle/_build/liboracle.so."""
    src = os.path.join(HERE, "tp_oracle.c")
    deps = [src, os.path.join(HERE, "tp_oracle.h"),
            os.path.join(ROOT, "test_particle_gb300", "csrc", "ellint_coeffs.h")]
    if (not force and os.path.exists(LIB_ORACLE) and
            os.path.getmtime(LIB_ORACLE) >= max(os.path.getmtime(d) for d in deps)):
        return LIB_ORACLE
    os.makedirs(BUILD, exist_ok=True)
    tmp = LIB_ORACLE + ".%d.tmp" % os.getpid()
    subprocess.check_call(["gcc", "-O2", "-fPIC", "-fopenmp", "-ffp-contract=off",
                           "-shared", "-o", tmp, src, "-lm"])
    os.replace(tmp, LIB_ORACLE)
    return LIB_ORACLE


def build_ref():
    """Compile the reference's own sources into oracle/_ref (needs the reference
    tree; the recipe says where it looks and exits without building when the
    tree is absent)."""
    subprocess.check_call(["bash", os.path.join(HERE, "build_ref.sh")])
    return LIB_REF if os.path.exists(LIB_REF) else None


def reference_dir():
    """The reference tree: $TP_REFERENCE_DIR, else the tree oracle/_ref was
    last built from; None when neither names an existing tree."""
    d = os.environ.get("TP_REFERENCE_DIR")
    if not d:
        try:
            with open(os.path.join(HERE, "_ref", "source_dir")) as f:
                d = f.read().strip()
        except OSError:
            d = None
    return d if d and os.path.isdir(os.path.join(d, "src")) else None


_oracle = None


def oracle():
    global _oracle
    if _oracle is None:
        _oracle = C.CDLL(build_oracle())
        _oracle.or_estep.restype = C.c_int
        _oracle.or_track_fixed.restype = C.c_int
        _oracle.or_energy_bin.restype = C.c_int
        _oracle.or_energy_bin_e.restype = C.c_int
        _oracle.or_bs_integrate.restype = C.c_int
        _oracle.or_bs_run_many.restype = C.c_long
    return _oracle


def ref_available():
    return os.path.exists(LIB_REF)


_ref = None


def ref():
    global _ref
    if _ref is None:
        _ref = C.CDLL(LIB_REF)
    return _ref


def ptr(a):
    return C.c_void_p(a.ctypes.data) if a is not None else None


def make_field(system_type=0, charge_mass=1.0, bc_flag=0, dom=None, grd=None,
               multi_tframe=0, interp_corrected=0, ellint_corrected=0,
               abc=(1.0, np.sqrt(2.0 / 3.0), np.sqrt(1.0 / 3.0)), B0=1.0, lambda0=1.0,
               vgrid_d=None, vgrid_d_ab=(None, None), vgrid_f=None, vgrid_f_ab=(None, None),
               bgrid=None, bgrid_ab=(None, None), egrid=None, egrid_ab=(None, None),
               wl=None, ibessel=0, modes=None):
    """Build an OrField; keeps references to the arrays it points at."""
    f = OrField()
    f.system_type = system_type
    f.charge_mass = charge_mass
    f.bc_flag = bc_flag
    if dom is not None:
        f.dom = dom
    if grd is not None:
        f.grd = grd
    f.multi_tframe = multi_tframe
    f.interp_corrected = interp_corrected
    f.ellint_corrected = ellint_corrected
    f.ffA, f.ffB, f.ffC = abc
    f.B0 = B0
    f.lambda0 = lambda0
    keep = []

    def setp(name, arr):
        if arr is not None:
            a = np.ascontiguousarray(arr)
            keep.append(a)
            setattr(f, name, a.ctypes.data)

    setp("vc_d", vgrid_d)
    setp("va_d", vgrid_d_ab[0])
    setp("vb_d", vgrid_d_ab[1])
    setp("vc_f", vgrid_f)
    setp("va_f", vgrid_f_ab[0])
    setp("vb_f", vgrid_f_ab[1])
    setp("bc_f", bgrid)
    setp("ba_f", bgrid_ab[0])
    setp("bb_f", bgrid_ab[1])
    setp("ec_f", egrid)
    setp("ea_f", egrid_ab[0])
    setp("eb_f", egrid_ab[1])
    if wl is not None:
        arr = (Wlcs * len(wl))(*wl)
        keep.append(arr)
        f.cfg = C.cast(arr, C.c_void_p)
        f.nwlcs = len(wl)
        f.iBessel = ibessel
    if modes is not None:
        m = np.ascontiguousarray(modes, dtype=MODE_DTYPE)
        keep.append(m)
        f.modes = m.ctypes.data
        f.nmodes = len(m)
    f._keep = keep
    return f


def spectrum(nbins, emin, emax):
    s = OrSpectrum()
    oracle().or_spectrum_init(C.byref(s), C.c_int(nbins), C.c_double(emin), C.c_double(emax))
    return s


def synth_pic_fields(modes_b, modes_v, B0z, nx, ny, nz, nthreads=0):
    """The synthetic gridded (E, B) of the test workload on the CPU, as float
    AoS arrays (n x 3 each), nodes x fastest."""
    mb = np.ascontiguousarray(modes_b, dtype=MODE_DTYPE)
    mv = np.ascontiguousarray(modes_v, dtype=MODE_DTYPE)
    n = nx * ny * nz
    e = np.zeros((n, 3), dtype=np.float32)
    b = np.zeros((n, 3), dtype=np.float32)
    oracle().or_synth_pic_fields(C.c_int(len(mb)), ptr(mb), C.c_int(len(mv)), ptr(mv),
                                 C.c_double(B0z), C.c_int(nx), C.c_int(ny), C.c_int(nz), ptr(e), ptr(b),
                                 C.c_int(nthreads))
    return e, b


def pic_records_from_c(data, scale, comp, rec):
    """The reference's reorder of one PIC HDF5 component ([nx][ny][nz] float32)
    into rec (n x 3 float32, x fastest), in place; returns rec."""
    d = np.ascontiguousarray(data, dtype=np.float32)
    nx, ny, nz = d.shape
    assert rec.dtype == np.float32 and rec.flags.c_contiguous and rec.size == 3 * d.size
    oracle().or_pic_records_from_c(ptr(d), C.c_long(nx), C.c_long(ny), C.c_long(nz), C.c_double(scale),
                                   C.c_int(comp), ptr(rec))
    return rec


def get_emf(f, xyzt):
    xyzt = np.ascontiguousarray(xyzt, dtype=np.float64).reshape(-1, 4)
    out = np.zeros((len(xyzt), 6))
    oracle().or_get_emf_batch(C.byref(f), C.c_int(len(xyzt)), ptr(xyzt), ptr(out))
    return out


def wirz_steps(f, ptl, dt, nsteps):
    p = np.array(ptl, dtype=PARTICLE_DTYPE, copy=True)
    esc = np.zeros(len(p), dtype=np.int32)
    oracle().or_wirz_steps(C.byref(f), C.c_int(len(p)), ptr(p), C.c_double(dt),
                           C.c_int(nsteps), ptr(esc))
    return p, esc


def energy_bins(s, ptl):
    p = np.ascontiguousarray(ptl, dtype=PARTICLE_DTYPE)
    out = np.zeros(len(p), dtype=np.int32)
    oracle().or_energy_bins(C.byref(s), C.c_int(len(p)), ptr(p), ptr(out))
    return out


def ellint(k, corrected=0):
    k = np.ascontiguousarray(k, dtype=np.float64)
    e = np.zeros_like(k)
    kk = np.zeros_like(k)
    lib = oracle()
    for i in range(len(k)):
        ee, ek = C.c_double(), C.c_double()
        lib.or_ellint(C.c_double(k[i]), C.c_int(corrected), C.byref(ee), C.byref(ek))
        e[i], kk[i] = ee.value, ek.value
    return e, kk


def trilinear(f, xyzt):
    xyzt = np.ascontiguousarray(xyzt, dtype=np.float64).reshape(-1, 4)
    c = np.zeros((len(xyzt), 8), dtype=np.int64)
    w = np.zeros((len(xyzt), 8))
    oracle().or_trilinear_batch(C.byref(f), C.c_int(len(xyzt)), ptr(xyzt), ptr(c), ptr(w))
    return c, w


def calc_diff_coeff(f, p0, p, dt):
    p0 = np.ascontiguousarray(p0, dtype=PARTICLE_DTYPE)
    p = np.ascontiguousarray(p, dtype=PARTICLE_DTYPE)
    out = np.zeros((len(p), 8))
    lib = oracle()
    o = np.zeros(8)
    for i in range(len(p)):
        lib.or_calc_diff_coeff(C.byref(f), ptr(p0[i:i + 1]), ptr(p[i:i + 1]), C.c_double(dt), ptr(o))
        out[i] = o
    return out


def track_fixed(f, s, ptl_init, dt, nt_out, nthreads=1):
    """Whole fixed-step run; returns dict of final particles and diagnostics."""
    lib = oracle()
    p0 = np.ascontiguousarray(ptl_init, dtype=PARTICLE_DTYPE)
    p = p0.copy()
    n = len(p)
    estep = lib.or_estep(C.byref(f), C.c_double(dt))
    nsdc = estep // 100 + 1
    esp = np.zeros(nt_out * s.nbins)
    ese = np.zeros(nt_out * s.nbins)
    dsum = np.zeros(8 * nsdc)
    rem = np.zeros(nsdc, dtype=np.int32)
    nst = np.zeros(n, dtype=np.int32)
    rc = lib.or_track_fixed(C.byref(f), C.byref(s), C.c_int(n), C.c_double(dt),
                            C.c_int(nt_out), ptr(p0), ptr(p), ptr(nst), ptr(esp), ptr(ese),
                            ptr(dsum), ptr(rem), C.c_int(nthreads))
    if rc < 0:
        raise ValueError("or_track_fixed failed: %d" % rc)
    return dict(ptl=p, estep=estep, espect=esp.reshape(nt_out, s.nbins),
                espect_escape=ese.reshape(nt_out, s.nbins),
                dsum=dsum.reshape(8, nsdc), remain=rem, nsteps=nst)


def bs_integrate(f, y0, t0, h0, nsteps, atol=1e-5, rtol=1e-14, kmaxx=8, max_rejects=0):
    cfg = OrBsCfg(atol, rtol, kmaxx, max_rejects)
    y = np.array(y0, dtype=np.float64, copy=True)
    out = np.zeros((nsteps, 8))
    rc = oracle().or_bs_integrate(C.byref(f), C.byref(cfg), ptr(y), C.c_double(t0),
                                  C.c_double(h0), C.c_int(nsteps), ptr(out))
    if rc != 0:
        raise ValueError("or_bs_integrate failed: %d" % rc)
    return out


def bs_run_many(f, y0, h0, nsteps, atol=1e-10, rtol=1e-10, kmaxx=8, nthreads=0):
    """nsteps accepted steps of every particle (OpenMP); returns the step total."""
    cfg = OrBsCfg(atol, rtol, kmaxx, 200)
    y = np.ascontiguousarray(y0, dtype=np.float64).copy()
    return oracle().or_bs_run_many(C.byref(f), C.byref(cfg), C.c_int(len(y)), ptr(y), C.c_double(h0),
                                   C.c_int(nsteps), C.c_int(nthreads))


def next_location_steps(f, seeds, step, nsteps):
    """nsteps RK4 field-line steps of the restatement from each seed; [n][nsteps][3]."""
    lib = oracle()
    s = np.ascontiguousarray(seeds, dtype=np.float64).reshape(-1, 3)
    out = np.zeros((len(s), nsteps, 3))
    for i in range(len(s)):
        x, y, z = C.c_double(s[i, 0]), C.c_double(s[i, 1]), C.c_double(s[i, 2])
        for k in range(nsteps):
            lib.or_next_location(C.byref(f), C.byref(x), C.byref(y), C.byref(z), C.c_double(step))
            out[i, k] = (x.value, y.value, z.value)
    return out


def poincare(f, seeds, face, step, length_max, ncross, nthreads=0):
    """Crossing points of every seed: (xpos, ypos, zpos) [n][ncross+1] and counts."""
    s = np.ascontiguousarray(seeds, dtype=np.float64).reshape(-1, 3)
    n = len(s)
    xo = np.zeros((n, ncross + 1))
    yo = np.zeros((n, ncross + 1))
    zo = np.zeros((n, ncross + 1))
    found = np.zeros(n, dtype=np.int32)
    oracle().or_poincare_many(C.byref(f), C.c_int(n), ptr(s), C.c_int(face), C.c_double(step),
                              C.c_double(length_max), C.c_int(ncross), ptr(xo), ptr(yo), ptr(zo),
                              ptr(found), C.c_int(nthreads))
    return xo, yo, zo, found
