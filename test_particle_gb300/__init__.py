"""GB300 test-particle tracer: Python host bindings of libtpgpu.so.

The compute path is the CUDA library built by ``test_particle_gb300.build``
(sm_103a); this module only loads it through ctypes and mirrors the reference
C API's set-up sequence (set_variables_* / set_ptl_params_tracking / the
field-array globals) so that Python callers drive the same entry points a C
caller of the reference would.  There is no CPU fallback: importing the
bindings without the built library raises.
"""
import ctypes as C
import os

import numpy as np

from . import build as _build

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = _build.LIB

# particles record, include/particle_info.h:6-12 (88 bytes)
PARTICLE_DTYPE = np.dtype([(n, "<f8") for n in
                           ("x", "y", "z", "qm", "ux", "uy", "uz", "t",
                            "xshift", "yshift", "zshift")])
MODE_DTYPE = np.dtype([("n", "<i4", 3), ("pad", "<i4"), ("amp_b", "<f8", 3),
                       ("amp_e", "<f8", 3), ("phase", "<f8"), ("pad2", "<f8")])

PREC_FP64, PREC_FP64_FAST, PREC_MIXED, PREC_SURROGATE = 0, 1, 2, 3
SYS_TEST, SYS_WLCS, SYS_FORCEFREE, SYS_MHD, SYS_PIC, SYS_MODESUM = range(6)


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


class ParamFF(C.Structure):
    _fields_ = [("B0", C.c_double), ("lambda0", C.c_double)]


class RunInfo(C.Structure):
    _fields_ = [("estep", C.c_int), ("einterval", C.c_int), ("nsdc", C.c_int),
                ("nt_out", C.c_int), ("nbins", C.c_int), ("grid", C.c_int),
                ("blocks_per_sm", C.c_int), ("kernel_ms", C.c_double), ("pushes", C.c_double),
                ("step_ms", C.c_double), ("launches", C.c_int)]


def _copy_struct(dst_type, src):
    d = dst_type()
    for name, _ in dst_type._fields_:
        setattr(d, name, getattr(src, name))
    return d


_lib = None
_keep = {}


def lib():
    """Load libtpgpu.so; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError("libtpgpu.so is not built (run test_particle_gb300.build.build()); "
                               "there is no CPU fallback")
        L = C.CDLL(LIB_PATH)
        L.tp_last_error.restype = C.c_char_p
        L.tp_session_create.restype = C.c_void_p
        L.get_tracking_time_interval.restype = C.c_double
        L.getgamma.restype = C.c_double
        L.modulus.restype = C.c_double
        for fn in ("tp_session_destroy", "tp_session_load", "tp_session_track", "tp_session_fetch"):
            getattr(L, fn).argtypes = None
        _lib = L
    return _lib


def check(rc, what="call"):
    if rc != 0:
        L = lib()
        msg = L.tp_last_error().decode(errors="replace")
        L.tp_clear_status()
        raise RuntimeError("%s failed: %s" % (what, msg))


def _ptr(a):
    return C.c_void_p(a.ctypes.data) if a is not None else None


def _set_ptr_global(name, arr):
    L = lib()
    v = C.c_void_p.in_dll(L, name)
    if arr is None:
        v.value = None
        _keep.pop(name, None)
    else:
        a = np.ascontiguousarray(arr)
        _keep[name] = a
        v.value = a.ctypes.data


_GRID_GLOBALS = ("magc_float", "maga_float", "magb_float", "efc_float", "efa_float", "efb_float",
                 "vc_float", "va_float", "vb_float", "magc_double", "maga_double", "magb_double",
                 "efc_double", "efa_double", "efb_double", "vc_double", "va_double", "vb_double")


def configure(system_type=SYS_TEST, charge_mass=1.0, bc_flag=0, dom=None, grd=None, mt=0,
              abc=(1.0, np.sqrt(2.0 / 3.0), np.sqrt(1.0 / 3.0)), B0=1.0, lambda0=1.0,
              vgrid_d=None, vgrid_d_ab=(None, None), vgrid_f=None, vgrid_f_ab=(None, None),
              bgrid=None, bgrid_ab=(None, None), egrid=None, egrid_ab=(None, None),
              wl=None, ibessel=0, modes=None, mode_B0=1.0, interp_corrected=0,
              ellint_corrected=0, **_unused):
    """Set the reference globals through the reference API, as a C caller would
    (get_system_info, src/domain.c:314-409, without the file reads)."""
    L = lib()
    d = _copy_struct(Domain, dom) if dom is not None else Domain()
    g = _copy_struct(Grids, grd) if grd is not None else Grids()
    L.set_variables_emfields(C.c_int(system_type))
    L.set_variables_tracking(C.byref(g), C.byref(d), C.c_int(system_type), C.c_int(mt))
    L.set_ptl_params_tracking(C.c_int(bc_flag), C.c_double(charge_mass))
    ParamFF.in_dll(L, "param").B0 = B0
    ParamFF.in_dll(L, "param").lambda0 = lambda0
    L.tp_set_abc(C.c_double(abc[0]), C.c_double(abc[1]), C.c_double(abc[2]))
    L.tp_set_interp_corrected(C.c_int(interp_corrected))
    L.tp_set_ellint_corrected(C.c_int(ellint_corrected))
    for name in _GRID_GLOBALS:
        _set_ptr_global(name, None)
    _set_ptr_global("vc_double", vgrid_d)
    _set_ptr_global("va_double", vgrid_d_ab[0])
    _set_ptr_global("vb_double", vgrid_d_ab[1])
    _set_ptr_global("vc_float", vgrid_f)
    _set_ptr_global("va_float", vgrid_f_ab[0])
    _set_ptr_global("vb_float", vgrid_f_ab[1])
    _set_ptr_global("magc_float", bgrid)
    _set_ptr_global("maga_float", bgrid_ab[0])
    _set_ptr_global("magb_float", bgrid_ab[1])
    _set_ptr_global("efc_float", egrid)
    _set_ptr_global("efa_float", egrid_ab[0])
    _set_ptr_global("efb_float", egrid_ab[1])
    if wl is not None:
        arr = (Wlcs * len(wl))(*[_copy_struct(Wlcs, w) for w in wl])
        _keep["config"] = arr
        C.c_void_p.in_dll(L, "config").value = C.cast(arr, C.c_void_p).value
        C.c_int.in_dll(L, "nwlcs").value = len(wl)
        C.c_int.in_dll(L, "iBessel").value = ibessel
    else:
        C.c_void_p.in_dll(L, "config").value = None
        C.c_int.in_dll(L, "nwlcs").value = 0
    if modes is not None:
        m = np.ascontiguousarray(modes, dtype=MODE_DTYPE)
        check(L.tp_set_modes(C.c_int(len(m)), _ptr(m), C.c_double(mode_B0)), "tp_set_modes")
    L.tp_mark_fields_dirty()


def set_spectrum(nbins, emin, emax):
    lib().tp_set_spectrum(C.c_int(nbins), C.c_double(emin), C.c_double(emax))


def get_emf(xyzt):
    xyzt = np.ascontiguousarray(xyzt, dtype=np.float64).reshape(-1, 4)
    out = np.zeros((len(xyzt), 6))
    check(lib().tp_get_emf_batch(C.c_int(len(xyzt)), _ptr(xyzt), _ptr(out)), "get_emf")
    return out


def get_emf_mixed(xyz):
    """The mixed path's FP32 field at points (n x 3) -> n x 6 float32 (B, E)."""
    xyz = np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1, 3)
    out = np.zeros((len(xyz), 6), dtype=np.float32)
    check(lib().tp_get_emf_mixed_batch(C.c_int(len(xyz)), _ptr(xyz), _ptr(out)), "get_emf_mixed")
    return out


def wirz_steps(ptl, dt, nsteps):
    p = np.array(ptl, dtype=PARTICLE_DTYPE, copy=True)
    esc = np.zeros(len(p), dtype=np.int32)
    check(lib().tp_wirz_steps(C.c_int(len(p)), _ptr(p), C.c_double(dt), C.c_int(nsteps),
                              _ptr(esc)), "wirz_steps")
    return p, esc


def energy_bins(ptl, nbins):
    p = np.ascontiguousarray(ptl, dtype=PARTICLE_DTYPE)
    out = np.zeros(len(p), dtype=np.int32)
    check(lib().tp_energy_bins(C.c_int(len(p)), _ptr(p), C.c_int(nbins), _ptr(out)), "energy_bins")
    return out


def energy_thresholds(nbins):
    thr = np.zeros(nbins - 1)
    check(lib().tp_energy_thresholds(C.c_int(nbins), _ptr(thr)), "energy_thresholds")
    return thr


def calc_diff_coeff(p0, p, dt):
    p0 = np.ascontiguousarray(p0, dtype=PARTICLE_DTYPE)
    p = np.ascontiguousarray(p, dtype=PARTICLE_DTYPE)
    out = np.zeros((len(p), 8))
    check(lib().tp_calc_diff_coeff_batch(C.c_int(len(p)), _ptr(p0), _ptr(p), C.c_double(dt),
                                         _ptr(out)), "calc_diff_coeff")
    return out


def trilinear(xyzt):
    xyzt = np.ascontiguousarray(xyzt, dtype=np.float64).reshape(-1, 4)
    c = np.zeros((len(xyzt), 8), dtype=np.int64)
    w = np.zeros((len(xyzt), 8))
    check(lib().tp_trilinear_batch(C.c_int(len(xyzt)), _ptr(xyzt), _ptr(c), _ptr(w)), "trilinear")
    return c, w


def set_tmax(tmax):
    """Change simul_domain.tmax (the total tracking time the step count derives from)."""
    Domain.in_dll(lib(), "simul_domain").tmax = tmax


def set_compaction(steps):
    """Open-boundary runs in segments of `steps` steps with departed particles
    dropped between them (0: one launch; -1: automatic)."""
    lib().tp_set_compaction(C.c_int(int(steps)))


def track(ptl_init, dt, nt_out, nbins, precision=PREC_FP64, ptl=None):
    """Fixed-step tracking of all particles on the GPU (host buffers in and out)."""
    L = lib()
    p0 = np.ascontiguousarray(ptl_init, dtype=PARTICLE_DTYPE)
    p = p0.copy() if ptl is None else np.array(ptl, dtype=PARTICLE_DTYPE, copy=True)
    n = len(p0)
    estep = int(Domain.in_dll(L, "simul_domain").tmax / dt)
    nsdc = estep // 100 + 1
    esp = np.zeros(nt_out * nbins)
    ese = np.zeros(nt_out * nbins)
    dsum = np.zeros(8 * nsdc)
    rem = np.zeros(nsdc, dtype=np.int32)
    nst = np.zeros(n, dtype=np.int32)
    info = RunInfo()
    check(L.tp_track_host(C.c_int(precision), C.c_int(n), C.c_double(dt), C.c_int(nt_out),
                          C.c_int(nbins), _ptr(p0), _ptr(p), _ptr(nst), _ptr(esp), _ptr(ese),
                          _ptr(dsum), _ptr(rem), C.byref(info)), "track")
    return dict(ptl=p, estep=info.estep, espect=esp.reshape(nt_out, nbins),
                espect_escape=ese.reshape(nt_out, nbins), dsum=dsum.reshape(8, nsdc),
                remain=rem, nsteps=nst, info=info)


def synth_pic_fields(modes_b, modes_v, B0z, to_host=False):
    """Generate the PIC grids on the GPU for the current simul_grid; optionally
    return the float AoS (E, B) arrays."""
    L = lib()
    mb = np.ascontiguousarray(modes_b, dtype=MODE_DTYPE)
    mv = np.ascontiguousarray(modes_v, dtype=MODE_DTYPE)
    he = hb = None
    if to_host:
        g = Grids.in_dll(L, "simul_grid")
        n = g.nx * g.ny * g.nz
        he = np.zeros((n, 3), dtype=np.float32)
        hb = np.zeros((n, 3), dtype=np.float32)
    check(L.tp_synth_pic_fields(C.c_int(len(mb)), _ptr(mb), C.c_int(len(mv)), _ptr(mv),
                                C.c_double(B0z), _ptr(he), _ptr(hb)), "synth_pic_fields")
    return he, hb


def release_device_fields():
    lib().tp_release_device_fields()


# ---------------------------------------------------------------- learned field model
def mlp_param_count():
    return lib().tp_mlp_param_count()


def mlp_init(freq, weights=None, seed=1):
    f = np.ascontiguousarray(freq, dtype=np.int32).reshape(64, 3)
    w = None if weights is None else np.ascontiguousarray(weights, dtype=np.float32)
    check(lib().tp_mlp_init(_ptr(f), _ptr(w), C.c_ulonglong(seed)), "mlp_init")


def mlp_set_output_norm(mean, std):
    m = np.ascontiguousarray(mean, dtype=np.float32)
    s = np.ascontiguousarray(std, dtype=np.float32)
    check(lib().tp_mlp_set_output_norm(_ptr(m), _ptr(s)), "mlp_set_output_norm")


def mlp_weights():
    w = np.zeros(mlp_param_count(), dtype=np.float32)
    check(lib().tp_mlp_get_weights(_ptr(w)), "mlp_get_weights")
    return w


def mlp_grad(u, t):
    u = np.ascontiguousarray(u, dtype=np.uint32).reshape(-1, 3)
    t = np.ascontiguousarray(t, dtype=np.float32).reshape(-1, 6)
    n = len(u)
    loss = C.c_double()
    y = np.zeros((n, 6), dtype=np.float32)
    g = np.zeros(mlp_param_count(), dtype=np.float32)
    check(lib().tp_mlp_grad(C.c_int(n), _ptr(u), _ptr(t), C.byref(loss), _ptr(y), _ptr(g)), "mlp_grad")
    return loss.value, y, g


def mlp_train(nsamples, batch, epochs, lr=2e-3, wd=0.0, seed=7):
    loss, ms = C.c_double(), C.c_double()
    check(lib().tp_mlp_train(C.c_longlong(nsamples), C.c_int(batch), C.c_int(epochs), C.c_double(lr),
                             C.c_double(wd), C.c_ulonglong(seed), C.byref(loss), C.byref(ms)),
          "mlp_train")
    return loss.value, ms.value


def mlp_eval(u):
    u = np.ascontiguousarray(u, dtype=np.uint32).reshape(-1, 3)
    out = np.zeros((len(u), 6), dtype=np.float32)
    check(lib().tp_mlp_eval(C.c_int(len(u)), _ptr(u), _ptr(out)), "mlp_eval")
    return out


def mlp_eval_kernel(u):
    u = np.ascontiguousarray(u, dtype=np.uint32).reshape(-1, 3)
    out = np.zeros((len(u), 6), dtype=np.float32)
    check(lib().tp_mlp_eval_kernel(C.c_int(len(u)), _ptr(u), _ptr(out)), "mlp_eval_kernel")
    return out


def device_status():
    return lib().tp_device_status()


class Session:
    """Device-resident particles: load once, track repeatedly, fetch results."""

    def __init__(self, nptl):
        self.L = lib()
        self.n = nptl
        self.h = self.L.tp_session_create(C.c_int(nptl))
        if not self.h:
            check(-1, "tp_session_create")

    def load(self, ptl_init, ptl=None):
        p0 = np.ascontiguousarray(ptl_init, dtype=PARTICLE_DTYPE)
        p = p0 if ptl is None else np.ascontiguousarray(ptl, dtype=PARTICLE_DTYPE)
        check(self.L.tp_session_load(C.c_void_p(self.h), _ptr(p0), _ptr(p)), "session load")

    def track(self, dt, nt_out, nbins, precision=PREC_FP64):
        info = RunInfo()
        check(self.L.tp_session_track(C.c_void_p(self.h), C.c_int(precision), C.c_double(dt),
                                      C.c_int(nt_out), C.c_int(nbins), C.byref(info)),
              "session track")
        return info

    def fetch(self, nt_out, nbins, nsdc, particles=True):
        """Results of the last run; particles=False skips the particle state
        and step counts (spectra, diffusion sums and remaining counts only)."""
        p = np.zeros(self.n, dtype=PARTICLE_DTYPE) if particles else None
        esp = np.zeros(nt_out * nbins)
        ese = np.zeros(nt_out * nbins)
        dsum = np.zeros(8 * nsdc)
        rem = np.zeros(nsdc, dtype=np.int32)
        nst = np.zeros(self.n, dtype=np.int32) if particles else None
        check(self.L.tp_session_fetch(C.c_void_p(self.h), _ptr(p), _ptr(nst), _ptr(esp),
                                      _ptr(ese), _ptr(dsum), _ptr(rem)), "session fetch")
        return dict(ptl=p, espect=esp.reshape(nt_out, nbins), espect_escape=ese.reshape(nt_out, nbins),
                    dsum=dsum.reshape(8, nsdc), remain=rem + self.n, nsteps=nst)

    def close(self):
        if self.h:
            self.L.tp_session_destroy(C.c_void_p(self.h))
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def poincare_trace(seeds, face, step, length_max, ncross):
    """Crossings of the plane pos[face] = seed[face] by the field lines of the
    gridded B through each seed (tp_poincare_trace): xpos, ypos, zpos
    [n][ncross + 1] (entry 0 the seed) and the crossings reached per seed."""
    s = np.ascontiguousarray(seeds, dtype=np.float64).reshape(-1, 3)
    n = len(s)
    xo = np.zeros((n, ncross + 1))
    yo = np.zeros((n, ncross + 1))
    zo = np.zeros((n, ncross + 1))
    found = np.zeros(n, dtype=np.int32)
    check(lib().tp_poincare_trace(C.c_int(n), _ptr(s), C.c_int(face), C.c_double(step),
                                  C.c_double(length_max), C.c_int(ncross), _ptr(xo), _ptr(yo),
                                  _ptr(zo), _ptr(found)), "poincare_trace")
    return xo, yo, zo, found


def measure_fma_peaks():
    """CUDA-core peaks from the library's FMA-chain microbenchmark (FLOP/s):
    {"fp32": ..., "fp64": ..., "fp32x2": ...}."""
    out = {}
    for kind, name in ((0, "fp32"), (1, "fp64"), (2, "fp32x2")):
        v = C.c_double()
        check(lib().tp_measure_fma_peak(C.c_int(kind), C.byref(v)), "measure_fma_peak")
        out[name] = v.value
    return out


def read_pic_fields_binary(filepath, ct):
    """Load <filepath>{bx,by,bz,ex,ey,ez}_<ct>.gda into device memory
    (tp_read_pic_fields_binary), scaled by the B0 / E0 set through
    set_variables_bfield / set_variables_efield."""
    check(lib().tp_read_pic_fields_binary(str(filepath).encode(), C.c_int(ct)), "read_pic_fields_binary")


def fetch_device_fields():
    """Host copies (E, B) of the device-resident PIC-style fields, n x 3 float32."""
    L = lib()
    g = Grids.in_dll(L, "simul_grid")
    n = g.nx * g.ny * g.nz
    he = np.zeros((n, 3), dtype=np.float32)
    hb = np.zeros((n, 3), dtype=np.float32)
    check(L.tp_fetch_device_fields(_ptr(he), _ptr(hb)), "fetch_device_fields")
    return he, hb


# ---------------------------------------------------------------- HDF5 files (no libhdf5)
def read_pic_fields_h5(fname, gname, with_e=True):
    """Load the [nx][ny][nz] datasets cbx, cby, cbz (and ex, ey, ez) of group
    gname into device memory, transposed to the reference's x-fastest records
    and scaled by B0 / E0 (tp_read_pic_fields_h5; the reference's
    read_pic_bfields_h5 / read_pic_efields_h5)."""
    check(lib().tp_read_pic_fields_h5(str(fname).encode(), str(gname).encode(), C.c_int(1 if with_e else 0)),
          "read_pic_fields_h5")


def save_pic_fields_h5(fname, gname, with_e=True):
    """Write the device-resident PIC fields as the reference's PIC HDF5 file
    (tp_save_pic_fields_h5): float datasets cbx, cby, cbz (ex, ey, ez) of
    [nx][ny][nz], the records divided by B0 (E0)."""
    check(lib().tp_save_pic_fields_h5(str(fname).encode(), str(gname).encode(), C.c_int(1 if with_e else 0)),
          "save_pic_fields_h5")


def h5_info(fname, gname, dset):
    """(dims, type class, type size) of dataset gname/dset (tp_h5_info)."""
    rank, cls, size = C.c_int(), C.c_int(), C.c_int()
    dims = (C.c_ulonglong * 32)()
    check(lib().tp_h5_info(str(fname).encode(), str(gname).encode(), str(dset).encode(), C.byref(rank), dims,
                           C.byref(cls), C.byref(size)), "h5_info")
    return tuple(dims[i] for i in range(rank.value)), cls.value, size.value


def h5_read(fname, gname, dset, offset=None, count=None, dtype=np.float64):
    """The hyperslab [offset, offset + count) of a numeric dataset as float64
    or float32 (tp_h5_read; the whole dataset by default)."""
    dims, _, _ = h5_info(fname, gname, dset)
    offset = [0] * len(dims) if offset is None else list(offset)
    count = [d - o for d, o in zip(dims, offset)] if count is None else list(count)
    dt = np.dtype(dtype)
    out = np.zeros(count, dtype=dt)
    r = len(dims)
    check(lib().tp_h5_read(str(fname).encode(), str(gname).encode(), str(dset).encode(), C.c_int(r),
                           (C.c_ulonglong * max(r, 1))(*count), (C.c_ulonglong * max(r, 1))(*offset),
                           C.c_int(dt.itemsize), _ptr(out)), "h5_read")
    return out


def save_particles_fields(fname, ptl, ntot=None, offset=0):
    """Write records [offset, offset + len(ptl)) of a particles_fields file of
    ntot records (default len(ptl)), with the fields at each record from the
    library's FP64 get_emf on the GPU (tp_save_particles_fields); the writer
    of the records at offset 0 also writes the file's metadata."""
    p = np.ascontiguousarray(ptl, dtype=PARTICLE_DTYPE)
    ntot = len(p) if ntot is None else int(ntot)
    acc = np.array([offset], dtype=np.int32)
    check(lib().tp_save_particles_fields(C.c_int(1 if offset else 0), C.c_int(len(p)), _ptr(p), C.c_int(ntot),
                                         _ptr(acc), str(fname).encode(), C.c_int(0)), "save_particles_fields")


def read_particles(fname, n, offset=0):
    """Records [offset, offset + n) of /particles_fields/particles
    (tp_read_particles); the shifts are zero."""
    p = np.zeros(n, dtype=PARTICLE_DTYPE)
    acc = np.array([offset], dtype=np.int32)
    check(lib().tp_read_particles(C.c_int(1 if offset else 0), C.c_int(n), _ptr(acc), _ptr(p),
                                  str(fname).encode()), "read_particles")
    return p


def trajectory_diagnostics(ptl, nsteps, ptl_init, dt, nptl_traj, nbins, nt_out, nsteps_output, system_type,
                           bc_flag=0, tracking_method=0, pmass=1.0):
    """The reference's trajectory diagnostics in one process
    (tp_trajectory_diagnostics): reads data/particles_fields_init.h5, writes
    data/particle_diagnostics.h5.  ptl and nsteps (final particles and their
    step counts) are updated in place as the reference updates them; returns
    the trajectory output interval actually used."""
    assert ptl.dtype == PARTICLE_DTYPE and ptl.flags.c_contiguous
    assert nsteps.dtype == np.int32 and nsteps.flags.c_contiguous
    init = np.ascontiguousarray(ptl_init, dtype=PARTICLE_DTYPE)
    every = C.c_int(nsteps_output)
    L = lib()
    L.tp_trajectory_diagnostics.argtypes = [C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_int, C.c_int,
                                            C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_void_p,
                                            C.c_int, C.c_int, C.c_void_p]
    check(L.tp_trajectory_diagnostics(0, 1, len(ptl), dt, pmass, nptl_traj, system_type, _ptr(ptl), None,
                                      _ptr(nsteps), nbins, nt_out, C.byref(every), bc_flag, tracking_method,
                                      _ptr(init)), "trajectory_diagnostics")
    return every.value
