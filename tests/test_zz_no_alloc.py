"""tp_track_mixed_noalloc, the tracking entry point that allocates no device
memory, for callers whose host framework owns every device allocation or
that may not allocate after start-up.  It is checked against the session
entry point of the same mixed-precision kernel (tp_track_host).  The caller
owns every buffer (torch tensors here), including the status word the kernel
reports into; two calls in a row must each reproduce the session's result,
which also shows that each call clears the shared scratch it reuses."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
tp = pytest.importorskip("test_particle_gb300")
torch = pytest.importorskip("torch")
import test_particle_gb300.workloads as wl  # noqa: E402

EINVAL, ETOOBIG = 1, 2
COLS = ("x", "y", "z", "qm", "ux", "uy", "uz", "t", "xshift", "yshift", "zshift")


class NoallocArgs(C.Structure):
    """tp_noalloc_args of include/tp_gpu.h."""
    _fields_ = [("n", C.c_int), ("system_type", C.c_int), ("estep", C.c_int),
                ("nt_out", C.c_int), ("nbins", C.c_int), ("bc_flag", C.c_int),
                ("interp_corrected", C.c_int), ("nx", C.c_int), ("ny", C.c_int),
                ("nz", C.c_int), ("dt", C.c_double), ("charge_mass", C.c_double),
                ("emin", C.c_double), ("emax", C.c_double), ("lo", C.c_double * 3),
                ("hi", C.c_double * 3), ("abc", C.c_double * 3), ("B0", C.c_double),
                ("lambda0", C.c_double), ("d_grid", C.c_void_p), ("d_state", C.c_void_p),
                ("d_state0", C.c_void_p), ("d_nsteps", C.c_void_p), ("d_espect", C.c_void_p),
                ("d_espect_escape", C.c_void_p), ("d_dsum", C.c_void_p),
                ("d_remain", C.c_void_p), ("stream", C.c_void_p), ("d_status", C.c_void_p)]


def _fn():
    f = tp.lib().tp_track_mixed_noalloc
    f.argtypes = [C.POINTER(NoallocArgs)]
    f.restype = C.c_int
    return f


def _case(kind, steps=300, n=4096, seed=21):
    """Configure the library globals for the session call and return the
    matching argument block (without buffers) and the initial particles."""
    dom = tp.Domain()
    a = NoallocArgs()
    if kind == "abc":
        cfg = wl.config_abc(nptl=n, steps=steps)
        dom.xmax = dom.ymax = dom.zmax = 1.0
        dom.tmax = steps * cfg["dt"] + 0.5 * cfg["dt"]
        tp.configure(system_type=tp.SYS_FORCEFREE, dom=dom, abc=(1.0, 1.0, 1.0), B0=1.0,
                     lambda0=2 * np.pi)
        a.system_type, a.bc_flag = tp.SYS_FORCEFREE, 0
        a.abc[:] = (1.0, 1.0, 1.0)
        a.B0, a.lambda0 = 1.0, 2 * np.pi
        grid = None
    else:
        ng = 40
        cfg = wl.config_grid(nptl=n, steps=steps, n=ng, dx=0.25)
        L = cfg["hi"][0]
        dom.xmax = dom.ymax = dom.zmax = L
        dom.tmax = steps * cfg["dt"] + 0.5 * cfg["dt"]
        grd = tp.Grids()
        grd.nx = grd.ny = grd.nz = ng
        grd.dx = grd.dy = grd.dz = 0.25
        tp.configure(system_type=tp.SYS_PIC, dom=dom, grd=grd, bc_flag=1)
        mb = wl.kolmogorov_modes(64, 1, 8, 0.5, seed)
        mv = wl.kolmogorov_modes(64, 1, 8, 0.1, seed + 1)
        he, hb = tp.synth_pic_fields(mb, mv, 1.0, to_host=True)
        g = np.zeros((len(he), 8), dtype=np.float32)  # per node {Ex,Ey,Ez,Bx,By,Bz,0,0}
        g[:, 0:3] = he
        g[:, 3:6] = hb
        grid = torch.from_numpy(g).cuda()
        a.system_type, a.bc_flag = tp.SYS_PIC, 1
        a.nx = a.ny = a.nz = ng
        a.d_grid = grid.data_ptr()
    tp.set_spectrum(200, 1e-3, 1e2)
    a.estep, a.nt_out, a.nbins = steps, 3, 200
    a.dt, a.charge_mass, a.emin, a.emax = cfg["dt"], 1.0, 1e-3, 1e2
    a.lo[:] = (dom.xmin, dom.ymin, dom.zmin)
    a.hi[:] = (dom.xmax, dom.ymax, dom.zmax)
    p0 = wl.shell_particles(n, 0.7, cfg["lo"], cfg["hi"], seed)
    return cfg, a, p0, grid


def _run_noalloc(a, p0, status=None):
    """One call on caller-owned buffers; `status` (a device int32 tensor, or
    None for no status word) receives the kernel's status bits."""
    n = len(p0)
    nsdc = a.estep // 100 + 1
    cols = np.stack([np.ascontiguousarray(p0[c]) for c in COLS])
    state0 = torch.from_numpy(cols).cuda()
    state = state0.clone()
    nsteps = torch.zeros(n, dtype=torch.int32, device="cuda")
    esp = torch.full((a.nt_out, a.nbins), 7, dtype=torch.int32, device="cuda")
    ese = torch.full((a.nt_out, a.nbins), 7, dtype=torch.int32, device="cuda")
    dsum = torch.zeros((8, nsdc), dtype=torch.float64, device="cuda")
    rem = torch.full((nsdc,), -5, dtype=torch.int32, device="cuda")
    a.n = n
    a.d_state, a.d_state0 = state.data_ptr(), state0.data_ptr()
    a.d_nsteps, a.d_espect, a.d_espect_escape = nsteps.data_ptr(), esp.data_ptr(), ese.data_ptr()
    a.d_dsum, a.d_remain = dsum.data_ptr(), rem.data_ptr()
    a.stream = torch.cuda.current_stream().cuda_stream
    a.d_status = status.data_ptr() if status is not None else None
    torch.cuda.synchronize()
    free_before = torch.cuda.mem_get_info()[0]
    rc = _fn()(C.byref(a))
    torch.cuda.synchronize()
    assert rc == 0, rc
    return dict(free_change=torch.cuda.mem_get_info()[0] - free_before,
                state=state.cpu().numpy(), nsteps=nsteps.cpu().numpy(),
                espect=esp.cpu().numpy().astype(np.float64),
                espect_escape=ese.cpu().numpy().astype(np.float64),
                dsum=dsum.cpu().numpy(), remain=rem.cpu().numpy())


def _compare(r, ref):
    for k, c in enumerate(COLS):
        assert np.array_equal(r["state"][k], ref["ptl"][c]), c
    assert np.array_equal(r["nsteps"], ref["nsteps"])
    assert np.array_equal(r["espect"], ref["espect"])
    assert np.array_equal(r["espect_escape"], ref["espect_escape"])
    assert np.array_equal(r["remain"], ref["remain"])
    # the same kernel on the same launch geometry: sums agree to rounding
    np.testing.assert_allclose(r["dsum"], ref["dsum"], rtol=1e-12, atol=1e-300)


@pytest.mark.parametrize("kind", ["abc", "pic"])
def test_noalloc_matches_session_twice(kind):
    cfg, a, p0, grid = _case(kind)
    ref = tp.track(p0, cfg["dt"], a.nt_out, a.nbins, precision=tp.PREC_MIXED)
    assert ref["estep"] == a.estep
    assert tp.device_status() == 0  # the session run raised no status bit
    st = torch.full((1,), -1, dtype=torch.int32, device="cuda")  # the call clears it
    first = _run_noalloc(a, p0, status=st)
    assert int(st.item()) == 0
    second = _run_noalloc(a, p0)  # no status word: the call still runs
    # the first call on a device may load the library's kernels; later calls
    # leave the device's free memory as they found it
    assert second["free_change"] == 0
    _compare(first, ref)
    _compare(second, ref)
    if kind == "pic":
        assert ref["espect_escape"].sum() > 0  # open boundary: some particles left
    del grid


def test_noalloc_reports_a_nonfinite_particle():
    """A particle with a NaN momentum (every index the kernel forms from a
    position stays inside the field whatever the value, so the run is safe)
    raises status bit 2 in the caller's word; the other particles are
    tracked as without it."""
    cfg, a, p0, _ = _case("abc", steps=100, n=512)
    bad = p0.copy()
    bad["ux"][17] = np.nan
    st = torch.zeros(1, dtype=torch.int32, device="cuda")
    r = _run_noalloc(a, bad, status=st)
    assert int(st.item()) & 2
    clean = _run_noalloc(a, p0, status=st)
    assert int(st.item()) == 0
    keep = np.arange(len(p0)) != 17
    for k in (4, 5, 6):  # ux, uy, uz of every other particle
        assert np.array_equal(r["state"][k][keep], clean["state"][k][keep])


def test_noalloc_rejects_bad_sizes():
    a = NoallocArgs()
    assert _fn()(C.byref(a)) == EINVAL  # n = 0 and null buffers
    buf = torch.zeros(64, dtype=torch.float64, device="cuda")
    p = buf.data_ptr()
    a.n, a.system_type, a.nt_out, a.nbins, a.dt = 1, tp.SYS_FORCEFREE, 1, 200, 0.1
    a.emin, a.emax, a.B0, a.lambda0 = 1e-3, 1e2, 1.0, 2 * np.pi
    a.abc[:] = (1.0, 1.0, 1.0)
    a.hi[:] = (1.0, 1.0, 1.0)
    a.d_state = a.d_state0 = a.d_nsteps = a.d_espect = a.d_espect_escape = p
    a.d_dsum = a.d_remain = p
    a.estep = 10_000_000  # 100001 rows of partial sums exceed the 4 MiB scratch
    assert _fn()(C.byref(a)) == ETOOBIG
    a.estep, a.nbins = 100, 5000
    assert _fn()(C.byref(a)) == EINVAL
    a.estep, a.nt_out, a.nbins = 600_000, 600_000, 4000  # 2.4e9 spectrum entries: past 32-bit indexing
    assert _fn()(C.byref(a)) == EINVAL
    a.estep, a.nt_out = 100, 1
    a.nbins, a.system_type = 200, tp.SYS_PIC  # no grid
    assert _fn()(C.byref(a)) == EINVAL
    a.nx = a.ny = a.nz = 2
    a.d_grid = p + 16  # a node is one 32-byte load: the grid must be 32-byte aligned
    assert _fn()(C.byref(a)) == EINVAL
    a.d_grid = p
    a.d_status = p + 2  # a status word must be 4-byte aligned
    assert _fn()(C.byref(a)) == EINVAL
    torch.cuda.synchronize()
