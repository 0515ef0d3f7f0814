"""Generate the golden fixtures in tests/golden from the reference itself.

The reference has no tests and no golden vectors of its own, so its outputs
are produced here by running the reference's own C sources, compiled where
they lie by oracle/build_ref.sh into oracle/_ref/libtpref.so, on seeded
inputs.  The fixtures pin both the oracle restatement (CPU tests) and the CUDA
path (GPU tests), which cannot see the reference tree at run time.

Run from the repository root in a container that has the reference tree:
    python tests/golden/make_golden.py
The reference runs single-threaded (OMP_NUM_THREADS=1) so that its
diffusion-coefficient sums are accumulated in particle order.
"""
import ctypes as C
import hashlib
import json
import multiprocessing as mp
import os
import sys

os.environ["OMP_NUM_THREADS"] = "1"
HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

from oracle import pyoracle as po  # noqa: E402

PD = po.PARTICLE_DTYPE


def ref_lib():
    lib = C.CDLL(po.LIB_REF)
    return lib


def p(a):
    return C.c_void_p(a.ctypes.data) if a is not None else None


# ---------------------------------------------------------------- scenarios
def domain(lo, hi, tmax):
    d = po.Domain()
    d.xmin_ptl, d.xmax_ptl, d.ymin_ptl, d.ymax_ptl, d.zmin_ptl, d.zmax_ptl = (
        lo[0], hi[0], lo[1], hi[1], lo[2], hi[2])
    d.xmin, d.xmax, d.ymin, d.ymax, d.zmin, d.zmax = lo[0], hi[0], lo[1], hi[1], lo[2], hi[2]
    d.tmin, d.tmax = 0.0, tmax
    return d


def grid_for(d, n, nt=1, tmax=1.0):
    g = po.Grids()
    g.nx, g.ny, g.nz = n
    g.nt = nt
    g.dx = (d.xmax - d.xmin) / (n[0] - 1.0)
    g.dy = (d.ymax - d.ymin) / (n[1] - 1.0)
    g.dz = (d.zmax - d.zmin) / (n[2] - 1.0)
    g.dt = (tmax - 0.0) / (nt - 1.0) if nt > 1 else 0.0
    return g


def wlcs_rec(cur_wr, wr, theta, phi, t0, cur_lp, r_lp, lp, alpha, beta, omega):
    w = po.Wlcs()
    w.cur_wr, (w.x_wr, w.y_wr, w.z_wr) = cur_wr, wr
    w.costheta_wr, w.sintheta_wr = np.cos(theta), np.sin(theta)
    w.cosphi_wr, w.sinphi_wr = np.cos(phi), np.sin(phi)
    w.t0, w.cur_lp, w.r_lp = t0, cur_lp, r_lp
    w.x_lp, w.y_lp, w.z_lp = lp
    w.cosalpha_lp, w.sinalpha_lp = np.cos(alpha), np.sin(alpha)
    w.cosbeta_lp, w.sinbeta_lp = np.cos(beta), np.sin(beta)
    w.omega = omega
    return w


def wl_to_array(wl):
    return np.array([[getattr(w, n) for n, _ in po.Wlcs._fields_] for w in wl])


def scenarios():
    """Field scenarios shared by the fixture generator and the tests."""
    rng = np.random.default_rng(20261203)
    sc = {}
    d01 = domain((0, 0, 0), (1, 1, 1), 100.0)
    sc["test"] = dict(system_type=0, charge_mass=1.0, dom=d01, grd=po.Grids(), mt=0)
    # ABC with a gridded double velocity (E = -v x B), reference A,B,C
    g8 = grid_for(d01, (8, 7, 6))
    v = rng.normal(0, 0.05, size=(6 * 7 * 8, 3))
    sc["ff_vel"] = dict(system_type=2, charge_mass=1.0, dom=d01, grd=g8, mt=0,
                        abc=(1.0, np.sqrt(2.0 / 3.0), np.sqrt(1.0 / 3.0)), B0=1.3,
                        lambda0=2 * np.pi, vgrid_d=v)
    # ABC A=B=C=1, lambda = 2 pi, zero velocity grid (the C1 benchmark field)
    sc["abc111"] = dict(system_type=2, charge_mass=1.0, dom=d01, grd=g8, mt=0,
                        abc=(1.0, 1.0, 1.0), B0=1.0, lambda0=2 * np.pi,
                        vgrid_d=np.zeros((6 * 7 * 8, 3)))
    # MHD: float v and B grids
    dm = domain((0, 0, 0), (2.0, 1.5, 1.0), 50.0)
    gm = grid_for(dm, (9, 7, 5))
    nn = 9 * 7 * 5
    sc["mhd"] = dict(system_type=3, charge_mass=1.0, dom=dm, grd=gm, mt=0,
                     vgrid_f=rng.normal(0, 0.05, (nn, 3)).astype(np.float32),
                     bgrid=(rng.normal(0, 0.3, (nn, 3)) + [0, 0, 1]).astype(np.float32))
    # PIC: float E and B grids, single frame
    dp = domain((0, 0, 0), (3.0, 2.0, 2.5), 50.0)
    gp = grid_for(dp, (11, 9, 10))
    npn = 11 * 9 * 10
    sc["pic"] = dict(system_type=4, charge_mass=-1.0, dom=dp, grd=gp, mt=0,
                     egrid=rng.normal(0, 0.05, (npn, 3)).astype(np.float32),
                     bgrid=(rng.normal(0, 0.4, (npn, 3)) + [0, 0, 1]).astype(np.float32))
    # PIC with two time frames blended linearly in time
    gp2 = grid_for(dp, (11, 9, 10), nt=3, tmax=4.0)
    sc["pic_mt"] = dict(system_type=4, charge_mass=-1.0, dom=dp, grd=gp2, mt=1,
                        egrid_ab=(rng.normal(0, 0.05, (npn, 3)).astype(np.float32),
                                  rng.normal(0, 0.05, (npn, 3)).astype(np.float32)),
                        bgrid_ab=((rng.normal(0, 0.4, (npn, 3)) + [0, 0, 1]).astype(np.float32),
                                  (rng.normal(0, 0.4, (npn, 3)) + [0, 0, 1]).astype(np.float32)))
    # PIC on a domain that does not start at 0 (pins the wrap branch's xmin = 0 assumption)
    dq = domain((-1.0, 0.5, -2.0), (2.0, 2.5, 0.5), 50.0)
    gq = grid_for(dq, (11, 9, 10))
    sc["pic_off"] = dict(system_type=4, charge_mass=1.0, dom=dq, grd=gq, mt=0,
                         egrid=rng.normal(0, 0.05, (npn, 3)).astype(np.float32),
                         bgrid=(rng.normal(0, 0.4, (npn, 3)) + [0, 0, 1]).astype(np.float32))
    # Wire-loop current systems: two systems with Euler angles, static wire
    dw = domain((0, 0, 0), (1, 1, 1), 100.0)
    wl = [wlcs_rec(0.3, (0.4, 0.5, 0.45), 0.3, 0.7, 0.0, 1.0, 0.25, (0.5, 0.45, 0.5), 0.4, 1.1, 0.001),
          wlcs_rec(-0.2, (0.6, 0.3, 0.5), 1.2, -0.4, 0.0, 0.5, 0.15, (0.35, 0.6, 0.55), -0.8, 0.3, 0.001)]
    sc["wlcs"] = dict(system_type=1, charge_mass=9.58e3, dom=dw, grd=po.Grids(), mt=0,
                      wl=wl, ibessel=0)
    # the benchmark loop: radius 1, current 1, no wire, centred, no rotation
    wl5 = [wlcs_rec(0.0, (0.0, 0.0, 0.0), 0.0, 0.0, 0.0, 1.0, 1.0, (0.0, 0.0, 0.0), 0.0, 0.0, 0.001)]
    d5 = domain((-3, -3, -3), (3, 3, 3), 100.0)
    sc["loop"] = dict(system_type=1, charge_mass=9.58e3, dom=d5, grd=po.Grids(), mt=0,
                      wl=wl5, ibessel=0)
    return sc


def field_from(sc, bc_flag=0, interp_corrected=0, ellint_corrected=0):
    kw = dict(system_type=sc["system_type"], charge_mass=sc["charge_mass"], bc_flag=bc_flag,
              dom=sc["dom"], grd=sc["grd"], multi_tframe=sc["mt"],
              interp_corrected=interp_corrected, ellint_corrected=ellint_corrected)
    for k in ("abc", "B0", "lambda0", "vgrid_d", "vgrid_f", "bgrid", "egrid", "wl", "ibessel"):
        if k in sc:
            kw[k] = sc[k]
    if "egrid_ab" in sc:
        kw["egrid_ab"] = sc["egrid_ab"]
        kw["bgrid_ab"] = sc["bgrid_ab"]
    return po.make_field(**kw)


def ref_setup(lib, sc, bc_flag=0):
    keep = []
    lib.refh_set_abc(C.c_double(sc.get("abc", (1.0, 0.0, 0.0))[0]),
                     C.c_double(sc.get("abc", (1.0, 0.0, 0.0))[1]),
                     C.c_double(sc.get("abc", (1.0, 0.0, 0.0))[2]))
    vdt = 8 if sc["system_type"] == 2 else 4
    lib.refh_setup(C.c_int(sc["system_type"]), C.c_double(sc["charge_mass"]), C.c_int(bc_flag),
                   C.byref(sc["dom"]), C.byref(sc["grd"]), C.c_int(sc["mt"]), C.c_int(vdt))
    lib.refh_set_ff(C.c_double(sc.get("B0", 1.0)), C.c_double(sc.get("lambda0", 1.0)))

    def arr(a):
        if a is None:
            return None
        a = np.ascontiguousarray(a)
        keep.append(a)
        return p(a)
    if "egrid" in sc or "egrid_ab" in sc or "bgrid" in sc:
        ea, eb = sc.get("egrid_ab", (None, None))
        ba, bb = sc.get("bgrid_ab", (None, None))
        lib.refh_set_pic_grids(arr(sc.get("egrid")), arr(sc.get("bgrid")), arr(ea), arr(eb),
                               arr(ba), arr(bb))
    lib.refh_set_velocity(arr(sc.get("vgrid_d")), None, None, arr(sc.get("vgrid_f")))
    if "wl" in sc:
        wl = (po.Wlcs * len(sc["wl"]))(*sc["wl"])
        keep.append(wl)
        lib.refh_set_wlcs(C.c_int(len(sc["wl"])), wl, C.c_int(sc["ibessel"]))
    return keep


def sample_points(sc, rng, n, outside=0.1):
    d = sc["dom"]
    lo = np.array([d.xmin, d.ymin, d.zmin])
    hi = np.array([d.xmax, d.ymax, d.zmax])
    span = hi - lo
    pts = lo + rng.uniform(-outside, 1 + outside, size=(n, 3)) * span
    if sc["system_type"] in (2, 3, 4):
        # keep clear of the exact upper faces, where the reference indexes past the grid
        pts = np.where(np.isclose(pts, hi), hi - 1e-9, pts)
    t = rng.uniform(0, 3.0, size=(n, 1))
    return np.hstack([pts, t])


def particles_for(sc, rng, n, speed=0.7, region=(0.0, 1.0), qm=None):
    d = sc["dom"]
    lo = np.array([d.xmin, d.ymin, d.zmin])
    hi = np.array([d.xmax, d.ymax, d.zmax])
    pos = lo + rng.uniform(region[0], region[1], size=(n, 3)) * (hi - lo)
    u = speed / np.sqrt(1 - speed ** 2)
    mu = rng.uniform(-1, 1, n)
    ph = rng.uniform(0, 2 * np.pi, n)
    s = np.sqrt(1 - mu ** 2)
    out = np.zeros(n, dtype=PD)
    out["x"], out["y"], out["z"] = pos.T
    out["qm"] = sc["charge_mass"] if qm is None else qm
    out["ux"], out["uy"], out["uz"] = u * s * np.cos(ph), u * s * np.sin(ph), u * mu
    return out


def ref_track(lib, sc, ptl0, dt, nbins, nt_out, emin, emax, bc_flag):
    keep = ref_setup(lib, sc, bc_flag)
    lib.refh_set_spectrum(C.c_int(nbins), C.c_double(emin), C.c_double(emax))
    p0 = ptl0.copy()
    pp = ptl0.copy()
    n = len(pp)
    nst = np.zeros(n, dtype=np.int32)
    esp = np.zeros(nt_out * nbins)
    ese = np.zeros(nt_out * nbins)
    lib.refh_track_fixed(C.c_int(n), C.c_double(dt), C.c_int(nbins), C.c_int(nt_out), p(p0), p(pp),
                         p(nst), p(esp), p(ese))
    estep = int(sc["dom"].tmax / dt)
    nsdc = estep // 100 + 1
    dsum = np.zeros(8 * nsdc)
    rem = np.zeros(nsdc, dtype=np.int32)
    got = lib.refh_captured_dcoeffs(p(dsum), p(rem), C.c_int(nsdc))
    assert got == nsdc
    del keep
    return dict(ptl=pp, nsteps=nst, espect=esp.reshape(nt_out, nbins),
                espect_escape=ese.reshape(nt_out, nbins), dsum=dsum.reshape(8, nsdc), remain=rem)


def _bs_worker(args):
    """One particle per fresh process: the reference stepper keeps static state."""
    name, y0, t0, h0, nsteps = args
    lib = C.CDLL(po.LIB_REF)
    sc = scenarios()[name]
    keep = ref_setup(lib, sc, 2)
    y = np.array(y0, dtype=np.float64)
    out = np.zeros((nsteps, 8))
    lib.refh_bs_integrate(p(y), C.c_double(t0), C.c_double(h0), C.c_int(nsteps), p(out))
    del keep
    return out


def source_digest():
    """Digest of the reference sources the fixtures came from (the tree that
    oracle/build_ref.sh compiled, or $TP_REFERENCE_DIR)."""
    ref_dir = po.reference_dir()
    h = hashlib.sha256()
    for sub in ("src", "src/unused", "include"):
        dd = os.path.join(ref_dir, sub)
        for fn in sorted(os.listdir(dd)):
            fp = os.path.join(dd, fn)
            if os.path.isfile(fp):
                h.update(fn.encode())
                with open(fp, "rb") as f:
                    h.update(f.read())
    return h.hexdigest()


def traj_fixture(lib, sc):
    """Trajectory diagnostics (particle_tracking_fixed_time_step with
    traj_diagnose = 1): records every nsteps_output steps into ptl_time at
    each particle's offset, the initial state first (src/diagnostics.c:541-551,
    src/tracking.c:436-447)."""
    rng = np.random.default_rng(31)
    out = {}
    for name, n, dt, steps, every in (("pic", 24, 0.05, 160, 16), ("test", 16, 0.05, 120, 10)):
        d = po.Domain.from_buffer_copy(sc[name]["dom"])
        d.tmax = steps * dt + 0.5 * dt
        s = dict(sc[name])
        s["dom"] = d
        keep = ref_setup(lib, s, 0)
        lib.refh_set_spectrum(C.c_int(20), C.c_double(1e-3), C.c_double(1e1))
        p0 = particles_for(s, rng, n)
        pp = p0.copy()
        nst = np.zeros(n, dtype=np.int32)
        npts = np.full(n, steps // every + 1, dtype=np.int32)  # every particle runs all steps
        acc = np.cumsum(npts).astype(np.int32)
        ptl_time = np.zeros(int(acc[-1]), dtype=PD)
        off = np.concatenate([[0], acc[:-1]])
        ptl_time[off] = p0
        lib.refh_track_traj(C.c_int(n), C.c_double(dt), C.c_int(20), C.c_int(2), C.c_int(every), p(acc),
                            p(p0.copy()), p(pp), p(nst), p(ptl_time))
        out[name + "_ptl0"] = p0
        out[name + "_ptl"] = pp
        out[name + "_acc"] = acc
        out[name + "_ptl_time"] = ptl_time
        out[name + "_meta"] = np.array([dt, steps, every, d.tmax])
        del keep
    np.savez_compressed(os.path.join(HERE, "traj.npz"), **out)


def fields_fixture(lib):
    """The reference's binary field readers (read_bfields_binary /
    read_efields_binary, float data, one frame): random .gda component files
    and the scaled {x,y,z} records the reference builds from them."""
    import tempfile
    rng = np.random.default_rng(41)
    nx, ny, nz, ct = 12, 10, 7, 3
    b0, e0 = 0.37, 1.9e-3
    comps = rng.normal(0, 1, size=(6, nz * ny * nx)).astype(np.float32)
    comps *= np.float32(10.0) ** rng.integers(-3, 3, size=comps.shape).astype(np.float32)
    g = po.Grids()
    g.nx, g.ny, g.nz, g.nt = nx, ny, nz, 1
    g.dx = g.dy = g.dz = 1.0
    d = po.Domain()
    d.xmax, d.ymax, d.zmax = nx - 1.0, ny - 1.0, nz - 1.0
    with tempfile.TemporaryDirectory() as tmp:
        for c, name in enumerate(("bx", "by", "bz", "ex", "ey", "ez")):
            comps[c].tofile(os.path.join(tmp, "%s_%d.gda" % (name, ct)))
        out_b = np.zeros(3 * nx * ny * nz, dtype=np.float32)
        out_e = np.zeros(3 * nx * ny * nz, dtype=np.float32)
        lib.refh_read_pic_binary(C.byref(g), C.byref(d), (tmp + "/").encode(), C.c_int(ct), C.c_double(b0),
                                 C.c_double(e0), p(out_b), p(out_e))
    np.savez_compressed(os.path.join(HERE, "fields.npz"), comps=comps, dims=np.array([nx, ny, nz, ct]),
                        scale=np.array([b0, e0]), records_b=out_b, records_e=out_e)


def poincare_fixture(lib, sc):
    """RK4 field-line steps of the reference (next_location,
    src/poincare_map.c:243-290) from seeds in the gridded scenarios, including
    steps that leave the box (periodic wrap of the stage points)."""
    rng = np.random.default_rng(8)
    out = {}
    for name in ("mhd", "pic", "pic_off"):
        keep = ref_setup(lib, sc[name])
        d = sc[name]["dom"]
        lo = np.array([d.xmin, d.ymin, d.zmin])
        hi = np.array([d.xmax, d.ymax, d.zmax])
        seeds = lo + rng.uniform(0, 1, size=(32, 3)) * (hi - lo)
        step = 0.02 * float(np.min(hi - lo))
        traj = np.zeros((32, 40, 3))
        lib.refh_next_location(C.c_int(32), p(seeds), C.c_double(step), C.c_int(40), p(traj))
        out[name + "_seeds"] = seeds
        out[name + "_step"] = step
        out[name + "_traj"] = traj
        del keep
    np.savez_compressed(os.path.join(HERE, "poincare.npz"), **out)


def main():
    if po.build_ref() is None:
        print("reference tree absent; nothing generated")
        return 1
    lib = ref_lib()
    if "--poincare" in sys.argv:  # this fixture alone
        poincare_fixture(lib, scenarios())
        return 0
    if "--traj" in sys.argv:  # this fixture alone
        traj_fixture(lib, scenarios())
        return 0
    if "--fields" in sys.argv:  # this fixture alone
        fields_fixture(lib)
        return 0
    rng = np.random.default_rng(7)
    sc = scenarios()
    meta = {"reference_sources_sha256": source_digest(), "fixtures": {}}

    # 1. get_emf samples per scenario
    emf = {}
    for name in ("test", "ff_vel", "abc111", "mhd", "pic", "pic_mt", "pic_off", "wlcs", "loop"):
        keep = ref_setup(lib, sc[name])
        pts = sample_points(sc[name], rng, 256)
        out = np.zeros((len(pts), 6))
        lib.refh_get_emf(C.c_int(len(pts)), p(pts), p(out))
        emf[name + "_xyzt"] = pts
        emf[name + "_emf"] = out
        del keep
    np.savez_compressed(os.path.join(HERE, "emf.npz"), **emf)

    # 2. trilinear corners / weights (PIC grid, incl. wrap branches)
    keep = ref_setup(lib, sc["pic_off"])
    pts = sample_points(sc["pic_off"], rng, 256, outside=0.03)
    cn = np.zeros((len(pts), 8), dtype=np.int64)
    wt = np.zeros((len(pts), 8))
    lib.refh_trilinear(C.c_int(len(pts)), p(pts), p(cn), p(wt))
    np.savez_compressed(os.path.join(HERE, "trilinear.npz"), xyzt=pts, corners=cn, weights=wt)
    del keep

    # 3. elliptic integrals over the whole m range, incl. interval edges
    ms = np.concatenate([rng.uniform(0, 1, 1500), np.linspace(0, 0.999999, 200),
                         [0.0, 0.1, 0.2, 0.5, 0.8, 0.85, 0.9, 0.95, 0.99, 0.9999]])
    ks = np.sqrt(ms)
    ee = np.zeros_like(ks)
    kk = np.zeros_like(ks)
    lib.refh_ellint(C.c_int(len(ks)), p(ks), p(ee), p(kk))
    np.savez_compressed(os.path.join(HERE, "ellint.npz"), k=ks, E=ee, K=kk)

    # 4. Wirz pushes: 1 step and 40 steps per scenario
    wz = {}
    dts = {"test": 0.05, "ff_vel": 0.02, "abc111": 0.05, "mhd": 0.05, "pic": 0.05,
           "pic_mt": 0.05, "pic_off": 0.05, "wlcs": 2e-5, "loop": 2e-4}
    for name, dt in dts.items():
        keep = ref_setup(lib, sc[name], 0 if name != "wlcs" and name != "loop" else 2)
        ptl = particles_for(sc[name], rng, 64)
        for ns in (1, 40):
            pp = ptl.copy()
            esc = np.zeros(len(pp), dtype=np.int32)
            lib.refh_wirz_steps(C.c_int(len(pp)), p(pp), C.c_double(dt), C.c_int(ns), p(esc))
            wz["%s_in" % name] = ptl
            wz["%s_out%d" % (name, ns)] = pp
        wz["%s_dt" % name] = np.array(dt)
        del keep
    np.savez_compressed(os.path.join(HERE, "wirz.npz"), **wz)

    # 5. energy bins: nbins 200, emin 1e-3, emax 1e2 (gamma - 1), incl. edges
    nb, e0, e1 = 200, 1e-3, 1e2
    lib.refh_set_spectrum(C.c_int(nb), C.c_double(e0), C.c_double(e1))
    ptl = np.zeros(4096, dtype=PD)
    ene = 10 ** rng.uniform(-5, 3, 4096)
    ene[:8] = [0.0, 1e-300, e0, e1, 1e300, 1.0, 10.0, 0.1]
    g = 1 + ene
    u = np.sqrt(np.maximum(g * g - 1, 0))
    ptl["ux"] = u
    bins = np.zeros(len(ptl), dtype=np.int32)
    lib.refh_ptl_energy_bins(C.c_int(len(ptl)), p(ptl), C.c_int(nb), p(bins))
    g5 = np.zeros(5)
    lib.refh_get_spectrum_globals(p(g5))
    np.savez_compressed(os.path.join(HERE, "ebins.npz"), ptl=ptl, bins=bins, nbins=nb,
                        emin=e0, emax=e1, globals=g5)

    # 6. calc_diff_coeff on constructed pairs (ABC with velocity grid)
    keep = ref_setup(lib, sc["ff_vel"])
    pa = particles_for(sc["ff_vel"], rng, 128)
    pb = particles_for(sc["ff_vel"], rng, 128)
    pb["t"] = rng.uniform(0, 10, 128)
    pb["xshift"] = rng.integers(-2, 3, 128) * 1.0
    dc = np.zeros((128, 8))
    lib.refh_calc_diff_coeff(C.c_int(128), p(pa), p(pb), C.c_double(0.01), p(dc))
    np.savez_compressed(os.path.join(HERE, "diffcoeff.npz"), p0=pa, p=pb, dt=0.01, out=dc)
    del keep

    # 7. whole fixed-step runs with fused diagnostics
    runs = {}
    cases = [
        ("test", 0, 0.05, 1000 * 0.05 + 0.025, 48, 10, (0.0, 1.0), 0.7),
        ("abc111", 0, 0.02, 1500 * 0.02 + 0.01, 48, 10, (0.0, 1.0), 0.7),
        ("ff_vel", 0, 0.02, 1200 * 0.02 + 0.01, 48, 6, (0.0, 1.0), 0.5),
        ("pic", 0, 0.05, 800 * 0.05 + 0.025, 48, 8, (0.0, 1.0), 0.6),
        ("mhd", 0, 0.05, 600 * 0.05 + 0.025, 32, 6, (0.0, 1.0), 0.5),
        ("ff_vel", 1, 0.01, 2000 * 0.01 + 0.005, 48, 10, (0.3, 0.7), 0.05),
        ("wlcs", 2, 2e-5, 700 * 2e-5 + 1e-5, 32, 7, (0.2, 0.8), 0.3),
    ]
    for ci, (name, bc, dt, tmax, n, nt_out, region, speed) in enumerate(cases):
        s = dict(sc[name])
        d = po.Domain.from_buffer_copy(s["dom"])
        d.tmax = tmax
        s["dom"] = d
        ptl0 = particles_for(s, rng, n, speed=speed, region=region)
        r = ref_track(lib, s, ptl0, dt, 200, nt_out, 1e-3, 1e2, bc)
        if bc == 1:
            # particles escaping before the first diffusion sample would carry
            # uninitialised per-thread values in the reference; keep such cases out
            assert r["remain"][1] == n, "early escape in bc=1 fixture"
        key = "case%d" % ci
        runs[key + "_meta"] = np.array(json.dumps(dict(name=name, bc=bc, dt=dt, tmax=tmax,
                                                       nt_out=nt_out, nbins=200, emin=1e-3,
                                                       emax=1e2)))
        runs[key + "_ptl0"] = ptl0
        for k2, v2 in r.items():
            runs[key + "_" + k2] = v2
    np.savez_compressed(os.path.join(HERE, "track.npz"), **runs)

    # 8. Bulirsch-Stoer steps through the reference stepper (fresh process per particle)
    jobs = []
    lo = sc["loop"]
    for i in range(6):
        r0 = 1.0 + rng.uniform(0.05, 0.3) * np.cos(rng.uniform(0, 2 * np.pi))
        ph = rng.uniform(0, 2 * np.pi)
        zz = rng.uniform(-0.2, 0.2)
        b = rng.uniform(0.1, 0.9)
        mu = rng.uniform(-1, 1)
        q = rng.uniform(0, 2 * np.pi)
        s_ = np.sqrt(1 - mu * mu)
        y0 = [r0 * np.cos(ph), r0 * np.sin(ph), zz, b * s_ * np.cos(q), b * s_ * np.sin(q), b * mu]
        jobs.append(("loop", y0, 0.0, 1e-6, 25))
    with mp.get_context("spawn").Pool(3, maxtasksperchild=1) as pool:
        outs = pool.map_async(_bs_worker, jobs).get(timeout=600)
    np.savez_compressed(os.path.join(HERE, "bs.npz"),
                        y0=np.array([j[1] for j in jobs]), h0=np.array([j[3] for j in jobs]),
                        out=np.array(outs))
    del lo

    # 9. Poincare map field-line steps
    poincare_fixture(lib, sc)
    # 10. trajectory diagnostics
    traj_fixture(lib, sc)
    # 11. binary field files
    fields_fixture(lib)

    meta["fixtures"] = sorted(f for f in os.listdir(HERE) if f.endswith(".npz"))
    with open(os.path.join(HERE, "golden_meta.json"), "w") as f:
        json.dump(meta, f, indent=1)
    print("golden fixtures written:", meta["fixtures"])
    return 0


if __name__ == "__main__":
    sys.exit(main())
