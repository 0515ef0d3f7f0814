"""Speed of the oracle port against the reference compiled from its own
sources (oracle/_ref), on the same host cores and the same inputs: the
headline workload's 512^3 gridded field (synthesised on the CPU), a bounded
sample of its particles, the reference's fixed-step tracking loop with its
diagnostics (particle_tracking_fixed_time_step, OpenMP).

The GPU host has neither the reference tree nor this machine's objects, so
the timed CPU baseline there is the port; this recipe, run where oracle/_ref
builds, measures how the port's speed compares with the reference's own.

    python oracle/compare_ref_speed.py [--nptl N] [--steps S] [--threads T]
"""
import argparse
import ctypes as C
import json
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

from oracle import pyoracle as po  # noqa: E402


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--nptl", type=int, default=16384)
    ap.add_argument("--steps", type=int, default=500)
    ap.add_argument("--threads", type=int, default=os.cpu_count() or 1)
    ap.add_argument("--grid", type=int, default=512)
    a = ap.parse_args()
    import test_particle_gb300.workloads as wl
    po.build_oracle()
    if po.build_ref() is None:
        print(json.dumps({"error": "oracle/_ref not built (reference tree absent)"}))
        return 1
    os.environ["OMP_NUM_THREADS"] = str(a.threads)
    cfg = wl.config_grid(nptl=a.nptl, steps=a.steps, n=a.grid)
    n = cfg["n"]
    mb = wl.kolmogorov_modes(cfg["nmodes"], cfg["kmin"], cfg["kmax"], cfg["dB"], cfg["seed"])
    mv = wl.kolmogorov_modes(cfg["nmodes"], cfg["kmin"], cfg["kmax"], cfg["v_rms"], cfg["seed"] + 1000)
    he, hb = po.synth_pic_fields(mb, mv, 1.0, n, n, n, nthreads=a.threads)
    dom = po.Domain()
    dom.xmin, dom.ymin, dom.zmin = cfg["lo"]
    dom.xmax, dom.ymax, dom.zmax = cfg["hi"]
    dom.xmin_ptl, dom.ymin_ptl, dom.zmin_ptl = cfg["lo"]
    dom.xmax_ptl, dom.ymax_ptl, dom.zmax_ptl = cfg["hi"]
    dt = cfg["dt"]
    dom.tmax = a.steps * dt + 0.5 * dt
    grd = po.Grids()
    grd.nx = grd.ny = grd.nz = n
    grd.nt = 1
    grd.dx = grd.dy = grd.dz = cfg["dx"]
    p0 = wl.shell_particles(a.nptl, cfg["speed"], cfg["lo"], cfg["hi"], 99)
    nt_out, nbins = 2, cfg["nbins"]

    # the reference's own loop
    lib = C.CDLL(po.LIB_REF)
    lib.refh_set_abc(C.c_double(1.0), C.c_double(0.0), C.c_double(0.0))
    lib.refh_setup(C.c_int(4), C.c_double(1.0), C.c_int(0), C.byref(dom), C.byref(grd), C.c_int(0), C.c_int(4))
    lib.refh_set_pic_grids(po.ptr(he), po.ptr(hb), None, None, None, None)
    lib.refh_set_spectrum(C.c_int(nbins), C.c_double(cfg["emin"]), C.c_double(cfg["emax"]))
    pr0, pr = p0.copy(), p0.copy()
    nst = np.zeros(a.nptl, dtype=np.int32)
    esp, ese = np.zeros(nt_out * nbins), np.zeros(nt_out * nbins)
    t0 = time.perf_counter()
    lib.refh_track_fixed(C.c_int(a.nptl), C.c_double(dt), C.c_int(nbins), C.c_int(nt_out), po.ptr(pr0),
                         po.ptr(pr), po.ptr(nst), po.ptr(esp), po.ptr(ese))
    t_ref = time.perf_counter() - t0

    # the port
    f = po.make_field(system_type=4, charge_mass=1.0, bc_flag=0, dom=dom, grd=grd, egrid=he, bgrid=hb)
    s = po.spectrum(nbins, cfg["emin"], cfg["emax"])
    t0 = time.perf_counter()
    out = po.track_fixed(f, s, p0, dt, nt_out, nthreads=a.threads)
    t_port = time.perf_counter() - t0
    same = all(np.array_equal(out["ptl"][k], pr[k]) for k in ("x", "y", "z", "ux", "uy", "uz"))
    pushes = a.nptl * a.steps
    print(json.dumps({"grid": n, "particles": a.nptl, "steps": a.steps, "threads": a.threads,
                      "reference_pushes_per_s": pushes / t_ref, "port_pushes_per_s": pushes / t_port,
                      "port_over_reference": t_ref / t_port, "identical_particles": bool(same),
                      "identical_spectra": bool(np.array_equal(out["espect"].ravel(), esp))}))
    return 0


if __name__ == "__main__":
    sys.exit(main())
