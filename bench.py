"""Benchmark: particle pushes per second on one GB300.

Workload of the headline line: gridded PIC-style fields on a 512^3 periodic
grid (6 FP32 components synthesised from seeded Kolmogorov modes, B0 = 1
along z, dB/B0 = 0.5, E = -v x B from a velocity field of rms 0.1),
trilinear interpolation, 1,048,576 particles per GPU at |v| = 0.7c, 5,000
Wirz steps per run with the fused energy-spectrum (200 bins, 10 frames) and
diffusion-coefficient diagnostics.  One bench step is one such run (5.24e9
pushes).  The field (4.3 GB node-interleaved FP32 plus the 3.2 GB AoS copy)
is far larger than L2, so no L2 flush is needed between steps.

value   the mixed-precision path (FP32 push and field, 64-bit fixed-point
        positions), particles resident in HBM.
e2e     the same through the C ABI with host buffers (particles copied in and
        results copied out every step).
fp64    the FP64 parity path on the same workload (3 or more runs, and its own
        e2e), with the accuracy of the mixed path against it per output frame.
gate    the spectrum-L1 <= 1e-3 / diffusion <= 1 % comparison of the mixed
        path against the FP64 path on an ensemble large enough that two
        independent samples of it differ by less than 1e-3 (2^26 particles).
secondary  the ABC, 512-mode, learned-field and Bulirsch-Stoer workloads.

python bench.py [--gpus N --steps K --warmup W] [--impl reference]
"""
import argparse
import json
import os
import subprocess
import tempfile
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "particle-pushes/s on 1 GB300: FP64 vs mixed+surrogate at stated spectrum error"
UNIT = "pushes/s"
# Per-push counters of track_mixed_kernel<PIC> from one ncu capture of the
# 512^3 headline field (python bench.py --profile mixed512: 1,048,576
# particles x 200 steps): DRAM bytes read + written per push, and thread-level
# instructions per push (smsp__inst_executed x 32 / pushes).  Summary:
# profiles/track_mixed_kernel_pic_512cube_1048576ptl.txt
DRAM_BYTES_PER_PUSH = (20.12e9 + 89.65e6) / 209715200.0
INSTR_PER_PUSH = 3055504469 * 32.0 / 209715200.0
SMS, SCHEDULERS_PER_SM = 152, 4
COEFFS = ["drr", "dxx", "dyy", "dzz", "dpp", "duu", "daa", "dee"]


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class Clocks:
    """nvidia-smi sampling during the timed region (reads settings only)."""

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(prefix="tp_clocks_%d_" % self.device, suffix=".csv")
        os.close(fd)
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), "--query-gpu=index,clocks.sm,clocks.max.sm,"
                 "power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
                 "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
                 "clocks_event_reasons.sw_power_cap", "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.f.close()

    def summary(self):
        try:
            rows = [r.split(",") for r in open(self.path).read().strip().splitlines() if r.strip()]
            sm = [float(r[1]) for r in rows]
            mx = [float(r[2]) for r in rows]
            reasons = set()
            names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
            for r in rows:
                for nm, v in zip(names, r[5:9]):
                    if v.strip().lower() == "active":
                        reasons.add(nm)
            return {"sm_mhz": float(np.median(sm)) if sm else None,
                    "sm_max_mhz": max(mx) if mx else None, "samples": len(rows),
                    "reasons": sorted(reasons)}
        except Exception as e:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "error": str(e)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
        pg = dist
    return world, rank, local, pg


def barrier(pg):
    if pg is not None:
        pg.barrier()


def allmax(pg, v):
    if pg is None:
        return v
    import torch
    t = torch.tensor([float(v)], dtype=torch.float64)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


# ------------------------------------------------------------------ accuracy
def l1_frames(fa, fb):
    """Per output frame, the L1 distance of two spectra each normalised to
    unit sum."""
    return [float(np.abs(a / max(1.0, a.sum()) - b / max(1.0, b.sum())).sum()) for a, b in zip(fa, fb)]


def sampling_floor(frames):
    """Per frame, the expected L1 distance of two independent ensembles of this
    size drawn from the spectrum: sum over bins of sqrt(4 p (1 - p) / (pi N))."""
    out = []
    for fb in frames:
        nb = max(1.0, fb.sum())
        q = fb / nb
        out.append(float(np.sqrt(4 * q * (1 - q) / (np.pi * nb)).sum()))
    return out


def sigma_l1(n):
    """Standard deviation of that L1 distance (Poisson bin counts)."""
    return float(np.sqrt(2.0 * (1.0 - 2.0 / np.pi) / n))


def diffusion_errors(d_fast, d_ref):
    """Relative errors of the diffusion sums, rows 1.. (steps 100, 200, ...),
    per coefficient: the largest over rows and the final row.  Coefficients
    that are rounding noise in the reference run (dee with E = 0) are left
    out."""
    ref = d_ref[:, 1:]
    fast = d_fast[:, 1:]
    scale = np.nanmax(np.abs(ref))
    out = {}
    for c, name in enumerate(COEFFS):
        if np.nanmax(np.abs(ref[c])) <= 1e-12 * scale:
            continue
        rel = np.abs(fast[c] - ref[c]) / np.maximum(np.abs(ref[c]), 1e-300)
        bad = ~np.isfinite(rel)
        # non-finite rows (a NaN sum) are counted, never printed as NaN
        out[name] = {"max_over_rows": float(np.max(rel[~bad])) if (~bad).any() else None,
                     "final_row": float(rel[-1]) if not bad[-1] else None,
                     "nonfinite_rows": int(bad.sum())}
    return out


def worst(dif):
    """The largest relative error over coefficients and rows, inf if any row
    was not finite."""
    if any(v["nonfinite_rows"] for v in dif.values()):
        return float("inf")
    return max(v["max_over_rows"] for v in dif.values())


def fp32_rounded(p0):
    p = p0.copy()
    for c in ("x", "y", "z", "ux", "uy", "uz"):
        p[c] = p[c].astype(np.float32).astype(np.float64)
    return p


# ------------------------------------------------------------------ workloads
def config_dict(cfg):
    """The workload as both arms report it."""
    return {"workload": cfg["name"], "particles_per_gpu": cfg["nptl"], "steps_per_run": cfg["steps"],
            "grid": [cfg["n"]] * 3, "field": "6 FP32 components per node from 512 seeded Kolmogorov "
            "modes, |n| in [1, 64], dB/B0 0.5, v rms 0.1, E = -v x B",
            "dt": cfg["dt"], "nbins": cfg["nbins"], "nt_out": cfg["nt_out"],
            "l2": "inputs larger than L2 (4.3 GB field), no flush",
            "parallelism": "particles sharded, replicas of the field"}


def grid_domain(tp_or_po, cfg):
    dom = tp_or_po.Domain()
    dom.xmin, dom.ymin, dom.zmin = cfg["lo"]
    dom.xmax, dom.ymax, dom.zmax = cfg["hi"]
    dom.xmin_ptl, dom.ymin_ptl, dom.zmin_ptl = cfg["lo"]
    dom.xmax_ptl, dom.ymax_ptl, dom.zmax_ptl = cfg["hi"]
    dom.tmax = cfg["steps"] * cfg["dt"] + 0.5 * cfg["dt"]
    grd = tp_or_po.Grids()
    grd.nx = grd.ny = grd.nz = cfg["n"]
    grd.nt = 1
    grd.dx = grd.dy = grd.dz = cfg["dx"]
    return dom, grd


def setup_grid(tp, wl, cfg, rank, to_host=False):
    dom, grd = grid_domain(tp, cfg)
    tp.configure(system_type=tp.SYS_PIC, charge_mass=1.0, bc_flag=0, dom=dom, grd=grd, mt=0)
    mb = wl.kolmogorov_modes(cfg["nmodes"], cfg["kmin"], cfg["kmax"], cfg["dB"], cfg["seed"])
    mv = wl.kolmogorov_modes(cfg["nmodes"], cfg["kmin"], cfg["kmax"], cfg["v_rms"], cfg["seed"] + 1000)
    he, hb = tp.synth_pic_fields(mb, mv, 1.0, to_host=to_host)
    tp.set_spectrum(cfg["nbins"], cfg["emin"], cfg["emax"])
    p0 = wl.shell_particles(cfg["nptl"], cfg["speed"], cfg["lo"], cfg["hi"], cfg["seed"] + 7 * rank)
    return dom, grd, p0, he, hb


def cpu_sample_runner(cfg, dom, grd, he, hb, cores):
    """run(nptl, nsteps) -> seconds: the oracle (the CPU restatement of the
    reference's FP64 path, pinned bit-exact to it) on `cores` threads, over
    particles of the workload's distribution."""
    from oracle import pyoracle as po
    import test_particle_gb300.workloads as wl
    d = po.Domain.from_buffer_copy(dom)
    g = po.Grids.from_buffer_copy(grd)
    f = po.make_field(system_type=4, charge_mass=1.0, bc_flag=0, dom=d, grd=g, egrid=he, bgrid=hb)
    s = po.spectrum(cfg["nbins"], cfg["emin"], cfg["emax"])
    dt = cfg["dt"]

    def run(nptl, nsteps, seed=99):
        d.tmax = nsteps * dt + 0.5 * dt
        f.dom = d
        p = wl.shell_particles(nptl, cfg["speed"], cfg["lo"], cfg["hi"], cfg["seed"] + seed)
        t0 = time.perf_counter()
        po.track_fixed(f, s, p, dt, 1, nthreads=cores)
        return time.perf_counter() - t0

    return run


def cpu_baseline(cfg, dom, grd, he, hb, target_s=12.0):
    """The oracle on every host core on a bounded sample of the same workload."""
    cores = os.cpu_count() or 1
    run = cpu_sample_runner(cfg, dom, grd, he, hb, cores)
    n_cal, s_cal = 4 * cores * 64, 200
    rate = n_cal * s_cal / run(n_cal, s_cal)
    nsteps = 1000
    nptl = int(max(cores * 64, min(cfg["nptl"], rate * target_s / nsteps)))
    t = run(nptl, nsteps)
    return {"value": nptl * nsteps / t, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": "%d particles x %d steps of the same field and dt (oracle FP64, OpenMP %d threads)"
                      % (nptl, nsteps, cores), "seconds": t}


def reference_arm(args, world, rank):
    """The reference's own CPU implementation of the path, on the host cores:
    the oracle restatement of the reference's FP64 tracking loop (pinned
    bit-exact to the reference compiled from its sources), with the
    workload's gridded field synthesised on the CPU.  No GPU code runs."""
    if rank != 0:
        return
    from oracle import pyoracle as po
    import test_particle_gb300.workloads as wl
    po.build_oracle()
    cfg = wl.config_grid()
    cores = os.cpu_count() or 1
    n = cfg["n"]
    t0 = time.perf_counter()
    mb = wl.kolmogorov_modes(cfg["nmodes"], cfg["kmin"], cfg["kmax"], cfg["dB"], cfg["seed"])
    mv = wl.kolmogorov_modes(cfg["nmodes"], cfg["kmin"], cfg["kmax"], cfg["v_rms"], cfg["seed"] + 1000)
    he, hb = po.synth_pic_fields(mb, mv, 1.0, n, n, n, nthreads=cores)
    synth_s = time.perf_counter() - t0
    dom, grd = grid_domain(po, cfg)
    run = cpu_sample_runner(cfg, dom, grd, he, hb, cores)
    # one calibration, then every step a sample of about step_s seconds
    n_cal, s_cal = 2 * cores * 64, 100
    rate = n_cal * s_cal / run(n_cal, s_cal)
    steps_sample = 500
    step_s = max(1.0, min(6.0, 90.0 / max(1, args.steps)))
    nptl = int(max(cores * 32, min(cfg["nptl"], rate * step_s / steps_sample)))
    for w in range(args.warmup):
        run(cores * 16, 50, seed=200 + w)
    times = [run(nptl, steps_sample, seed=300 + k) for k in range(max(1, args.steps))]
    total = float(np.sum(times))
    v = nptl * steps_sample * len(times) / total
    sample = ("%d particles x %d steps per step of the same 512^3 field and dt (the oracle: the reference's "
              "FP64 tracking loop restated in C, OpenMP %d threads; field synthesised on the CPU in %.1f s)"
              % (nptl, steps_sample, cores, synth_s))
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": total / len(times) * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded Kolmogorov fields and particles)", "config": config_dict(cfg),
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------------ headline pieces
def gate_run(tp, wl, cfg, nptl, steps, seed):
    """The accuracy gate of the mixed path: mixed vs FP64 from the same
    initial state on nptl particles over `steps` steps of the headline field,
    a spectrum frame and a diffusion row every 100 steps."""
    dt, nbins = cfg["dt"], cfg["nbins"]
    nt_out = max(1, steps // 100)
    tp.set_tmax(steps * dt + 0.5 * dt)
    p = wl.shell_particles(nptl, cfg["speed"], cfg["lo"], cfg["hi"], seed)
    sess = tp.Session(nptl)
    out = {}
    try:
        res = {}
        for label, code in (("mixed", tp.PREC_MIXED), ("fp64", tp.PREC_FP64)):
            sess.load(p)
            info = sess.track(dt, nt_out, nbins, code)
            res[label] = sess.fetch(nt_out, nbins, info.nsdc, particles=False)
            out[label + "_pushes_per_s"] = info.pushes / info.kernel_ms * 1e3
    finally:
        sess.close()
        del p
    l1 = l1_frames(res["mixed"]["espect"], res["fp64"]["espect"])
    floor = sampling_floor(res["fp64"]["espect"])
    dif = diffusion_errors(res["mixed"]["dsum"], res["fp64"]["dsum"])
    dmax = worst(dif)
    out.update(particles=nptl, steps=steps, frame_steps=[100 * (k + 1) for k in range(nt_out)],
               spectrum_l1_mixed_vs_fp64_per_frame=l1, spectrum_l1_sampling_floor_per_frame=floor,
               l1_sigma=sigma_l1(nptl), diffusion_rel_err_mixed_vs_fp64=dif,
               spectrum_l1_max=max(l1), diffusion_rel_err_max=dmax if np.isfinite(dmax) else None,
               met=bool(max(l1) <= 1e-3 and dmax <= 0.01),
               target="spectrum L1 <= 1e-3 at every frame and diffusion relative error <= 1 % at every "
                      "row, mixed path against the FP64 path on the same particles")
    return out


def cpu_port_rate(field, dom, cfg, nptl, steps, seed=77):
    """pushes/s of the oracle (the reference's FP64 fixed-step loop restated,
    pinned bit-exact to it) on every host core, over a bounded sample of the
    workload's particles."""
    from oracle import pyoracle as po
    import test_particle_gb300.workloads as wl
    cores = os.cpu_count() or 1
    d = po.Domain.from_buffer_copy(dom)
    d.tmax = steps * cfg["dt"] + 0.5 * cfg["dt"]
    field.dom = d
    p = wl.shell_particles(nptl, cfg["speed"], cfg["lo"], cfg["hi"], cfg["seed"] + seed)
    t0 = time.perf_counter()
    po.track_fixed(field, po.spectrum(cfg["nbins"], cfg["emin"], cfg["emax"]), p, cfg["dt"], 1, nthreads=cores)
    sec = time.perf_counter() - t0
    return {"value": nptl * steps / sec, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": "%d particles x %d steps (oracle FP64, OpenMP %d threads)" % (nptl, steps, cores),
            "seconds": sec}


def secondary_abc(tp, wl):
    """C1: the ABC force-free field, 65,536 particles x 10,000 steps."""
    cfg = wl.config_abc()
    dom = tp.Domain()
    dom.xmax = dom.ymax = dom.zmax = 1.0
    dom.tmax = cfg["steps"] * cfg["dt"] + 0.5 * cfg["dt"]
    tp.configure(system_type=tp.SYS_FORCEFREE, dom=dom, abc=(1.0, 1.0, 1.0), B0=1.0, lambda0=2 * np.pi)
    tp.set_spectrum(cfg["nbins"], cfg["emin"], cfg["emax"])
    n, dt, nt = cfg["nptl"], cfg["dt"], cfg["nt_out"]
    p0 = wl.shell_particles(n, cfg["speed"], cfg["lo"], cfg["hi"], cfg["seed"])
    sess = tp.Session(n)
    rates, res = {}, {}
    try:
        for label, code, pp in (("fp64", tp.PREC_FP64, p0), ("fp64fast", tp.PREC_FP64_FAST, p0),
                                ("mixed", tp.PREC_MIXED, p0), ("fp64_from_fp32_start", tp.PREC_FP64,
                                                               fp32_rounded(p0))):
            best = None
            for _ in range(2 if label == "mixed" else 1):
                sess.load(pp)
                info = sess.track(dt, nt, cfg["nbins"], code)
                best = info if best is None or info.kernel_ms < best.kernel_ms else best
            res[label] = sess.fetch(nt, cfg["nbins"], info.nsdc, particles=False)
            if label != "fp64_from_fp32_start":
                rates[label] = best.pushes / best.kernel_ms * 1e3
    finally:
        sess.close()
    pk = compute_peaks(tp)
    roof = {"flops_per_push": ABC_FLOPS_PER_PUSH,
            "flops_note": "the reference's push counted on the oracle (90 add, 154 mul, 12 div; sqrt, sin, cos "
                          "not counted); peaks from the FMA-chain microbenchmark, a multiply-add counting 2",
            "compute_peaks": pk}
    for label, peak in (("fp64", "fp64_tflops"), ("fp64fast", "fp64_tflops"), ("mixed", "fp32_tflops")):
        ach = rates[label] * ABC_FLOPS_PER_PUSH / 1e12
        roof[label] = {"achieved_tflops": ach, "peak": peak, "frac": ach / pk[peak]}
    from oracle import pyoracle as po
    cpu = cpu_port_rate(po.make_field(system_type=2, charge_mass=1.0, bc_flag=0, abc=(1.0, 1.0, 1.0), B0=1.0,
                                      lambda0=2 * np.pi), dom, cfg, 65536, 1000)
    return {"workload": cfg["name"], "pushes_per_s": rates, "roofline": roof, "cpu_baseline": cpu,
            "mixed_over_cpu": rates["mixed"] / cpu["value"], "fp64_over_cpu": rates["fp64"] / cpu["value"],
            "mixed_over_fp64": rates["mixed"] / rates["fp64"],
            "accuracy_vs_fp64": {
                "particles": n, "steps": cfg["steps"],
                "spectrum_l1_mixed_per_frame": l1_frames(res["mixed"]["espect"], res["fp64"]["espect"]),
                "diffusion_rel_err_mixed": diffusion_errors(res["mixed"]["dsum"], res["fp64"]["dsum"]),
                "diffusion_rel_err_fp64_from_fp32_start": diffusion_errors(res["fp64_from_fp32_start"]["dsum"],
                                                                           res["fp64"]["dsum"])}}


def secondary_modesum(tp, wl, args):
    """C3: 512 plane waves, |n| in [1, 64], dB/B0 = 1; C4: the learned field of
    it.  Rates: mixed on 4,194,304 particles x 1,000 steps, FP64 on 1,048,576
    x 200 steps, the learned field on 16,777,216 x 100 steps.  Accuracy on
    1,048,576 particles x 200 steps against the FP64 exact sum, with the FP64
    run from the FP32-rounded start as the chaos floor."""
    cfg = wl.config_modesum()
    dom = tp.Domain()
    dom.xmax = dom.ymax = dom.zmax = 1.0
    modes = wl.kolmogorov_modes(cfg["nmodes"], cfg["kmin"], cfg["kmax"], cfg["dB"], cfg["seed"], va=cfg["va"])
    tp.configure(system_type=tp.SYS_MODESUM, dom=dom, modes=modes, mode_B0=cfg["B0"])
    tp.set_spectrum(cfg["nbins"], cfg["emin"], cfg["emax"])
    dt, nbins = cfg["dt"], cfg["nbins"]
    c3 = {"workload": cfg["name"], "pushes_per_s": {}}
    c4 = {"workload": "surrogate_of_" + cfg["name"].replace("4194304ptl", "16777216ptl"),
          "pushes_per_s": {}}

    def rate(n, steps, code, seed=0, fetch=False):
        tp.set_tmax(steps * dt + 0.5 * dt)
        p = wl.shell_particles(n, cfg["speed"], cfg["lo"], cfg["hi"], cfg["seed"] + seed)
        s = tp.Session(n)
        try:
            s.load(p)
            info = s.track(dt, max(1, steps // 100), nbins, code)
            r = s.fetch(max(1, steps // 100), nbins, info.nsdc, particles=False) if fetch else None
        finally:
            s.close()
        return info.pushes / info.kernel_ms * 1e3, r

    c3["pushes_per_s"]["mixed"] = rate(4194304, 1000, tp.PREC_MIXED)[0]
    na, sa = 1048576, 200
    pa = wl.shell_particles(na, cfg["speed"], cfg["lo"], cfg["hi"], cfg["seed"] + 1)
    tp.set_tmax(sa * dt + 0.5 * dt)
    runs = {}
    s = tp.Session(na)
    try:
        for label, code, pp in (("fp64", tp.PREC_FP64, pa), ("mixed", tp.PREC_MIXED, pa),
                                ("fp64_from_fp32_start", tp.PREC_FP64, fp32_rounded(pa))):
            s.load(pp)
            info = s.track(dt, 2, nbins, code)
            runs[label] = s.fetch(2, nbins, info.nsdc, particles=False)
            if label == "fp64":
                c3["pushes_per_s"]["fp64"] = info.pushes / info.kernel_ms * 1e3
    finally:
        s.close()
    c3["mixed_over_fp64"] = c3["pushes_per_s"]["mixed"] / c3["pushes_per_s"]["fp64"]
    from oracle import pyoracle as po
    c3["cpu_baseline"] = cpu_port_rate(po.make_field(system_type=5, charge_mass=1.0, bc_flag=0, modes=modes,
                                                     B0=cfg["B0"]), dom, cfg, 4096, 50)
    c3["mixed_over_cpu"] = c3["pushes_per_s"]["mixed"] / c3["cpu_baseline"]["value"]
    pk = compute_peaks(tp)
    flops = 2 * cfg["nmodes"] * 18  # per push: 2 evaluations x 512 modes x ~18 flops (+ one cosine per mode)
    c3["roofline"] = {"flops_per_push": flops, "compute_peaks": pk,
                      "flops_note": "2 evaluations x modes x 18 (the phase, the cosine's argument, 6 amplitude "
                                    "products and sums); the cosine not counted",
                      "mixed": {"achieved_tflops": c3["pushes_per_s"]["mixed"] * flops / 1e12,
                                "frac_fp32": c3["pushes_per_s"]["mixed"] * flops / 1e12 / pk["fp32_tflops"]},
                      "fp64": {"achieved_tflops": c3["pushes_per_s"]["fp64"] * flops / 1e12,
                               "frac_fp64": c3["pushes_per_s"]["fp64"] * flops / 1e12 / pk["fp64_tflops"]}}
    acc = {"particles": na, "steps": sa, "frame_steps": [100, 200],
           "spectrum_l1_mixed_per_frame": l1_frames(runs["mixed"]["espect"], runs["fp64"]["espect"]),
           "spectrum_l1_fp64_from_fp32_start_per_frame": l1_frames(runs["fp64_from_fp32_start"]["espect"],
                                                                    runs["fp64"]["espect"]),
           "spectrum_l1_sampling_floor_per_frame": sampling_floor(runs["fp64"]["espect"]),
           "diffusion_rel_err_mixed": diffusion_errors(runs["mixed"]["dsum"], runs["fp64"]["dsum"]),
           "diffusion_rel_err_fp64_from_fp32_start": diffusion_errors(runs["fp64_from_fp32_start"]["dsum"],
                                                                      runs["fp64"]["dsum"])}
    c3["accuracy_vs_fp64"] = acc
    # C4: train the learned field of this table, then track with it
    try:
        train = train_surrogate(tp, modes, cfg, args)
        c4["train"] = train
        c4["pushes_per_s"]["surrogate"] = rate(16777216, 100, tp.PREC_SURROGATE)[0]
        c4["pushes_per_s"]["fp64_exact_sum"] = c3["pushes_per_s"]["fp64"]
        c4["surrogate_over_fp64"] = c4["pushes_per_s"]["surrogate"] / c3["pushes_per_s"]["fp64"]
        c4["cpu_baseline"] = dict(c3["cpu_baseline"], note="the exact mode sum on the CPU, as for C3")
        c4["surrogate_over_cpu"] = c4["pushes_per_s"]["surrogate"] / c3["cpu_baseline"]["value"]
        c4["surrogate_over_mixed_exact_sum"] = c4["pushes_per_s"]["surrogate"] / c3["pushes_per_s"]["mixed"]
        tp.set_tmax(sa * dt + 0.5 * dt)
        s = tp.Session(na)
        try:
            s.load(pa)
            info = s.track(dt, 2, nbins, tp.PREC_SURROGATE)
            rs = s.fetch(2, nbins, info.nsdc, particles=False)
        finally:
            s.close()
        c4["accuracy_vs_fp64_exact_sum"] = {
            "particles": na, "steps": sa,
            "spectrum_l1_surrogate_per_frame": l1_frames(rs["espect"], runs["fp64"]["espect"]),
            "diffusion_rel_err_surrogate": diffusion_errors(rs["dsum"], runs["fp64"]["dsum"])}
        c4["gain_4096_modes"] = surrogate_gain(tp, wl, cfg, args, dom)
    except Exception as e:  # the C3 figures stand without it
        c4["error"] = str(e)
    return c3, c4


def field_errors(tp, B0, model=None, exact=None):
    """Relative RMS errors of dB and E against the current (exact) field on
    65,536 fixed points; model None: the tensor-core model's field."""
    rng = np.random.default_rng(5)
    u = rng.integers(0, 2 ** 32, size=(65536, 3), dtype=np.uint64).astype(np.uint32)
    xyzt = np.zeros((len(u), 4))
    xyzt[:, :3] = u / 2 ** 32
    ex = tp.get_emf(xyzt) if exact is None else exact
    md = tp.mlp_eval_kernel(u) if model is None else model
    dB = ex[:, :3] - [0, 0, B0]
    return (float(np.sqrt(np.mean((md[:, :3] - ex[:, :3]) ** 2) / np.mean(dB ** 2))),
            float(np.sqrt(np.mean((md[:, 3:] - ex[:, 3:]) ** 2) / np.mean(ex[:, 3:] ** 2))), ex, xyzt)


def train_surrogate(tp, modes, cfg, args, samples=16777216):
    """Train the learned field on samples of the exact mode sum (features: the
    64 strongest distinct lattice vectors) and measure its field error on
    fresh points."""
    import test_particle_gb300.workloads as wl
    tp.mlp_init(wl.surrogate_features(modes), seed=3)
    loss, ms = tp.mlp_train(samples, 65536, args.epochs, lr=2e-3)
    eb, ee, _, _ = field_errors(tp, cfg["B0"])
    flop = 3 * 2 * (128 * 256 + 3 * 256 * 256 + 256 * 6) * samples * args.epochs
    return {"samples": samples, "epochs": args.epochs, "final_loss": loss, "train_ms": ms,
            "train_tflops": flop / (ms * 1e-3) / 1e12, "rel_rms_err_dB": eb, "rel_rms_err_E": ee}


def surrogate_gain(tp, wl, cfg, args, dom, nmodes=4096):
    """What the trained model gains over the method without it, on a field of
    nmodes modes with the same spectrum: pushes/s of the model against the
    exact FP32 sum, and, at equal cost, its field error against the exact sum
    truncated to the K strongest modes that run at the model's speed."""
    big = wl.kolmogorov_modes(nmodes, cfg["kmin"], cfg["kmax"], cfg["dB"], cfg["seed"] + 5, va=cfg["va"])
    tp.configure(system_type=tp.SYS_MODESUM, dom=dom, modes=big, mode_B0=cfg["B0"])
    tp.set_spectrum(cfg["nbins"], cfg["emin"], cfg["emax"])
    train = train_surrogate(tp, big, cfg, args)
    dt = cfg["dt"]
    tp.set_tmax(50 * dt + 0.5 * dt)
    p0 = wl.shell_particles(1048576, cfg["speed"], cfg["lo"], cfg["hi"], cfg["seed"] + 6)
    s = tp.Session(len(p0))
    r = {}
    try:
        for label, code in (("exact_fp32_sum", tp.PREC_MIXED), ("model", tp.PREC_SURROGATE)):
            best = None
            for _ in range(2):
                s.load(p0)
                info = s.track(dt, 1, cfg["nbins"], code)
                best = info.kernel_ms if best is None else min(best, info.kernel_ms)
            r[label] = info.pushes / best * 1e3
    finally:
        s.close()
    keq = max(1, int(nmodes * r["exact_fp32_sum"] / r["model"]))
    # the exact sum truncated to the keq strongest modes, measured on the same points
    _, _, exact, xyzt = field_errors(tp, cfg["B0"], model=np.zeros((65536, 6)))
    top = big[np.argsort(-np.linalg.norm(big["amp_b"], axis=1))[:keq]]
    tp.configure(system_type=tp.SYS_MODESUM, dom=dom, modes=top, mode_B0=cfg["B0"])
    eb_t, ee_t, _, _ = field_errors(tp, cfg["B0"], model=tp.get_emf(xyzt), exact=exact)
    return {"modes": nmodes, "train": train, "pushes_per_s": r,
            "model_over_exact_sum": r["model"] / r["exact_fp32_sum"],
            "equal_cost_modes": keq, "truncated_sum_rel_rms_err_dB": eb_t, "truncated_sum_rel_rms_err_E": ee_t,
            "model_more_accurate_at_equal_cost": bool(train["rel_rms_err_dB"] < eb_t)}


def bs_setup(tp):
    dom = tp.Domain()
    for a in ("xmin", "ymin", "zmin"):
        setattr(dom, a, -3.0)
    for a in ("xmax", "ymax", "zmax"):
        setattr(dom, a, 3.0)
    w = tp.Wlcs()
    w.costheta_wr = w.cosphi_wr = w.cosalpha_lp = w.cosbeta_lp = 1.0
    w.cur_lp, w.r_lp, w.omega = 1.0, 1.0, 0.001
    tp.configure(system_type=tp.SYS_WLCS, charge_mass=9.58e3, bc_flag=2, dom=dom, wl=[w])
    tp.set_spectrum(100, 1e-3, 10.0)
    return dom, w


def bs_run(tp, wl, n, t_end=0.05, seed=31):
    """One circular loop (radius 1, current 1, no wire), E = 0; particles on a
    torus around the wire, |v| in [0.1, 0.9] c; the reference's equations
    (beta form, positions in L0, CGS q/m of a proton); rtol = atol = 1e-10."""
    import ctypes as C
    y0 = wl.torus_particles(n, 1.0, 0.05, 0.3, 0.1, 0.9, seed)
    y = y0.copy()
    t = np.zeros(n)
    steps = np.zeros(n, dtype=np.int32)
    st = np.zeros(n, dtype=np.int32)
    esp = np.zeros(10 * 100)
    dfr = np.zeros(8 * 11)
    info = tp.RunInfo()
    tp.check(tp.lib().tp_bs_run(C.c_int(n), tp._ptr(y), tp._ptr(t), C.c_double(t_end), C.c_int(10),
                                C.c_int(100), C.c_double(1e-6), C.c_double(1e-10), C.c_double(1e-10),
                                C.c_int(8), C.c_int(0), C.c_int(1000000), tp._ptr(steps), tp._ptr(st),
                                tp._ptr(esp), tp._ptr(dfr), C.byref(info)), "bs_run")
    return y0, y, steps, st, info


def secondary_bs(tp, wl, cpu=True, n=1048576):
    """C5: adaptive Bulirsch-Stoer, 1,048,576 particles in the wire-loop field
    (n: a smaller case for a profiler capture)."""
    dom, w = bs_setup(tp)
    y0, y, steps, st, info = bs_run(tp, wl, n)
    out = {"workload": "wire_loop_bs_%dptl" % n,
           "accepted_steps_per_s": info.pushes / info.kernel_ms * 1e3, "kernel_ms": info.kernel_ms,
           "t_end": 0.05, "steps_min_median_max": [int(steps.min()), float(np.median(steps)), int(steps.max())],
           "status_nonzero": int((st != 0).sum()),
           "beta_rel_drift_max": float(np.max(np.abs(np.linalg.norm(y[:, 3:], axis=1) /
                                                     np.linalg.norm(y0[:, 3:], axis=1) - 1)))}
    if cpu:
        from oracle import pyoracle as po
        cores = os.cpu_count() or 1
        m = cores * 8
        f = po.make_field(system_type=1, charge_mass=9.58e3, bc_flag=2,
                          dom=po.Domain.from_buffer_copy(dom), wl=[po.Wlcs.from_buffer_copy(w)])
        t0 = time.perf_counter()
        nsteps = po.bs_run_many(f, y0[:m], 1e-6, 100, atol=1e-10, rtol=1e-10, nthreads=cores)
        dtc = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": nsteps / dtc, "unit": "accepted steps/s", "cores": cores,
                               "kind": "port", "sample": "%d particles x 100 steps" % m}
        out["gpu_over_cpu"] = out["accepted_steps_per_s"] / out["cpu_baseline"]["value"]
    return out


# Floating-point operations of one FP64 Wirz push in the ABC field (90 add/sub,
# 154 mul, 12 div; 8 sqrt, 8 sin and 8 cos not counted), counted on the
# oracle's restatement of the reference's push and pinned by
# tests/test_opcount.py.
ABC_FLOPS_PER_PUSH = 90 + 154 + 12
_COMPUTE_PEAKS = {}


def compute_peaks(tp):
    """The CUDA-core FP32, FP64 and packed FP32-pair rates from the library's
    FMA-chain microbenchmark (MEASURED_PEAKS.json holds HBM and tensor-core
    figures only), measured once per process."""
    if not _COMPUTE_PEAKS:
        for k, v in tp.measure_fma_peaks().items():
            _COMPUTE_PEAKS[k + "_tflops"] = v / 1e12
        _COMPUTE_PEAKS["how"] = ("FMA chains, 8 per thread, 32 warps on every SM, CUDA events; a multiply-add "
                                 "counts 2")
    return _COMPUTE_PEAKS


def host_buffer(arr, pinned):
    """A copy of arr in page-locked host memory (a pinned torch buffer viewed
    as numpy), so that the e2e copies run at the link's rate; pageable if
    that is not available.  Appends whether it is page-locked to `pinned`."""
    try:
        import torch
        buf = torch.empty(arr.nbytes, dtype=torch.uint8, pin_memory=True)
        out = buf.numpy().view(arr.dtype).reshape(arr.shape)
        out[...] = arr
        host_buffer.keep.append(buf)
        pinned.append(True)
        return out
    except Exception:
        pinned.append(False)
        return arr.copy()


host_buffer.keep = []


def headline(args, world, rank, local, pg):
    import ctypes as C
    import test_particle_gb300 as tp
    import test_particle_gb300.workloads as wl
    tp.check(tp.lib().tp_init(local), "tp_init")
    cfg = wl.config_grid()
    want_cpu = rank == 0 and world == 1 and not args.no_cpu_baseline
    dom, grd, p0, he, hb = setup_grid(tp, wl, cfg, rank, to_host=want_cpu)
    n = cfg["nptl"]
    sess = tp.Session(n)
    sess.load(p0)
    dt, nt_out, nbins = cfg["dt"], cfg["nt_out"], cfg["nbins"]

    # ---- mixed-precision path, particles resident in HBM; every run starts
    # from the workload's initial particles (reloaded outside the device-timed
    # run, on the device: the same workload each step)
    for _ in range(max(3, args.warmup)):
        sess.load(p0)
        sess.track(dt, nt_out, nbins, tp.PREC_MIXED)
    barrier(pg)
    kms, sms, launches = [], [], 0
    with Clocks(local) as clk:
        for _ in range(args.steps):
            sess.load(p0)
            info = sess.track(dt, nt_out, nbins, tp.PREC_MIXED)
            kms.append(info.kernel_ms)
            sms.append(info.step_ms)
            launches += info.launches
    barrier(pg)
    dev_s = allmax(pg, sum(sms) / 1e3)
    pushes = info.pushes
    value = pushes * args.steps * world / dev_s
    clocks = clk.summary()
    sess.load(p0)
    sess.track(dt, nt_out, nbins, tp.PREC_MIXED)
    diag = sess.fetch(nt_out, nbins, info.nsdc)

    # ---- FP64 parity path on the same workload (fresh particle state each run)
    f64 = []
    for _ in range(max(3, args.fp64_steps)):
        sess.load(p0)
        f64.append(sess.track(dt, nt_out, nbins, tp.PREC_FP64).kernel_ms)
    fp64_value = pushes / (float(np.median(f64)) / 1e3)
    d64 = sess.fetch(nt_out, nbins, info.nsdc)
    # the FP64 path from the initial state rounded to FP32: how far two FP64
    # runs drift apart from one FP32 rounding (the chaos floor)
    sess.load(fp32_rounded(p0))
    sess.track(dt, nt_out, nbins, tp.PREC_FP64)
    d64r = sess.fetch(nt_out, nbins, info.nsdc, particles=False)
    sess.close()

    # ---- e2e: host buffers (page-locked) through the C ABI, copies inside
    # the timed region
    L = tp.lib()
    nsdc = info.nsdc
    pinned = []
    p_in = host_buffer(p0, pinned)
    ptl = host_buffer(p0, pinned)
    esp, ese = host_buffer(np.zeros(nt_out * nbins), pinned), host_buffer(np.zeros(nt_out * nbins), pinned)
    dsum, rem = host_buffer(np.zeros(8 * nsdc), pinned), host_buffer(np.zeros(nsdc, dtype=np.int32), pinned)
    nst = host_buffer(np.zeros(n, dtype=np.int32), pinned)
    ri = tp.RunInfo()

    def e2e_once(prec):
        ptl[...] = p_in  # every run from the workload's initial particles (untimed)
        t1 = time.perf_counter()
        tp.check(L.tp_track_host(C.c_int(prec), C.c_int(n), C.c_double(dt), C.c_int(nt_out),
                                 C.c_int(nbins), tp._ptr(p_in), tp._ptr(ptl), tp._ptr(nst), tp._ptr(esp),
                                 tp._ptr(ese), tp._ptr(dsum), tp._ptr(rem), C.byref(ri)), "e2e")
        return time.perf_counter() - t1

    e2e_once(tp.PREC_MIXED)
    e2e_times = [e2e_once(tp.PREC_MIXED) for _ in range(args.steps)]
    e2e_s = allmax(pg, float(np.median(e2e_times)))
    fp64_e2e_s = allmax(pg, e2e_once(tp.PREC_FP64))
    h2d = 2 * n * 88
    d2h = n * 88 + n * 4 + 2 * nt_out * nbins * 4 + 8 * nsdc * 8 + nsdc * 4

    # ---- roofline of the dominant kernel (physical figures; see DESIGN)
    hbm, peak_kind = peaks()
    kernel_s = float(np.median(kms)) / 1e3
    traffic = DRAM_BYTES_PER_PUSH * pushes
    dram_gbs = traffic / kernel_s / 1e9
    sm_hz = (clocks.get("sm_mhz") or 2070.0) * 1e6
    issue = INSTR_PER_PUSH * pushes / kernel_s / 32.0 / (SMS * SCHEDULERS_PER_SM * sm_hz)

    frames = [int(cfg["steps"] // nt_out * (k + 1)) for k in range(nt_out)]
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": max(3, args.warmup), "ms_per_step": dev_s * 1e3 / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded Kolmogorov fields and particles)",
            "precision": "FP32 push and field, 64-bit fixed-point positions, FP64 diffusion sums",
            "config": config_dict(cfg),
            "e2e": {"value": pushes * world / e2e_s, "unit": UNIT, "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h, "host_memory": "page-locked" if all(pinned) else "pageable"},
            "gpu_launches": launches,
            "clocks": clocks,
            "compute_peaks": compute_peaks(tp),
            "roofline": {"bound": "hbm", "achieved": dram_gbs, "peak": hbm, "unit": "GB/s",
                         "frac": dram_gbs / hbm, "peak_kind": peak_kind, "traffic": traffic,
                         "kernel": "track_mixed_kernel<PIC>",
                         "achieved_is": "DRAM bytes per launch (ncu, per push x pushes) / CUDA-event time",
                         "dram_bytes_per_push": DRAM_BYTES_PER_PUSH,
                         "issue_frac": issue,
                         "issue_note": "%.0f instructions per push (ncu) at the pushes/s above over 152 SMs x "
                                       "4 schedulers at the sampled SM clock" % INSTR_PER_PUSH,
                         "gather_bytes_served_per_push": 384,
                         "gather_gbs_served": pushes * 384.0 / kernel_s / 1e9,
                         "gather_note": "2 evaluations x 8 corners x 6 FP32 components; most are served by "
                                        "the register cell cache, L1 and L2, not DRAM"},
            "fp64": {"value": fp64_value * world, "unit": UNIT, "runs": len(f64),
                     "kernel_ms": [float(v) for v in f64],
                     "e2e": {"value": pushes * world / fp64_e2e_s, "unit": UNIT, "h2d_bytes_per_step": h2d,
                             "d2h_bytes_per_step": d2h},
                     "mixed_over_fp64": value / (fp64_value * world),
                     "frame_steps": frames,
                     "spectrum_l1_mixed_vs_fp64_per_frame": l1_frames(diag["espect"], d64["espect"]),
                     "spectrum_l1_fp64_from_fp32_rounded_start_per_frame": l1_frames(d64r["espect"],
                                                                                       d64["espect"]),
                     "spectrum_l1_sampling_floor_per_frame": sampling_floor(d64["espect"]),
                     "diffusion_rel_err_mixed_vs_fp64": diffusion_errors(diag["dsum"], d64["dsum"]),
                     "diffusion_rel_err_fp64_from_fp32_rounded_start": diffusion_errors(d64r["dsum"],
                                                                                         d64["dsum"])}}
    del diag, d64, d64r

    # ---- the accuracy gate on an ensemble whose sampling floor is below 1e-3
    if rank == 0 and args.gate_nptl > 0:
        try:
            line["gate"] = gate_run(tp, wl, cfg, args.gate_nptl, args.gate_steps, cfg["seed"] + 4242)
        except Exception as e:
            line["gate"] = {"error": str(e)}
        tp.set_tmax(cfg["steps"] * dt + 0.5 * dt)

    # ---- the other workloads
    if rank == 0 and not args.no_secondary:
        sec = {}
        for name, fn in (("C1_abc", lambda: secondary_abc(tp, wl)),
                         ("C3_C4_modesum", lambda: secondary_modesum(tp, wl, args)),
                         ("C5_bs", lambda: secondary_bs(tp, wl))):
            try:
                r = fn()
                if name == "C3_C4_modesum":
                    sec["C3_modesum"], sec["C4_surrogate"] = r
                else:
                    sec[name] = r
            except Exception as e:
                sec[name] = {"error": str(e)}
        line["secondary"] = sec

    if want_cpu:
        try:
            line["cpu_baseline"] = cpu_baseline(cfg, dom, grd, he, hb)
        except Exception as e:
            line["cpu_baseline"] = {"value": None, "error": str(e)}
    return line


# ------------------------------------------------------------------ separate runs
def profile_case(prec):
    """Small case of a tracking kernel, one launch after a warm-up: the
    gridded field (256^3, 0.5 GB interleaved, larger than L2; 131072
    particles, 200 steps) for mixed / fp64 / fp64fast; the headline 512^3
    field with its 1,048,576 particles over 200 steps for mixed512; the
    512-mode field with an untrained learned model (the kernel's work does not
    depend on the weights; 155648 particles = 2 x 304 blocks of 256, 20 steps)
    for surrogate; the mixed kernel on the 512-mode field (155648 particles,
    20 steps) for modesum and on the ABC field (65536 particles, 1000 steps)
    for abc."""
    import test_particle_gb300 as tp
    import test_particle_gb300.workloads as wl
    if prec == "train":
        # one epoch of the learned field's training on 1,048,576 samples of the
        # 512-mode field, batch 65,536 (16 steps)
        tp.check(tp.lib().tp_init(0), "tp_init")
        cfg = wl.config_modesum()
        dom = tp.Domain()
        dom.xmax = dom.ymax = dom.zmax = 1.0
        modes = wl.kolmogorov_modes(cfg["nmodes"], cfg["kmin"], cfg["kmax"], cfg["dB"], cfg["seed"],
                                    va=cfg["va"])
        tp.configure(system_type=tp.SYS_MODESUM, dom=dom, modes=modes, mode_B0=cfg["B0"])
        tp.mlp_init(wl.surrogate_features(modes), seed=3)
        loss, ms = tp.mlp_train(1 << 20, 65536, 1, lr=2e-3)
        flop = 3 * 2 * (128 * 256 + 3 * 256 * 256 + 256 * 6) * (1 << 20)
        print(json.dumps({"profile": "train", "train_ms": ms, "ms_per_batch": ms / 16,
                          "train_tflops": flop / (ms * 1e-3) / 1e12}))
        return
    if prec == "h5":
        # the PIC HDF5 field file of a 256^3 grid written from and read into
        # device memory (tp_save_pic_fields_h5, tp_read_pic_fields_h5): the
        # reorder kernels on 64 MB components
        import ctypes as C
        import shutil
        cfg = wl.config_grid(nptl=1024, steps=1, n=256)
        dom, grd, _, _, _ = setup_grid(tp, wl, cfg, 0)
        L = tp.lib()
        L.set_variables_bfield(C.byref(grd), C.byref(dom), C.c_double(1.0), C.c_int(0), C.c_int(4))
        L.set_variables_efield(C.byref(grd), C.byref(dom), C.c_double(1.0), C.c_int(0), C.c_int(4))
        work = tempfile.mkdtemp(prefix="tp_h5prof_")
        try:
            fn = os.path.join(work, "fields_0.h5")
            t0 = time.perf_counter()
            tp.save_pic_fields_h5(fn, "Timestep_0")
            t1 = time.perf_counter()
            tp.read_pic_fields_h5(fn, "Timestep_0")
            t2 = time.perf_counter()
        finally:
            shutil.rmtree(work, ignore_errors=True)
        print(json.dumps({"profile": "h5", "save_s": t1 - t0, "load_s": t2 - t1}))
        return
    if prec == "abc":
        tp.check(tp.lib().tp_init(0), "tp_init")
        cfg = wl.config_abc(steps=1000)
        dom = tp.Domain()
        dom.xmax = dom.ymax = dom.zmax = 1.0
        dom.tmax = cfg["steps"] * cfg["dt"] + 0.5 * cfg["dt"]
        tp.configure(system_type=tp.SYS_FORCEFREE, dom=dom, abc=(1.0, 1.0, 1.0), B0=1.0,
                     lambda0=2 * np.pi)
        tp.set_spectrum(cfg["nbins"], cfg["emin"], cfg["emax"])
        p0 = wl.shell_particles(cfg["nptl"], cfg["speed"], cfg["lo"], cfg["hi"], cfg["seed"])
    elif prec in ("surrogate", "modesum"):
        tp.check(tp.lib().tp_init(0), "tp_init")
        cfg = wl.config_modesum(nptl=155648, steps=20)
        dom = tp.Domain()
        dom.xmax = dom.ymax = dom.zmax = 1.0
        dom.tmax = cfg["steps"] * cfg["dt"] + 0.5 * cfg["dt"]
        modes = wl.kolmogorov_modes(cfg["nmodes"], cfg["kmin"], cfg["kmax"], cfg["dB"], cfg["seed"],
                                    va=cfg["va"])
        tp.configure(system_type=tp.SYS_MODESUM, dom=dom, modes=modes, mode_B0=cfg["B0"])
        tp.set_spectrum(cfg["nbins"], cfg["emin"], cfg["emax"])
        if prec == "surrogate":
            tp.mlp_init(wl.surrogate_features(modes), seed=3)
            tp.mlp_set_output_norm(np.array([0, 0, 1, 0, 0, 0]), np.ones(6))
        p0 = wl.shell_particles(cfg["nptl"], cfg["speed"], cfg["lo"], cfg["hi"], cfg["seed"])
    elif prec == "mixed512":
        cfg = wl.config_grid(steps=200)
        dom, grd, p0, _, _ = setup_grid(tp, wl, cfg, 0)
        prec = "mixed"
    else:
        cfg = wl.config_grid(nptl=131072, steps=200, n=256)
        dom, grd, p0, _, _ = setup_grid(tp, wl, cfg, 0)
    sess = tp.Session(cfg["nptl"])
    code = {"mixed": tp.PREC_MIXED, "fp64": tp.PREC_FP64, "fp64fast": tp.PREC_FP64_FAST,
            "surrogate": tp.PREC_SURROGATE, "modesum": tp.PREC_MIXED, "abc": tp.PREC_MIXED}[prec]
    sess.load(p0)
    sess.track(cfg["dt"], 2, cfg["nbins"], code)
    sess.load(p0)
    info = sess.track(cfg["dt"], 2, cfg["nbins"], code)
    print(json.dumps({"profile": prec, "kernel_ms": info.kernel_ms, "pushes": info.pushes,
                      "pushes_per_s": info.pushes / info.kernel_ms * 1e3, "grid": info.grid,
                      "blocks_per_sm": info.blocks_per_sm}))
    sess.close()


def open_box(tp, wl, args):
    """Open boundaries: a 128^3 gridded field in an open box that most
    particles leave within the run; one launch against segments with the
    departed particles compacted away (identical results)."""
    n = args.nptl or 262144
    steps = args.run_steps or 4000
    cfg = wl.config_grid(nptl=n, steps=steps, n=128, dx=0.25)
    L = cfg["hi"][0]
    dom = tp.Domain()
    dom.xmax = dom.ymax = dom.zmax = L
    dom.xmax_ptl = dom.ymax_ptl = dom.zmax_ptl = L
    dom.tmax = steps * cfg["dt"] + 0.5 * cfg["dt"]
    grd = tp.Grids()
    grd.nx = grd.ny = grd.nz = 128
    grd.nt = 1
    grd.dx = grd.dy = grd.dz = 0.25
    tp.configure(system_type=tp.SYS_PIC, charge_mass=1.0, bc_flag=1, dom=dom, grd=grd, mt=0)
    mb = wl.kolmogorov_modes(cfg["nmodes"], cfg["kmin"], 16.0, cfg["dB"], cfg["seed"])
    mv = wl.kolmogorov_modes(cfg["nmodes"], cfg["kmin"], 16.0, cfg["v_rms"], cfg["seed"] + 1000)
    tp.synth_pic_fields(mb, mv, 1.0)
    tp.set_spectrum(cfg["nbins"], cfg["emin"], cfg["emax"])
    p0 = wl.shell_particles(n, cfg["speed"], cfg["lo"], cfg["hi"], cfg["seed"])
    rates, res = {}, {}
    for label, seg in (("one_launch", 0), ("compacted", -1)):
        tp.set_compaction(seg)
        best = None
        for _ in range(3):
            r = tp.track(p0, cfg["dt"], 10, cfg["nbins"], precision=tp.PREC_MIXED)
            if best is None or r["info"].kernel_ms < best["info"].kernel_ms:
                best = r
        res[label] = best
        rates[label] = {"particle_steps_per_s": n * steps / best["info"].kernel_ms * 1e3,
                        "kernel_ms": best["info"].kernel_ms, "launches": best["info"].launches}
    tp.set_compaction(-1)
    a, b = res["one_launch"], res["compacted"]
    left = float(a["espect_escape"].sum())
    tp.release_device_fields()
    return {"workload": "open_box_pic_128^3_%dptl_%dsteps" % (n, steps), "rates": rates,
            "departed_fraction": left / n, "pushes_done": int(a["nsteps"].sum() - n),
            "identical": bool(all(np.array_equal(a["ptl"][c], b["ptl"][c]) for c in ("x", "y", "z", "ux", "uy", "uz"))
                              and np.array_equal(a["espect"], b["espect"])
                              and np.array_equal(a["espect_escape"], b["espect_escape"])
                              and np.array_equal(a["remain"], b["remain"])),
            "speedup": rates["one_launch"]["kernel_ms"] / rates["compacted"]["kernel_ms"]}


def io_files(tp, wl, args):
    """The field and particle files of the headline workload through the
    library: the 512^3 field written as the reference's
    PIC HDF5 file (6 float datasets, 3.2 GB) and as .gda files, read back into
    device memory (records identical to the synthesised ones), against the
    reference's CPU path for the same file (the dataset read, then its serial
    reorder loop, restated in the oracle, timed per component); and
    particles_fields_init.h5 of the 1,048,576 particles written with the GPU
    get_emf and read back, against the reference's serial get_emf loop (the
    oracle on a sample) plus the write of the same bytes.  Files in a
    temporary directory, in the page cache when read."""
    import ctypes as C
    import shutil
    cfg = wl.config_grid()
    dom, grd, p0, _, _ = setup_grid(tp, wl, cfg, 0)
    L = tp.lib()
    L.set_variables_bfield(C.byref(grd), C.byref(dom), C.c_double(1.0), C.c_int(0), C.c_int(4))
    L.set_variables_efield(C.byref(grd), C.byref(dom), C.c_double(1.0), C.c_int(0), C.c_int(4))
    he, hb = tp.fetch_device_fields()
    n = cfg["n"]
    nbytes = 6 * 4 * n ** 3
    work = tempfile.mkdtemp(prefix="tp_io_")
    out = {"workload": "pic_%dcube_fields_and_%dptl_particles_fields" % (n, cfg["nptl"]), "dir_in_page_cache": True}
    try:
        h5 = os.path.join(work, "fields_0.h5")
        t0 = time.perf_counter()
        tp.save_pic_fields_h5(h5, "Timestep_0")
        t_save = time.perf_counter() - t0
        for c, name in enumerate(("bx", "by", "bz", "ex", "ey", "ez")):
            (hb if c < 3 else he)[:, c % 3].tofile(os.path.join(work, "%s_0.gda" % name))
        tp.release_device_fields()
        walls = {}
        for kind in ("binary", "h5", "binary", "h5"):
            t0 = time.perf_counter()
            if kind == "h5":
                tp.read_pic_fields_h5(h5, "Timestep_0")
            else:
                tp.read_pic_fields_binary(work + "/", 0)
            walls[kind] = time.perf_counter() - t0  # the second of each: files cached
            if kind == "h5":
                e2, b2 = tp.fetch_device_fields()
                same = bool(np.array_equal(e2, he) and np.array_equal(b2, hb))
                del e2, b2
            tp.release_device_fields()
        # the reference's CPU path for one component: read the dataset, reorder (serial)
        from oracle import h5ref
        from oracle import pyoracle as po
        po.build_oracle()
        f = h5ref.File(h5)
        addr = f.info("/Timestep_0/cbx")[2][1]
        base = f.base
        del f
        rec = np.zeros((n ** 3, 3), np.float32)
        t0 = time.perf_counter()
        data = np.fromfile(h5, dtype="<f4", count=n ** 3, offset=base + addr).reshape(n, n, n)
        t_read = time.perf_counter() - t0
        t0 = time.perf_counter()
        po.pic_records_from_c(data, 1.0, 0, rec)
        t_loop = time.perf_counter() - t0
        ref_same = bool(np.array_equal(rec[:, 0], hb[:, 0]))
        del data, rec
        cpu_s = 6 * (t_read + t_loop)
        out["f2"] = {"file_gb": nbytes / 1e9,
                     "save_h5_s": t_save, "save_h5_gbs": nbytes / t_save / 1e9,
                     "load_h5_s": walls["h5"], "load_h5_gbs": nbytes / walls["h5"] / 1e9,
                     "load_binary_s": walls["binary"], "load_binary_gbs": nbytes / walls["binary"] / 1e9,
                     "records_identical": same,
                     "cpu_reference_path": {"s": cpu_s, "gbs": nbytes / cpu_s / 1e9, "cores": 1,
                                            "kind": "port", "read_s_per_component": t_read,
                                            "reorder_s_per_component": t_loop,
                                            "records_identical": ref_same,
                                            "sample": "one component timed (read + serial reorder loop), x 6"},
                     "load_h5_over_cpu_reference": cpu_s / walls["h5"]}
        # f1: particles_fields_init.h5
        fn = os.path.join(work, "particles_fields_init.h5")
        tp.synth_pic_fields(*[wl.kolmogorov_modes(cfg["nmodes"], cfg["kmin"], cfg["kmax"], a, cfg["seed"] + o)
                              for a, o in ((cfg["dB"], 0), (cfg["v_rms"], 1000))], 1.0)
        p = np.ascontiguousarray(p0)
        ts = []
        for _ in range(2):
            t0 = time.perf_counter()
            tp.save_particles_fields(fn, p)
            ts.append(time.perf_counter() - t0)
        t0 = time.perf_counter()
        q = tp.read_particles(fn, len(p))
        t_rd = time.perf_counter() - t0
        back = bool(all(np.array_equal(q[k], p[k]) for k in ("x", "y", "z", "qm", "ux", "uy", "uz", "t")))
        sample = 65536
        xyzt = np.stack([p["x"][:sample], p["y"][:sample], p["z"][:sample], p["t"][:sample]], 1)
        d = po.Domain.from_buffer_copy(dom)
        g = po.Grids.from_buffer_copy(grd)
        fo = po.make_field(system_type=4, charge_mass=1.0, bc_flag=0, dom=d, grd=g, egrid=he, bgrid=hb)
        t0 = time.perf_counter()
        emf_ref = po.get_emf(fo, xyzt)
        t_emf = (time.perf_counter() - t0) * len(p) / sample
        fields_same = bool(np.array_equal(emf_ref, tp.get_emf(xyzt)))
        blob = np.zeros(len(p) * 14, np.float64)
        t0 = time.perf_counter()
        blob.tofile(os.path.join(work, "blob"))
        t_w = time.perf_counter() - t0
        out["f1"] = {"particles": len(p), "file_mb": os.path.getsize(fn) / 1e6,
                     "save_s": min(ts), "save_particles_per_s": len(p) / min(ts),
                     "read_s": t_rd, "read_particles_per_s": len(p) / t_rd, "read_back_identical": back,
                     "fields_identical_to_oracle_get_emf": fields_same,
                     "cpu_reference_path": {"s": t_emf + t_w, "particles_per_s": len(p) / (t_emf + t_w), "cores": 1,
                                            "kind": "port", "sample": "serial get_emf on %d particles scaled to %d, "
                                            "plus writing the same bytes" % (sample, len(p))},
                     "save_over_cpu_reference": (t_emf + t_w) / min(ts)}
    finally:
        shutil.rmtree(work, ignore_errors=True)
    return out


def poincare_maps(tp, wl, args):
    """Poincare maps (src/poincare_map.c) on the headline's 512^3 gridded B (B0
    along z): field lines from a 128 x 128 grid of seeds on the plane z = L / 2,
    RK4 steps of half a cell, 20 crossings of that plane (about 20 box lengths)
    or 12,288 cells of length each.  The GPU trace of
    every seed against the oracle's (the reference's next_location loop,
    pinned bit-exact to it) on every host core for a sample of seeds, the
    sample compared bit for bit."""
    cfg = wl.config_grid()
    dom, grd, _, _, _ = setup_grid(tp, wl, cfg, 0)
    n = cfg["n"]
    L = cfg["hi"][0] - cfg["lo"][0]
    side = args.nptl or 128
    u = (np.arange(side) + 0.5) / side
    yy, zz = np.meshgrid(u, u, indexing="ij")
    seeds = np.stack([yy.ravel() * L, zz.ravel() * L, np.full(side * side, 0.5 * L)], 1)
    step, ncross, face = 0.5 * cfg["dx"], 20, 2
    lmax = 12288 * cfg["dx"]
    tp.poincare_trace(seeds[:256], face, step, lmax, ncross)  # warm-up
    t0 = time.perf_counter()
    xo, yo, zo, found = tp.poincare_trace(seeds, face, step, lmax, ncross)
    t_gpu = time.perf_counter() - t0
    from oracle import pyoracle as po
    he, hb = tp.fetch_device_fields()
    d = po.Domain.from_buffer_copy(dom)
    g = po.Grids.from_buffer_copy(grd)
    f = po.make_field(system_type=4, charge_mass=1.0, bc_flag=0, dom=d, grd=g, egrid=he, bgrid=hb)
    cores = os.cpu_count() or 1
    sample = np.arange(0, len(seeds), max(1, len(seeds) // (8 * cores)))
    t0 = time.perf_counter()
    ref = po.poincare(f, seeds[sample], face, step, lmax, ncross, nthreads=cores)
    t_cpu = (time.perf_counter() - t0) * len(seeds) / len(sample)
    same = bool(all(np.array_equal(a[sample], r) for a, r in zip((xo, yo, zo, found), ref)))
    return {"workload": "poincare_pic_%dcube_%dseeds_%dcrossings" % (n, len(seeds), ncross),
            "seeds": len(seeds), "step_cells": 0.5, "length_max_cells": 12288, "ncross": ncross,
            "crossings_found": int(found.sum()), "gpu_s": t_gpu, "seeds_per_s": len(seeds) / t_gpu,
            "sample_identical_to_oracle": same,
            "cpu_baseline": {"s": t_cpu, "seeds_per_s": len(seeds) / t_cpu, "cores": cores, "kind": "port",
                             "sample": "%d of the seeds, scaled" % len(sample)},
            "gpu_over_cpu": t_cpu / t_gpu}


def fullsize_modesum(tp, wl, args):
    """C3 and C4 at their configs' own sizes (minutes of GPU time, not in the
    default line): the exact FP32 mode sum on 4,194,304 particles x 20,000
    steps and the learned field, trained as in the default line, on
    16,777,216 particles x 20,000 steps; one run each, device time."""
    cfg = wl.config_modesum()
    dom = tp.Domain()
    dom.xmax = dom.ymax = dom.zmax = 1.0
    modes = wl.kolmogorov_modes(cfg["nmodes"], cfg["kmin"], cfg["kmax"], cfg["dB"], cfg["seed"], va=cfg["va"])
    tp.configure(system_type=tp.SYS_MODESUM, dom=dom, modes=modes, mode_B0=cfg["B0"])
    tp.set_spectrum(cfg["nbins"], cfg["emin"], cfg["emax"])
    dt, nbins, steps = cfg["dt"], cfg["nbins"], cfg["steps"]
    out = {}

    def run(n, code, label):
        tp.set_tmax(steps * dt + 0.5 * dt)
        p = wl.shell_particles(n, cfg["speed"], cfg["lo"], cfg["hi"], cfg["seed"])
        s = tp.Session(n)
        try:
            s.load(p)
            info = s.track(dt, cfg["nt_out"], nbins, code)
            r = s.fetch(cfg["nt_out"], nbins, info.nsdc, particles=False)
        finally:
            s.close()
        out[label] = {"particles": n, "steps": steps, "kernel_s": info.kernel_ms / 1e3,
                      "pushes_per_s": info.pushes / info.kernel_ms * 1e3, "status": tp.device_status(),
                      "spectrum_counts_all_frames": float(np.sum(r["espect"]))}  # n x frames when none escape

    run(4194304, tp.PREC_MIXED, "C3_mixed_exact_sum")
    train = train_surrogate(tp, modes, cfg, args)
    out["C4_train"] = train
    run(16777216, tp.PREC_SURROGATE, "C4_surrogate")
    return out


def config_bench(name, args):
    """One workload on its own (not the headline line)."""
    import test_particle_gb300 as tp
    import test_particle_gb300.workloads as wl
    tp.check(tp.lib().tp_init(0), "tp_init")
    if name == "abc":
        out = secondary_abc(tp, wl)
    elif name in ("modesum", "surrogate"):
        c3, c4 = secondary_modesum(tp, wl, args)
        out = {"C3_modesum": c3, "C4_surrogate": c4}
    elif name == "bs":
        out = secondary_bs(tp, wl, cpu=args.cpu_bs, n=args.nptl or 1048576)
    elif name == "open":
        out = open_box(tp, wl, args)
    elif name == "io":
        out = io_files(tp, wl, args)
    elif name == "poincare":
        out = poincare_maps(tp, wl, args)
    elif name == "fullsize":
        out = fullsize_modesum(tp, wl, args)
    elif name == "gate":
        cfg = wl.config_grid()
        setup_grid(tp, wl, cfg, 0)
        out = gate_run(tp, wl, cfg, args.gate_nptl, args.gate_steps, cfg["seed"] + 4242)
    else:
        raise ValueError(name)
    out["config"] = name
    print(json.dumps(out), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-secondary", action="store_true")
    ap.add_argument("--fp64-steps", type=int, default=3)
    ap.add_argument("--gate-nptl", type=int, default=1 << 26,
                    help="particles of the accuracy gate run (0: skip it)")
    ap.add_argument("--gate-steps", type=int, default=500)
    ap.add_argument("--config", choices=["abc", "modesum", "surrogate", "bs", "open", "gate", "io", "poincare", "fullsize"], default=None,
                    help="one workload on its own instead of the headline line")
    ap.add_argument("--nptl", type=int, default=0)
    ap.add_argument("--run-steps", type=int, default=0)
    ap.add_argument("--epochs", type=int, default=16)
    ap.add_argument("--cpu-bs", action="store_true")
    ap.add_argument("--profile", choices=["mixed", "mixed512", "fp64", "fp64fast", "surrogate", "modesum",
                                          "abc", "train", "h5"],
                    default=None,
                    help="one tracking launch of a small case for a profiler capture (gridded "
                         "field 256^3, 131072 particles, 200 steps; mixed512: the 512^3 headline field "
                         "and particles, 200 steps; surrogate and modesum: 512-mode field, 155648 "
                         "particles, 20 steps; abc: 65536 particles, 1000 steps; train: one training "
                         "epoch of the learned field on 1,048,576 samples; h5: a 256^3 PIC HDF5 field "
                         "file written and read)")
    args = ap.parse_args()
    if args.profile:
        profile_case(args.profile)
        return
    if args.config:
        config_bench(args.config, args)
        return
    world, rank, local, pg = dist_setup()
    if args.impl == "reference":
        reference_arm(args, world, rank)
    else:
        line = headline(args, world, rank, local, pg)
        if rank == 0:
            print(json.dumps(line), flush=True)
    if pg is not None:
        pg.destroy_process_group()


if __name__ == "__main__":
    main()
