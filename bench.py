"""Benchmark: particle pushes per second on one GB300.

Workload (the configuration the headline metric is quoted on): gridded
PIC-style fields on a 512^3 periodic grid (6 FP32 components, synthesised on
the GPU from seeded Kolmogorov modes, B0 = 1 along z, dB/B0 = 0.5,
E = -v x B from a velocity field of rms 0.1), trilinear interpolation,
1,048,576 particles per GPU at |v| = 0.7c, 5,000 Wirz steps per run with the
fused energy-spectrum and diffusion-coefficient diagnostics.  One bench step
is one such run (5.24e9 pushes).  The field (4.3 GB node-interleaved FP32 plus
the 3.2 GB reference AoS copy) is far larger than L2, so no L2 flush is needed
between steps.

value: mixed-precision path (FP32 push and field, 64-bit fixed-point
positions), particles resident in HBM.  e2e: the same through the C ABI with
host buffers (particles copied in and results copied out every step).  The
FP64 parity path is measured on the same workload and reported beside it.

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
# DRAM bytes (read + write) per push of track_mixed_kernel<4>, from one ncu
# capture of `python bench.py --profile mixed` (256^3 grid, 131072 particles,
# 200 steps: 2.130 GB for 26,214,400 pushes); the headline workload has the
# same particle density per cell, so its traffic scales with the pushes.
# Summary: profiles/track_mixed_kernel_pic_256cube_131072ptl.txt
DRAM_BYTES_PER_PUSH = (2.119311e9 + 10.339840e6) / 26214400.0


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


def setup_grid(tp, wl, cfg, rank, to_host=False):
    n = cfg["n"]
    dom = tp.Domain()
    dom.xmin, dom.ymin, dom.zmin = cfg["lo"]
    dom.xmax, dom.ymax, dom.zmax = cfg["hi"]
    dom.xmin_ptl, dom.ymin_ptl, dom.zmin_ptl = cfg["lo"]
    dom.xmax_ptl, dom.ymax_ptl, dom.zmax_ptl = cfg["hi"]
    dom.tmax = cfg["steps"] * cfg["dt"] + 0.5 * cfg["dt"]
    grd = tp.Grids()
    grd.nx = grd.ny = grd.nz = n
    grd.nt = 1
    grd.dx = grd.dy = grd.dz = cfg["dx"]
    tp.configure(system_type=tp.SYS_PIC, charge_mass=1.0, bc_flag=0, dom=dom, grd=grd, mt=0)
    mb = wl.kolmogorov_modes(cfg["nmodes"], cfg["kmin"], cfg["kmax"], cfg["dB"], cfg["seed"])
    mv = wl.kolmogorov_modes(cfg["nmodes"], cfg["kmin"], cfg["kmax"], cfg["v_rms"], cfg["seed"] + 1000)
    he, hb = tp.synth_pic_fields(mb, mv, 1.0, to_host=to_host)
    tp.set_spectrum(cfg["nbins"], cfg["emin"], cfg["emax"])
    p0 = wl.shell_particles(cfg["nptl"], cfg["speed"], cfg["lo"], cfg["hi"], cfg["seed"] + 7 * rank)
    return dom, grd, p0, he, hb


def cpu_baseline(cfg, dom, grd, he, hb, target_s=12.0):
    """The oracle (CPU restatement of the reference's FP64 path) on every host
    core, on a bounded sample of the same workload."""
    from oracle import pyoracle as po
    import test_particle_gb300.workloads as wl
    cores = os.cpu_count() or 1
    d = po.Domain.from_buffer_copy(dom)
    g = po.Grids.from_buffer_copy(grd)
    f = po.make_field(system_type=4, charge_mass=1.0, bc_flag=0, dom=d, grd=g, egrid=he, bgrid=hb)
    s = po.spectrum(cfg["nbins"], cfg["emin"], cfg["emax"])
    dt = cfg["dt"]

    def run(nptl, nsteps):
        d.tmax = nsteps * dt + 0.5 * dt
        f.dom = d
        p = wl.shell_particles(nptl, cfg["speed"], cfg["lo"], cfg["hi"], cfg["seed"] + 99)
        t0 = time.perf_counter()
        po.track_fixed(f, s, p, dt, 1, nthreads=cores)
        return time.perf_counter() - t0

    n_cal, s_cal = 4 * cores * 64, 200
    t_cal = run(n_cal, s_cal)
    rate = n_cal * s_cal / t_cal
    nsteps = 1000
    nptl = int(max(cores * 64, min(cfg["nptl"], rate * target_s / nsteps)))
    t = run(nptl, nsteps)
    return {"value": nptl * nsteps / t, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": "%d particles x %d steps of the same field and dt (oracle FP64, OpenMP %d threads)"
                      % (nptl, nsteps, cores), "seconds": t}


def reference_arm(args, world, rank):
    """The reference's own CPU implementation of the path (its C restatement;
    the reference tree itself is not on the GPU machine)."""
    if rank != 0:
        return
    import test_particle_gb300 as tp
    import test_particle_gb300.workloads as wl
    cfg = wl.config_grid()
    tp.lib().tp_init(0)
    dom, grd, p0, he, hb = setup_grid(tp, wl, cfg, 0, to_host=True)
    vals = []
    base = None
    for _ in range(max(1, args.steps)):
        base = cpu_baseline(cfg, dom, grd, he, hb, target_s=8.0)
        vals.append(base["value"])
    v = float(np.median(vals))
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
            "config": {"workload": cfg["name"], "particles_per_gpu": cfg["nptl"],
                       "steps_per_run": cfg["steps"], "grid": [cfg["n"]] * 3},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": base["cores"], "kind": "port",
                             "sample": base["sample"]},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def profile_case(prec):
    """Small case of a tracking kernel, one launch after a warm-up: the
    gridded field (256^3, 0.5 GB interleaved, larger than L2; 131072
    particles, 200 steps) for mixed / fp64 / fp64fast; the 512-mode field
    with an untrained learned model (the kernel's work does not depend on the
    weights; 155648 particles = 2 x 304 blocks of 256, 20 steps) for surrogate;
    the mixed kernel on the 512-mode field (155648 particles, 20 steps) for
    modesum and on the ABC field (65536 particles, 1000 steps) for abc."""
    import test_particle_gb300 as tp
    import test_particle_gb300.workloads as wl
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
            amp = np.linalg.norm(modes["amp_b"], axis=1)
            tp.mlp_init(modes["n"][np.argsort(-amp)[:64]], seed=3)
            tp.mlp_set_output_norm(np.array([0, 0, 1, 0, 0, 0]), np.ones(6))
        p0 = wl.shell_particles(cfg["nptl"], cfg["speed"], cfg["lo"], cfg["hi"], cfg["seed"])
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


def config_bench(name, args):
    """Secondary workloads (not the headline line): pushes/s per precision and
    the accuracy of the fast paths against the FP64 path on the same inputs."""
    import ctypes as C
    import test_particle_gb300 as tp
    import test_particle_gb300.workloads as wl
    tp.check(tp.lib().tp_init(0), "tp_init")
    out = {"config": name}
    if name in ("abc", "modesum", "surrogate"):
        if name == "abc":
            cfg = wl.config_abc()
            dom = tp.Domain()
            dom.xmax = dom.ymax = dom.zmax = 1.0
            tp.configure(system_type=tp.SYS_FORCEFREE, dom=dom, abc=(1.0, 1.0, 1.0), B0=1.0,
                         lambda0=2 * np.pi)
        else:
            cfg = wl.config_modesum()
            dom = tp.Domain()
            dom.xmax = dom.ymax = dom.zmax = 1.0
            modes = wl.kolmogorov_modes(cfg["nmodes"], cfg["kmin"], cfg["kmax"], cfg["dB"], cfg["seed"],
                                        va=cfg["va"])
            tp.configure(system_type=tp.SYS_MODESUM, dom=dom, modes=modes, mode_B0=cfg["B0"])
        tp.set_spectrum(cfg["nbins"], cfg["emin"], cfg["emax"])
        dt = cfg["dt"]
        out.update(workload=cfg["name"], dt=dt)
        if name == "surrogate":
            # features: the 64 strongest modes' lattice vectors
            amp = np.linalg.norm(modes["amp_b"], axis=1)
            freq = modes["n"][np.argsort(-amp)[:64]]
            tp.mlp_init(freq, seed=3)
            loss, ms = tp.mlp_train(16777216, 65536, args.epochs, lr=2e-3)
            rng = np.random.default_rng(5)
            u = rng.integers(0, 2 ** 32, size=(65536, 3), dtype=np.uint64).astype(np.uint32)
            xyzt = np.zeros((len(u), 4))
            xyzt[:, :3] = u / 2 ** 32
            exact = tp.get_emf(xyzt)
            model = tp.mlp_eval_kernel(u)
            dB = exact[:, :3] - [0, 0, cfg["B0"]]
            out["train"] = {"samples": 16777216, "epochs": args.epochs, "final_loss": loss,
                            "train_ms": ms,
                            "rel_rms_err_dB": float(np.sqrt(np.mean((model[:, :3] - exact[:, :3]) ** 2) /
                                                            np.mean(dB ** 2))),
                            "rel_rms_err_E": float(np.sqrt(np.mean((model[:, 3:] - exact[:, 3:]) ** 2) /
                                                           np.mean(exact[:, 3:] ** 2)))}
        n = args.nptl or cfg["nptl"]
        steps = args.run_steps or cfg["steps"]
        p0 = wl.shell_particles(n, cfg["speed"], cfg["lo"], cfg["hi"], cfg["seed"])
        precs = {"abc": [("fp64", tp.PREC_FP64), ("fp64fast", tp.PREC_FP64_FAST), ("mixed", tp.PREC_MIXED)],
                 "modesum": [("fp64", tp.PREC_FP64), ("mixed", tp.PREC_MIXED)],
                 "surrogate": [("surrogate", tp.PREC_SURROGATE), ("mixed", tp.PREC_MIXED)]}[name]
        sess = tp.Session(n)
        rates = {}
        for label, code in precs:
            st = min(steps, args.fp64_steps_cap) if label.startswith("fp64") else steps
            tp.set_tmax(st * dt + 0.5 * dt)
            sess.load(p0)
            info = sess.track(dt, max(1, st // 1000), cfg["nbins"], code)
            rates[label] = {"pushes_per_s": info.pushes / info.kernel_ms * 1e3, "steps": st,
                            "particles": n, "kernel_ms": info.kernel_ms}
        if name == "surrogate":
            # what the model gains: the exact sum's cost grows with the mode count, the model's does not
            big = wl.kolmogorov_modes(4096, cfg["kmin"], cfg["kmax"], cfg["dB"], cfg["seed"] + 5, va=cfg["va"])
            tp.configure(system_type=tp.SYS_MODESUM, dom=dom, modes=big, mode_B0=cfg["B0"])
            tp.set_spectrum(cfg["nbins"], cfg["emin"], cfg["emax"])
            st = min(steps, 50)
            tp.set_tmax(st * dt + 0.5 * dt)
            sess.load(p0)
            info = sess.track(dt, 1, cfg["nbins"], tp.PREC_MIXED)
            rates["mixed_exact_4096_modes"] = {"pushes_per_s": info.pushes / info.kernel_ms * 1e3, "steps": st,
                                               "particles": n, "kernel_ms": info.kernel_ms}
            tp.configure(system_type=tp.SYS_MODESUM, dom=dom, modes=modes, mode_B0=cfg["B0"])
            tp.set_spectrum(cfg["nbins"], cfg["emin"], cfg["emax"])
        out["rates"] = rates
        # accuracy of the fast path(s) against FP64 (or against the exact field for the surrogate)
        na, sa = args.acc_nptl, args.acc_steps
        pa = wl.shell_particles(na, cfg["speed"], cfg["lo"], cfg["hi"], cfg["seed"] + 1)
        pb = pa.copy()
        rng = np.random.default_rng(77)
        for k in ("ux", "uy", "uz"):  # 1-ulp-level perturbation: the FP64-vs-FP64 noise floor
            pb[k] = pa[k] * (1 + 1e-15 * rng.standard_normal(na))
        tp.set_tmax(sa * dt + 0.5 * dt)
        ref_code = tp.PREC_MIXED if name == "surrogate" else tp.PREC_FP64
        runs = {}
        for label, code, pp in (("ref", ref_code, pa), ("ref_perturbed", ref_code, pb),
                                ("fast", tp.PREC_SURROGATE if name == "surrogate" else tp.PREC_MIXED, pa)):
            s2 = tp.Session(na)
            s2.load(pp)
            info = s2.track(dt, 10, cfg["nbins"], code)
            runs[label] = s2.fetch(10, cfg["nbins"], info.nsdc)
            s2.close()

        def spec_l1(a, b):
            return float(np.abs(a["espect"][-1] / na - b["espect"][-1] / na).sum())

        def dc_rel(a, b):
            x, y = a["dsum"][:, -1], b["dsum"][:, -1]
            return [float(v) for v in np.abs(x - y) / np.maximum(np.abs(y), 1e-300)]
        out["accuracy"] = {"particles": na, "steps": sa, "against": "fp64" if name != "surrogate" else "exact mode sum (mixed)",
                           "spectrum_l1_fast": spec_l1(runs["fast"], runs["ref"]),
                           "spectrum_l1_noise_floor": spec_l1(runs["ref_perturbed"], runs["ref"]),
                           "diffusion_rel_err_fast": dc_rel(runs["fast"], runs["ref"]),
                           "diffusion_rel_err_noise_floor": dc_rel(runs["ref_perturbed"], runs["ref"]),
                           "diffusion_order": ["drr", "dxx", "dyy", "dzz", "dpp", "duu", "daa", "dee"]}
        sess.close()
    elif name == "open":
        # open boundaries: a 128^3 gridded field in an open box that most
        # particles leave within the run; one launch against segments with the
        # departed particles compacted away (identical results)
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
        out.update(workload="open_box_pic_128^3_%dptl_%dsteps" % (n, steps), rates=rates,
                   departed_fraction=left / n,
                   pushes_done=int(a["nsteps"].sum() - n),
                   identical=bool(all(np.array_equal(a["ptl"][c], b["ptl"][c]) for c in ("x", "y", "z", "ux", "uy", "uz"))
                                  and np.array_equal(a["espect"], b["espect"])
                                  and np.array_equal(a["espect_escape"], b["espect_escape"])
                                  and np.array_equal(a["remain"], b["remain"])),
                   speedup=rates["one_launch"]["kernel_ms"] / rates["compacted"]["kernel_ms"])
        tp.release_device_fields()
    elif name == "bs":
        # one circular loop (radius 1, current 1, no wire), E = 0; particles on a
        # torus around the wire, |v| in [0.1, 0.9] c; the reference's equations
        # (beta form, positions in L0, CGS q/m of a proton); rtol = atol = 1e-10
        dom = tp.Domain()
        for a in ("xmin", "ymin", "zmin"):
            setattr(dom, a, -3.0)
        for a in ("xmax", "ymax", "zmax"):
            setattr(dom, a, 3.0)
        w = tp.Wlcs()
        w.costheta_wr = w.cosphi_wr = w.cosalpha_lp = w.cosbeta_lp = 1.0
        w.cur_lp, w.r_lp, w.omega = 1.0, 1.0, 0.001
        tp.configure(system_type=tp.SYS_WLCS, charge_mass=9.58e3, bc_flag=2, dom=dom, wl=[w])
        n = args.nptl or 1048576
        t_end = 0.05
        tp.set_spectrum(100, 1e-3, 10.0)
        y0 = wl.torus_particles(n, 1.0, 0.05, 0.3, 0.1, 0.9, 31)
        L = tp.lib()
        res = {}
        for rep in range(2):
            y = y0.copy()
            t = np.zeros(n)
            steps = np.zeros(n, dtype=np.int32)
            st = np.zeros(n, dtype=np.int32)
            esp = np.zeros(10 * 100)
            dfr = np.zeros(8 * 11)
            info = tp.RunInfo()
            tp.check(L.tp_bs_run(C.c_int(n), tp._ptr(y), tp._ptr(t), C.c_double(t_end), C.c_int(10),
                                 C.c_int(100), C.c_double(1e-6), C.c_double(1e-10), C.c_double(1e-10),
                                 C.c_int(8), C.c_int(0), C.c_int(1000000), tp._ptr(steps), tp._ptr(st),
                                 tp._ptr(esp), tp._ptr(dfr), C.byref(info)), "bs_run")
            res = {"accepted_steps_per_s": info.pushes / info.kernel_ms * 1e3,
                   "kernel_ms": info.kernel_ms, "particles": n, "t_end": t_end,
                   "steps_min_median_max": [int(steps.min()), float(np.median(steps)), int(steps.max())],
                   "status_nonzero": int((st != 0).sum()),
                   "beta_rel_drift_max": float(np.max(np.abs(np.linalg.norm(y[:, 3:], axis=1) /
                                                             np.linalg.norm(y0[:, 3:], axis=1) - 1)))}
        out.update(workload="wire_loop_bs_%dptl" % n, rates={"bs_fp64": res})
        if args.cpu_bs:
            from oracle import pyoracle as po
            cores = os.cpu_count() or 1
            m = cores * 16
            f = po.make_field(system_type=1, charge_mass=9.58e3, bc_flag=2,
                              dom=po.Domain.from_buffer_copy(dom), wl=[po.Wlcs.from_buffer_copy(w)])
            t0 = time.perf_counter()
            nsteps = po.bs_run_many(f, y0[:m], 1e-6, 100, atol=1e-10, rtol=1e-10, nthreads=cores)
            dtc = time.perf_counter() - t0
            out["cpu_baseline"] = {"value": nsteps / dtc, "unit": "accepted steps/s", "cores": cores,
                                   "kind": "port", "sample": "%d particles x 100 steps" % m}
    print(json.dumps(out), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--fp64-steps", type=int, default=1)
    ap.add_argument("--config", choices=["abc", "modesum", "surrogate", "bs", "open"], default=None,
                    help="secondary workload instead of the headline line")
    ap.add_argument("--nptl", type=int, default=0)
    ap.add_argument("--run-steps", type=int, default=0)
    ap.add_argument("--fp64-steps-cap", type=int, default=1000)
    ap.add_argument("--acc-nptl", type=int, default=65536)
    ap.add_argument("--acc-steps", type=int, default=2000)
    ap.add_argument("--epochs", type=int, default=4)
    ap.add_argument("--cpu-bs", action="store_true")
    ap.add_argument("--profile", choices=["mixed", "fp64", "fp64fast", "surrogate", "modesum", "abc"],
                    default=None,
                    help="one tracking launch of a small case for a profiler capture (gridded "
                         "field 256^3, 131072 particles, 200 steps; surrogate and modesum: 512-mode "
                         "field, 155648 particles, 20 steps; abc: 65536 particles, 1000 steps)")
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
        return
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

    # ---- mixed-precision path, particles resident in HBM
    for _ in range(max(3, args.warmup)):
        sess.track(dt, nt_out, nbins, tp.PREC_MIXED)
    barrier(pg)
    kms, sms, launches = [], [], 0
    with Clocks(local) as clk:
        t0 = time.perf_counter()
        for _ in range(args.steps):
            info = sess.track(dt, nt_out, nbins, tp.PREC_MIXED)
            kms.append(info.kernel_ms)
            sms.append(info.step_ms)
            launches += info.launches
        wall = time.perf_counter() - t0
    barrier(pg)
    dev_s = allmax(pg, sum(sms) / 1e3)
    pushes = info.pushes
    value = pushes * args.steps * world / dev_s
    clocks = clk.summary()
    # one run of each path from the same initial state, for the accuracy figures
    sess.load(p0)
    sess.track(dt, nt_out, nbins, tp.PREC_MIXED)
    diag = sess.fetch(nt_out, nbins, info.nsdc)

    # ---- FP64 parity path on the same workload (fresh particle state)
    f64 = []
    for _ in range(max(1, args.fp64_steps)):
        sess.load(p0)
        f64.append(sess.track(dt, nt_out, nbins, tp.PREC_FP64).kernel_ms)
    fp64_value = pushes / (float(np.median(f64)) / 1e3)
    d64 = sess.fetch(nt_out, nbins, info.nsdc)
    # the FP64 path again from the initial state rounded to FP32: how far two
    # FP64 runs drift apart from a difference of one FP32 rounding (chaos)
    p0r = p0.copy()
    for c in ("x", "y", "z", "ux", "uy", "uz"):
        p0r[c] = p0r[c].astype(np.float32).astype(np.float64)
    sess.load(p0r)
    sess.track(dt, nt_out, nbins, tp.PREC_FP64)
    d64r = sess.fetch(nt_out, nbins, info.nsdc)
    e1 = diag["espect"][-1] / max(1.0, diag["espect"][-1].sum())
    e2 = d64["espect"][-1] / max(1.0, d64["espect"][-1].sum())
    spec_l1 = float(np.abs(e1 - e2).sum())
    # per output frame: the L1 distance of the two spectra, and the distance
    # two independent ensembles of this size drawn from the FP64 spectrum would
    # show (sum over bins of sqrt(4 p (1 - p) / (pi N))): while the paths still
    # follow the same trajectories the first is far below the second, once
    # chaos has decorrelated them it sits at it
    def l1(fa, fb):
        return float(np.abs(fa / max(1.0, fa.sum()) - fb / max(1.0, fb.sum())).sum())

    frames_l1 = [l1(fa, fb) for fa, fb in zip(diag["espect"], d64["espect"])]
    frames_chaos = [l1(fa, fb) for fa, fb in zip(d64r["espect"], d64["espect"])]
    frames_floor = []
    for fb in d64["espect"]:
        nb = max(1.0, fb.sum())
        q = fb / nb
        frames_floor.append(float(np.sqrt(4 * q * (1 - q) / (np.pi * nb)).sum()))
    dc_chaos = np.abs(d64r["dsum"][:, -1] - d64["dsum"][:, -1]) / np.maximum(np.abs(d64["dsum"][:, -1]), 1e-300)
    dc_rel = np.abs(diag["dsum"][:, -1] - d64["dsum"][:, -1]) / np.maximum(np.abs(d64["dsum"][:, -1]), 1e-300)
    sess.close()

    # ---- e2e: host buffers through the C ABI, copies inside the timed region
    ptl = p0.copy()
    e2e_times = []
    import ctypes as C
    L = tp.lib()
    esp = np.zeros(nt_out * nbins)
    ese = np.zeros(nt_out * nbins)
    nsdc = info.nsdc
    dsum = np.zeros(8 * nsdc)
    rem = np.zeros(nsdc, dtype=np.int32)
    nst = np.zeros(n, dtype=np.int32)
    ri = tp.RunInfo()
    for it in range(1 + args.steps):
        t1 = time.perf_counter()
        tp.check(L.tp_track_host(C.c_int(tp.PREC_MIXED), C.c_int(n), C.c_double(dt), C.c_int(nt_out),
                                 C.c_int(nbins), tp._ptr(p0), tp._ptr(ptl), tp._ptr(nst), tp._ptr(esp),
                                 tp._ptr(ese), tp._ptr(dsum), tp._ptr(rem), C.byref(ri)), "e2e")
        if it > 0:
            e2e_times.append(time.perf_counter() - t1)
    e2e_s = allmax(pg, float(np.median(e2e_times)))
    h2d = 2 * n * 88
    d2h = n * 88 + n * 4 + 2 * nt_out * nbins * 4 + 8 * nsdc * 8 + nsdc * 4

    hbm, peak_kind = peaks()
    kernel_s = float(np.median(kms)) / 1e3
    alg_bytes = pushes * 384.0  # 2 field evaluations x 8 corners x 6 FP32 components
    achieved = alg_bytes / kernel_s / 1e9
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": max(3, args.warmup), "ms_per_step": dev_s * 1e3 / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded Kolmogorov fields and particles)",
            "config": {"workload": cfg["name"], "particles_per_gpu": n, "steps_per_run": cfg["steps"],
                       "grid": [cfg["n"]] * 3, "field_bytes": cfg["n"] ** 3 * 32,
                       "precision": "FP32 push/field, 64-bit fixed-point positions, FP64 sums",
                       "l2": "inputs larger than L2 (4.3 GB field), no flush",
                       "parallelism": "particles sharded, replicas of the field"},
            "e2e": {"value": pushes * world / e2e_s, "unit": UNIT, "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h},
            "gpu_launches": launches,
            "clocks": clocks,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                         "frac": achieved / hbm, "peak_kind": peak_kind,
                         "traffic": DRAM_BYTES_PER_PUSH * pushes,
                         "traffic_note": "ncu DRAM bytes of the 256^3 case scaled by pushes per launch",
                         "kernel": "track_mixed_kernel<PIC>",
                         "algorithmic_bytes_per_push": 384,
                         # the gathers above 1.0 are served by the register cell cache,
                         # L1 and L2; what reaches DRAM is the traffic over the same time
                         "dram_gbs": DRAM_BYTES_PER_PUSH * pushes / kernel_s / 1e9,
                         "dram_frac": DRAM_BYTES_PER_PUSH * pushes / kernel_s / 1e9 / hbm},
            "fp64": {"value": fp64_value * world, "unit": UNIT,
                     "mixed_over_fp64": value / (fp64_value * world),
                     "spectrum_l1_mixed_vs_fp64": spec_l1,
                     "spectrum_l1_per_frame": frames_l1,
                     "spectrum_l1_fp64_from_fp32_rounded_start_per_frame": frames_chaos,
                     "spectrum_l1_sampling_floor_per_frame": frames_floor,
                     "diffusion_rel_err_fp64_from_fp32_rounded_start_final": [float(v) for v in dc_chaos],
                     "frame_steps": [int(cfg["steps"] // nt_out * k) for k in range(nt_out)],
                     "diffusion_rel_err_mixed_vs_fp64_final": [float(v) for v in dc_rel],
                     "diffusion_order": ["drr", "dxx", "dyy", "dzz", "dpp", "duu", "daa", "dee"]},
            }
    if want_cpu:
        try:
            line["cpu_baseline"] = cpu_baseline(cfg, dom, grd, he, hb)
        except Exception as e:
            line["cpu_baseline"] = {"value": None, "error": str(e)}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if pg is not None:
        pg.destroy_process_group()


if __name__ == "__main__":
    main()
