"""The learned field model: tensor-core training gradients against the FP64
oracle, the two inference paths against each other, training against the
mode-sum field it learns, and tracking with it against the exact field."""
import numpy as np
import pytest

from oracle import mlp_oracle as mo

pytestmark = pytest.mark.gpu
tp = pytest.importorskip("test_particle_gb300")
import test_particle_gb300.workloads as wl  # noqa: E402


def bf16_round(a):
    a = np.asarray(a, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32)


def lattice_freq(seed=3):
    rng = np.random.default_rng(seed)
    f = rng.integers(-8, 9, size=(64, 3))
    f[np.all(f == 0, axis=1)] = [1, 0, 0]
    return f


def test_gradients_match_fp64_oracle():
    freq = lattice_freq()
    tp.mlp_init(freq, seed=5)
    tp.mlp_set_output_norm(np.zeros(6), np.ones(6))
    w = tp.mlp_weights()
    rng = np.random.default_rng(11)
    n = 1024
    u = rng.integers(0, 2 ** 32, size=(n, 3), dtype=np.uint64).astype(np.uint32)
    t = rng.normal(0, 1, size=(n, 6)).astype(np.float32)
    loss, y, g = tp.mlp_grad(u, t)
    # the device computes with BF16 weights and features: give the oracle the same
    wq = w.astype(np.float64)
    off = 0
    for i, o in mo.SIZES:
        wq[off:off + i * o] = bf16_round(w[off:off + i * o])
        off += i * o + o
    x = bf16_round(mo.features(u, freq)).astype(np.float64)
    rloss, ry, rg = mo.loss_and_grads(wq, x, t.astype(np.float64))
    assert abs(loss - rloss) / rloss < 2e-2
    assert np.abs(y - ry).max() < 0.05 * np.abs(ry).max()
    off = 0
    for l, (i, o) in enumerate(mo.SIZES):
        for name, sz in (("W", i * o), ("b", o)):
            a, b = g[off:off + sz], rg[off:off + sz]
            off += sz
            rel = np.linalg.norm(a - b) / np.linalg.norm(b)
            cos = a @ b / (np.linalg.norm(a) * np.linalg.norm(b))
            assert rel < 0.05 and cos > 0.998, (l, name, rel, cos)


def small_modes(seed=21):
    return wl.kolmogorov_modes(16, 1, 4, 0.5, seed, va=0.1)


def test_training_learns_a_small_field():
    modes = small_modes()
    dom = tp.Domain()
    dom.xmax = dom.ymax = dom.zmax = 1.0
    tp.configure(system_type=tp.SYS_MODESUM, dom=dom, modes=modes, mode_B0=1.0)
    # the field's own lattice vectors among the features
    freq = np.zeros((64, 3), dtype=np.int64)
    freq[:16] = modes["n"]
    freq[16:] = lattice_freq(4)[16:] // 2 + np.array([1, 0, 0])
    tp.mlp_init(freq, seed=9)
    loss, ms = tp.mlp_train(1 << 20, 8192, 3, lr=2e-3)
    assert loss < 1e-2, loss
    rng = np.random.default_rng(2)
    u = rng.integers(0, 2 ** 32, size=(4096, 3), dtype=np.uint64).astype(np.uint32)
    xyzt = np.zeros((4096, 4))
    xyzt[:, :3] = u / 2 ** 32
    exact = tp.get_emf(xyzt)
    model = tp.mlp_eval(u)
    err_b = np.sqrt(np.mean((model[:, :3] - exact[:, :3]) ** 2)) / np.sqrt(np.mean((exact[:, :3] - [0, 0, 1]) ** 2))
    assert err_b < 0.1, err_b
    # the in-kernel evaluation path agrees with the training forward pass
    mk = tp.mlp_eval_kernel(u)
    assert np.abs(mk - model).max() < 2e-2 * np.abs(model).max()


def test_surrogate_tracking_runs_and_tracks_the_exact_field():
    """Tracking with the trained model of a 16-mode field against tracking
    with the exact FP32 sum: per output frame the spectra differ by no more
    than two independent ensembles of this size drawn from the exact run's
    spectrum would (the sampling floor) plus 3 sigma of that distance."""
    modes = small_modes()
    dom = tp.Domain()
    dom.xmax = dom.ymax = dom.zmax = 1.0
    steps = 400
    dt = wl.gyro_dt(0.7, 1.0)
    dom.tmax = steps * dt + 0.5 * dt
    tp.configure(system_type=tp.SYS_MODESUM, dom=dom, modes=modes, mode_B0=1.0)
    freq = np.zeros((64, 3), dtype=np.int64)
    freq[:16] = modes["n"]
    freq[16:] = lattice_freq(4)[16:] // 2 + np.array([1, 0, 0])
    tp.mlp_init(freq, seed=9)
    tp.mlp_train(1 << 20, 8192, 3, lr=2e-3)
    tp.set_spectrum(200, 1e-3, 1e2)
    n = 16384
    p0 = wl.shell_particles(n, 0.7, (0, 0, 0), (1, 1, 1), 8)
    a = tp.track(p0, dt, 4, 200, precision=tp.PREC_MIXED)
    b = tp.track(p0, dt, 4, 200, precision=tp.PREC_SURROGATE)
    assert b["espect"].sum() == a["espect"].sum() == 4 * n
    assert np.all(b["nsteps"] == steps + 1)
    l1 = np.abs(a["espect"] / n - b["espect"] / n).sum(axis=1)
    q = a["espect"] / n
    floor = np.sqrt(4 * q * (1 - q) / (np.pi * n)).sum(axis=1)
    sigma = np.sqrt(2 * (1 - 2 / np.pi) / n)
    print("surrogate vs exact L1 %s sampling floor %s" % (l1, floor))
    assert np.all(l1 <= floor + 3 * sigma), (l1, floor)
    assert tp.device_status() == 0


def test_stalled_pipeline_is_reported_and_the_context_survives():
    """The bounded hand-over waits of the tensor-core pipeline: with a limit of
    one poll they run out, the tracking kernel raises status bit 16 and stops
    its blocks cleanly; with the default limit restored the same run gives the
    ordinary results on the same context."""
    modes = small_modes()
    dom = tp.Domain()
    dom.xmax = dom.ymax = dom.zmax = 1.0
    steps = 50
    dt = wl.gyro_dt(0.7, 1.0)
    dom.tmax = steps * dt + 0.5 * dt
    tp.configure(system_type=tp.SYS_MODESUM, dom=dom, modes=modes, mode_B0=1.0)
    tp.mlp_init(lattice_freq(5), seed=4)
    tp.set_spectrum(200, 1e-3, 1e2)
    p0 = wl.shell_particles(2048, 0.7, (0, 0, 0), (1, 1, 1), 9)
    tp.device_status()
    ref = tp.track(p0, dt, 1, 200, precision=tp.PREC_SURROGATE)
    assert tp.device_status() == 0
    tp.check(tp.lib().tp_set_wait_limit(1), "wait limit")
    try:
        tp.track(p0, dt, 1, 200, precision=tp.PREC_SURROGATE)
        status = tp.device_status()
    finally:
        tp.check(tp.lib().tp_set_wait_limit(0), "wait limit")
    assert status & 16, status
    again = tp.track(p0, dt, 1, 200, precision=tp.PREC_SURROGATE)
    assert tp.device_status() == 0
    for c in ("x", "y", "z", "ux", "uy", "uz"):
        assert np.array_equal(again["ptl"][c], ref["ptl"][c]), c
    assert np.array_equal(again["espect"], ref["espect"])


def test_tensor_core_inference_matches_fp64_forward():
    """The in-kernel evaluation (tcgen05.mma chain, BF16 weights and
    activations, FP32 accumulation in tensor memory) against the FP64 forward
    pass of the same BF16 weights, on 3 tiles of 256 positions plus a ragged
    tail."""
    freq = lattice_freq(7)
    tp.mlp_init(freq, seed=13)
    tp.mlp_set_output_norm(np.zeros(6), np.ones(6))
    w = tp.mlp_weights().astype(np.float64)
    off = 0
    for i, o in mo.SIZES:
        w[off:off + i * o] = bf16_round(w[off:off + i * o])
        off += i * o + o
    rng = np.random.default_rng(17)
    u = rng.integers(0, 2 ** 32, size=(3 * 256 + 77, 3), dtype=np.uint64).astype(np.uint32)
    x = bf16_round(mo.features(u, freq)).astype(np.float64)
    ref, _, _ = mo.forward(mo.unflatten(w), x)
    got = tp.mlp_eval_kernel(u)
    scale = np.abs(ref).max()
    assert scale > 0
    err = np.abs(got - ref).max() / scale
    assert err < 3e-2, err
    c = np.corrcoef(got.ravel(), ref.ravel())[0, 1]
    assert c > 0.999, c
    gemm = tp.mlp_eval(u)
    assert np.abs(got - gemm).max() < 2e-2 * scale
    assert tp.device_status() == 0


def test_trained_model_gains_over_the_exact_sum():
    """What the trained model gains over the method without it, on a field of
    4096 plane waves with the workload's spectrum: tracking with the model is
    more than 3x faster than with the exact FP32 sum (its cost does not grow
    with the mode count), and at equal cost -- the exact sum truncated to the
    K strongest modes that run as fast as the model -- its field error is the
    smaller one."""
    cfg = wl.config_modesum()
    modes = wl.kolmogorov_modes(4096, cfg["kmin"], cfg["kmax"], cfg["dB"], cfg["seed"] + 5, va=cfg["va"])
    dom = tp.Domain()
    dom.xmax = dom.ymax = dom.zmax = 1.0
    steps = 20
    dt = wl.gyro_dt(0.7, 1.0)
    dom.tmax = steps * dt + 0.5 * dt
    tp.configure(system_type=tp.SYS_MODESUM, dom=dom, modes=modes, mode_B0=1.0)
    tp.set_spectrum(200, 1e-3, 1e2)
    tp.mlp_init(wl.surrogate_features(modes), seed=3)
    tp.mlp_train(1 << 24, 65536, 16, lr=2e-3)
    rng = np.random.default_rng(2)
    u = rng.integers(0, 2 ** 32, size=(65536, 3), dtype=np.uint64).astype(np.uint32)
    xyzt = np.zeros((len(u), 4))
    xyzt[:, :3] = u / 2 ** 32
    exact = tp.get_emf(xyzt)
    db2 = np.mean((exact[:, :3] - [0, 0, 1]) ** 2)
    err_model = np.sqrt(np.mean((tp.mlp_eval_kernel(u)[:, :3] - exact[:, :3]) ** 2) / db2)
    p0 = wl.shell_particles(262144, 0.7, (0, 0, 0), (1, 1, 1), 6)
    s = tp.Session(len(p0))
    rate = {}
    for label, code in (("exact", tp.PREC_MIXED), ("model", tp.PREC_SURROGATE)):
        best = None
        for _ in range(2):  # the first run includes one-time set-up
            s.load(p0)
            info = s.track(dt, 1, 200, code)
            best = info.kernel_ms if best is None else min(best, info.kernel_ms)
        rate[label] = info.pushes / best
    s.close()
    k = int(4096 * rate["exact"] / rate["model"])
    top = modes[np.argsort(-np.linalg.norm(modes["amp_b"], axis=1))[:k]]
    tp.configure(system_type=tp.SYS_MODESUM, dom=dom, modes=top, mode_B0=1.0)
    err_trunc = np.sqrt(np.mean((tp.get_emf(xyzt)[:, :3] - exact[:, :3]) ** 2) / db2)
    print("model %.3gx the exact sum's pushes/s; field error model %.3f, exact sum of the %d strongest "
          "modes %.3f" % (rate["model"] / rate["exact"], err_model, k, err_trunc))
    assert rate["model"] > 3 * rate["exact"], rate
    assert err_model < err_trunc, (err_model, err_trunc, k)
    assert tp.device_status() == 0
