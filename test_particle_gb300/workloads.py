"""Seeded synthetic workloads for the benchmark configurations.

No dataset ships with the reference (its VPIC field files are not part of
it), so the inputs are synthesised from seeds with the shapes, sizes and
value distributions the benchmark configurations state:

* particles: positions uniform in the box, momenta on an isotropic shell of
  fixed speed (the single-velocity branch of init_ptl, src/particle_info.c:345-352);
* turbulent fields: integer-lattice plane waves n (|n| log-uniform in
  [nmin, nmax], isotropic directions), polarisation perpendicular to n
  (solenoidal, as the projection (I - kk/k^2) of data/turbulence.c), random
  phases, and a Kolmogorov power spectrum E(k) ~ k^-5/3: with log-uniform
  sampling each mode carries energy ~ k * E(k), i.e. amplitude ~ k^-1/3;
  amplitudes scaled to the stated rms.
"""
import numpy as np

from . import MODE_DTYPE, PARTICLE_DTYPE


def kolmogorov_modes(nmodes, nmin, nmax, rms, seed, va=0.0, index=-5.0 / 3.0):
    """Plane-wave modes on the integer lattice; amp_e = -va * (n/|n|) x amp_b."""
    rng = np.random.default_rng(seed)
    out = np.zeros(nmodes, dtype=MODE_DTYPE)
    m = 0
    while m < nmodes:
        k = np.exp(rng.uniform(np.log(nmin), np.log(nmax)))
        mu = rng.uniform(-1, 1)
        ph = rng.uniform(0, 2 * np.pi)
        d = np.array([np.sqrt(1 - mu * mu) * np.cos(ph), np.sqrt(1 - mu * mu) * np.sin(ph), mu])
        n = np.rint(k * d).astype(np.int64)
        if not n.any():
            continue
        nn = n / np.linalg.norm(n)
        a = rng.normal(size=3)
        e = a - nn * (a @ nn)
        e /= np.linalg.norm(e)
        kk = np.linalg.norm(n)
        amp = kk ** ((index + 1.0) / 2.0)  # energy per log-uniform sample ~ k E(k)
        out[m]["n"] = n
        out[m]["amp_b"] = amp * e
        out[m]["phase"] = rng.uniform(0, 2 * np.pi)
        m += 1
    scale = rms / np.sqrt(0.5 * np.sum(out["amp_b"] ** 2))
    out["amp_b"] *= scale
    nhat = out["n"] / np.linalg.norm(out["n"], axis=1, keepdims=True)
    out["amp_e"] = -va * np.cross(nhat, out["amp_b"])
    return out


def surrogate_features(modes, k=64):
    """Fourier-feature frequencies of the learned field: the k strongest
    distinct lattice vectors of a mode table, up to sign, by the energy of the
    plane waves that share each vector (modes whose n round to the same lattice
    vector add to one plane wave, sum_m a_m exp(+-i phase_m)).  Low-|n| vectors
    recur among many modes, so taking the k strongest *modes* instead would
    repeat a few vectors and leave features unused."""
    acc = {}
    for q in np.asarray(modes):
        n = tuple(int(v) for v in q["n"])
        m = tuple(-v for v in n)
        c, sgn = (n, 1.0) if n >= m else (m, -1.0)
        acc[c] = acc.get(c, 0) + q["amp_b"] * np.exp(1j * sgn * q["phase"])
    order = sorted(acc, key=lambda c: (-float(np.sum(np.abs(acc[c]) ** 2)), c))
    out = np.zeros((k, 3), dtype=np.int32)
    for i, c in enumerate(order[:k]):
        out[i] = c
    for i in range(len(order), k):  # fewer distinct vectors than features: unit axes
        out[i] = [(i % 3) == 0, (i % 3) == 1, (i % 3) == 2]
    return out


def shell_particles(n, speed, lo, hi, seed, qm=1.0):
    """Uniform positions in [lo, hi), isotropic momenta with |v| = speed (c = 1)."""
    rng = np.random.default_rng(seed)
    p = np.zeros(n, dtype=PARTICLE_DTYPE)
    lo = np.asarray(lo, dtype=np.float64)
    hi = np.asarray(hi, dtype=np.float64)
    pos = lo + rng.random((n, 3)) * (hi - lo)
    p["x"], p["y"], p["z"] = pos.T
    p["qm"] = qm
    u = speed / np.sqrt(1.0 - speed * speed)
    mu = rng.uniform(-1.0, 1.0, n)
    ph = rng.uniform(0.0, 2.0 * np.pi, n)
    s = np.sqrt(1.0 - mu * mu)
    p["ux"], p["uy"], p["uz"] = u * s * np.cos(ph), u * s * np.sin(ph), u * mu
    return p


def torus_particles(n, major, minor_lo, minor_hi, speed_lo, speed_hi, seed):
    """Particles on a torus around a circular loop in the z = 0 plane, with
    |v| uniform in [speed_lo, speed_hi]; returns (x, y, z, beta) rows."""
    rng = np.random.default_rng(seed)
    r = rng.uniform(minor_lo, minor_hi, n)
    a = rng.uniform(0, 2 * np.pi, n)
    phi = rng.uniform(0, 2 * np.pi, n)
    R = major + r * np.cos(a)
    y = np.zeros((n, 6))
    y[:, 0], y[:, 1], y[:, 2] = R * np.cos(phi), R * np.sin(phi), r * np.sin(a)
    b = rng.uniform(speed_lo, speed_hi, n)
    mu = rng.uniform(-1, 1, n)
    ph = rng.uniform(0, 2 * np.pi, n)
    s = np.sqrt(1 - mu * mu)
    y[:, 3], y[:, 4], y[:, 5] = b * s * np.cos(ph), b * s * np.sin(ph), b * mu
    return y


def gyro_dt(speed, B, qm=1.0, fraction=0.01):
    """dt = fraction of the gyroperiod 2 pi gamma / (q/m B)."""
    gamma = 1.0 / np.sqrt(1.0 - speed * speed)
    return fraction * 2.0 * np.pi * gamma / (qm * B)


# ---------------------------------------------------------------- configurations
def config_abc(nptl=65536, steps=10000, seed=11):
    """ABC force-free field A = B = C = 1, k = 2 pi, L = 1, E = 0, periodic cube;
    |v| = 0.7c; dt = 0.01 gyroperiod at the rms field |B| = sqrt(3); 200 log
    bins every 1000 steps (nbins 200, gamma - 1 in [1e-3, 1e2])."""
    dt = gyro_dt(0.7, np.sqrt(3.0))
    return dict(name="abc_ffA1_65536ptl_10000steps", system_type=2, nptl=nptl, steps=steps,
                dt=dt, lo=(0.0, 0.0, 0.0), hi=(1.0, 1.0, 1.0), abc=(1.0, 1.0, 1.0), B0=1.0,
                lambda0=2 * np.pi, nbins=200, emin=1e-3, emax=1e2, nt_out=steps // 1000,
                speed=0.7, seed=seed)


def config_grid(nptl=1048576, steps=5000, n=512, dx=0.25, seed=12):
    """Gridded PIC-style E, B: n^3 nodes, spacing dx (gyroradius ~4 cells),
    B = z + dB with rms dB = 0.5 from 512 Kolmogorov modes, |n| in [1, 64]
    (>= 8 cells per wavelength), velocity rms 0.1 from another 512 modes,
    E = -v x B at the nodes; |v| = 0.7c; dt = 0.01 gyroperiod at B0."""
    L = (n - 1) * dx
    return dict(name="pic_grid_%d^3_%dptl_%dsteps" % (n, nptl, steps), system_type=4, nptl=nptl,
                steps=steps, dt=gyro_dt(0.7, 1.0), n=n, dx=dx, lo=(0.0, 0.0, 0.0), hi=(L, L, L),
                nmodes=512, kmin=1.0, kmax=64.0, dB=0.5, v_rms=0.1, nbins=200, emin=1e-3,
                emax=1e2, nt_out=10, speed=0.7, seed=seed)


def config_modesum(nptl=4194304, steps=20000, seed=13):
    """Analytic turbulence: 512 plane waves, k in [2 pi, 2 pi 64] (L = 1),
    Kolmogorov amplitudes, dB/B0 = 1, B0 = 1 along z, E = -v_A k^ x dB with
    v_A = 0.1; |v| = 0.7c; dt = 0.01 gyroperiod at B0."""
    return dict(name="modesum_512modes_%dptl_%dsteps" % (nptl, steps), system_type=5, nptl=nptl,
                steps=steps, dt=gyro_dt(0.7, 1.0), lo=(0.0, 0.0, 0.0), hi=(1.0, 1.0, 1.0),
                nmodes=512, kmin=1.0, kmax=64.0, dB=1.0, va=0.1, B0=1.0, nbins=200, emin=1e-3,
                emax=1e2, nt_out=steps // 1000, speed=0.7, seed=seed)
