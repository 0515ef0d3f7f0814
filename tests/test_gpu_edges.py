"""Edge cases of the tracking entry point against the oracle: no particles,
one particle with the smallest spectrum (3 bins) and a diagnostic frame every
step, and spectra too wide for the per-block shared histogram (global
atomics).  The uniform field (system 0) keeps orbits regular, so the FP64
path stays within rounding of the oracle and energy bins are exact."""
import numpy as np
import pytest

import make_golden as mg
from oracle import pyoracle as po

pytestmark = pytest.mark.gpu
tp = pytest.importorskip("test_particle_gb300")
SC = mg.scenarios()


def setup_test_field(steps, dt, bc=0):
    s = SC["test"]
    d = po.Domain.from_buffer_copy(s["dom"])
    d.tmax = steps * dt + 0.5 * dt
    tp.configure(system_type=0, charge_mass=1.0, bc_flag=bc, dom=d, grd=s["grd"])
    f = po.make_field(system_type=0, charge_mass=1.0, bc_flag=bc, dom=d, grd=s["grd"])
    return f


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_no_particles(prec):
    setup_test_field(250, 0.05)
    tp.set_spectrum(50, 1e-3, 1e1)
    p0 = np.zeros(0, dtype=tp.PARTICLE_DTYPE)
    code = tp.PREC_FP64 if prec == "fp64" else tp.PREC_MIXED
    out = tp.track(p0, 0.05, 5, 50, precision=code)
    assert out["espect"].sum() == 0 and out["espect_escape"].sum() == 0
    assert np.all(out["dsum"] == 0) and np.all(out["remain"] == 0)
    assert len(out["ptl"]) == 0
    assert tp.device_status() == 0


def test_one_particle_three_bins_every_step():
    steps, dt = 60, 0.05
    f = setup_test_field(steps, dt)
    tp.set_spectrum(3, 1e-2, 1e1)
    s = po.spectrum(3, 1e-2, 1e1)
    p0 = mg.particles_for(SC["test"], np.random.default_rng(9), 1)
    out = tp.track(p0, dt, steps, 3, precision=tp.PREC_FP64)  # einterval = 1
    ref = po.track_fixed(f, s, p0, dt, steps)
    assert np.array_equal(out["espect"], ref["espect"])
    assert np.array_equal(out["nsteps"], ref["nsteps"])
    assert np.array_equal(out["remain"], ref["remain"])
    for k in ("x", "y", "z", "ux", "uy", "uz"):
        np.testing.assert_allclose(out["ptl"][k], ref["ptl"][k], rtol=1e-11, atol=1e-13)
    assert np.array_equal(out["ptl"]["t"], ref["ptl"]["t"])
    assert tp.device_status() == 0


@pytest.mark.parametrize("nbins", [4096, 6000])
def test_wide_spectra(nbins):
    """4096 bins: the largest shared-memory histogram; 6000: global atomics."""
    steps, dt = 200, 0.05
    f = setup_test_field(steps, dt, bc=1)
    tp.set_spectrum(nbins, 1e-4, 1e2)
    s = po.spectrum(nbins, 1e-4, 1e2)
    rng = np.random.default_rng(12)
    p0 = mg.particles_for(SC["test"], rng, 1000)
    # spread the energies over the bins
    scale = np.exp(rng.uniform(-4, 2, len(p0)))
    for k in ("ux", "uy", "uz"):
        p0[k] *= scale
    out = tp.track(p0, dt, 4, nbins, precision=tp.PREC_FP64)
    ref = po.track_fixed(f, s, p0, dt, 4)
    assert np.array_equal(out["espect"], ref["espect"])
    assert np.array_equal(out["espect_escape"], ref["espect_escape"])
    assert np.array_equal(out["remain"], ref["remain"])
    assert ref["espect_escape"].sum() > 0
    assert tp.device_status() == 0
