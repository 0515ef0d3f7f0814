"""Poincare maps (src/poincare_map.c) on the GPU: field lines of the gridded
B traced with the reference's RK4 step in FP64 without FMA contraction, so
the crossings are the oracle's bit for bit (gridded interpolation has no
transcendental functions), for periodic wraps and ragged seed counts."""
import numpy as np
import pytest

import make_golden as mg
from oracle import pyoracle as po

pytestmark = pytest.mark.gpu
tp = pytest.importorskip("test_particle_gb300")
SC = mg.scenarios()


def configure(name):
    s = SC[name]
    tp.configure(system_type=s["system_type"], charge_mass=s["charge_mass"], dom=s["dom"],
                 grd=s["grd"], mt=s["mt"], vgrid_f=s.get("vgrid_f"), bgrid=s.get("bgrid"),
                 egrid=s.get("egrid"))


def seeds_in(name, n, seed):
    d = SC[name]["dom"]
    lo = np.array([d.xmin, d.ymin, d.zmin])
    hi = np.array([d.xmax, d.ymax, d.zmax])
    return lo + np.random.default_rng(seed).uniform(0, 1, size=(n, 3)) * (hi - lo), hi - lo


@pytest.mark.parametrize("name,face", [("mhd", 0), ("pic", 1), ("pic_off", 2)])
def test_poincare_matches_oracle_bitexact(name, face):
    configure(name)
    seeds, span = seeds_in(name, 131, 5)  # a ragged block count
    step = 0.02 * float(span.min())
    lmax, ncross = 400 * step, 6
    got = tp.poincare_trace(seeds, face, step, lmax, ncross)
    ref = po.poincare(mg.field_from(SC[name]), seeds, face, step, lmax, ncross)
    for g, r in zip(got, ref):
        assert np.array_equal(g, r)
    assert got[3].max() > 0  # some field lines cross the plane
    assert tp.device_status() == 0


def test_poincare_bad_arguments_are_errors():
    configure("pic")
    seeds, span = seeds_in("pic", 4, 1)
    with pytest.raises(RuntimeError):
        tp.poincare_trace(seeds, 3, 0.01, 1.0, 2)
    with pytest.raises(RuntimeError):
        tp.poincare_trace(seeds, 0, 0.0, 1.0, 2)
    configure("abc111")
    with pytest.raises(RuntimeError):
        tp.poincare_trace(seeds, 0, 0.01, 1.0, 2)
