"""The oracle restatement against golden vectors produced by the reference's own
C sources (tests/golden/make_golden.py).  Bit-exact: same operation order,
no FMA contraction, same libm."""
import json

import numpy as np
import pytest

import make_golden as mg
from oracle import pyoracle as po

G = mg.HERE
SC = mg.scenarios()
NAMES = ("test", "ff_vel", "abc111", "mhd", "pic", "pic_mt", "pic_off", "wlcs", "loop")


def load(name):
    return np.load("%s/%s.npz" % (G, name))


def same_particles(a, b):
    return all(np.array_equal(a[k], b[k], equal_nan=True) for k in a.dtype.names)


@pytest.mark.parametrize("name", NAMES)
def test_get_emf_bitexact(name):
    emf = load("emf")
    f = mg.field_from(SC[name])
    out = po.get_emf(f, emf[name + "_xyzt"])
    assert np.array_equal(out, emf[name + "_emf"], equal_nan=True)


def test_trilinear_bitexact():
    tl = load("trilinear")
    c, w = po.trilinear(mg.field_from(SC["pic_off"]), tl["xyzt"])
    assert np.array_equal(c, tl["corners"])
    assert np.array_equal(w, tl["weights"])


def test_ellint_bitexact():
    el = load("ellint")
    e, k = po.ellint(el["k"])
    assert np.array_equal(e, el["E"]) and np.array_equal(k, el["K"])


@pytest.mark.parametrize("name", NAMES)
@pytest.mark.parametrize("nsteps", [1, 40])
def test_wirz_bitexact(name, nsteps):
    wz = load("wirz")
    f = mg.field_from(SC[name], bc_flag=2 if name in ("wlcs", "loop") else 0)
    out, _ = po.wirz_steps(f, wz[name + "_in"], float(wz[name + "_dt"]), nsteps)
    assert same_particles(out, wz["%s_out%d" % (name, nsteps)])


def test_energy_bins_bitexact():
    eb = load("ebins")
    s = po.spectrum(int(eb["nbins"]), float(eb["emin"]), float(eb["emax"]))
    assert np.array_equal([s.emin, s.emax, s.logemin, s.logemax, s.logde], eb["globals"])
    assert np.array_equal(po.energy_bins(s, eb["ptl"]), eb["bins"])


def test_calc_diff_coeff_bitexact():
    dc = load("diffcoeff")
    out = po.calc_diff_coeff(mg.field_from(SC["ff_vel"]), dc["p0"], dc["p"], float(dc["dt"]))
    assert np.array_equal(out, dc["out"])


@pytest.mark.parametrize("case", range(7))
def test_track_fixed_bitexact(case):
    tr = load("track")
    key = "case%d_" % case
    m = json.loads(str(tr[key + "meta"]))
    s2 = dict(SC[m["name"]])
    d = po.Domain.from_buffer_copy(s2["dom"])
    d.tmax = m["tmax"]
    s2["dom"] = d
    f = mg.field_from(s2, bc_flag=m["bc"])
    sp = po.spectrum(m["nbins"], m["emin"], m["emax"])
    o = po.track_fixed(f, sp, tr[key + "ptl0"], m["dt"], m["nt_out"], nthreads=1)
    assert same_particles(o["ptl"], tr[key + "ptl"])
    assert np.array_equal(o["espect"], tr[key + "espect"])
    assert np.array_equal(o["espect_escape"], tr[key + "espect_escape"])
    assert np.array_equal(o["dsum"], tr[key + "dsum"])
    assert np.array_equal(o["remain"], tr[key + "remain"])
    assert np.array_equal(o["nsteps"], tr[key + "nsteps"])


def test_track_threads_agree():
    """Threaded oracle runs give the same particles and counts; sums agree to rounding."""
    tr = load("track")
    m = json.loads(str(tr["case1_meta"]))
    s2 = dict(SC[m["name"]])
    d = po.Domain.from_buffer_copy(s2["dom"])
    d.tmax = m["tmax"]
    s2["dom"] = d
    f = mg.field_from(s2)
    sp = po.spectrum(m["nbins"], m["emin"], m["emax"])
    a = po.track_fixed(f, sp, tr["case1_ptl0"], m["dt"], m["nt_out"], nthreads=1)
    b = po.track_fixed(f, sp, tr["case1_ptl0"], m["dt"], m["nt_out"], nthreads=4)
    assert same_particles(a["ptl"], b["ptl"])
    assert np.array_equal(a["espect"], b["espect"])
    np.testing.assert_allclose(a["dsum"], b["dsum"], rtol=1e-13, atol=0)


def test_bs_bitexact():
    bs = load("bs")
    f = mg.field_from(SC["loop"], bc_flag=2)
    for i in range(len(bs["y0"])):
        o = po.bs_integrate(f, bs["y0"][i], 0.0, float(bs["h0"][i]), bs["out"].shape[1])
        assert np.array_equal(o, bs["out"][i], equal_nan=True)


@pytest.mark.parametrize("name", ["mhd", "pic", "pic_off"])
def test_poincare_rk4_steps_bitexact(name):
    """The field-line RK4 step (src/poincare_map.c:243-290) against the
    reference's next_location, 40 steps from 32 seeds, wrap included."""
    pc = load("poincare")
    f = mg.field_from(SC[name])
    got = po.next_location_steps(f, pc[name + "_seeds"], float(pc[name + "_step"]), 40)
    assert np.array_equal(got, pc[name + "_traj"])


def test_poincare_crossings_follow_the_steps():
    """The crossing loop (src/poincare_map.c:158-181): every recorded point is
    the first step after a sign change of pos[face] - seed[face], found by
    replaying the RK4 steps; unfilled entries keep the fill value 2 * max."""
    f = mg.field_from(SC["pic"])
    d = SC["pic"]["dom"]
    rng = np.random.default_rng(4)
    seeds = np.array([d.xmin, d.ymin, d.zmin]) + rng.uniform(0, 1, size=(6, 3)) * \
        np.array([d.xmax - d.xmin, d.ymax - d.ymin, d.zmax - d.zmin])
    step, lmax, ncross, face = 0.05, 60.0, 5, 1
    xo, yo, zo, found = po.poincare(f, seeds, face, step, lmax, ncross)
    nsteps = int(np.ceil(lmax / step)) + 1
    for i in range(len(seeds)):
        traj = po.next_location_steps(f, seeds[i], step, nsteps)[0]
        init = seeds[i, face]
        pre = np.concatenate([[seeds[i, face]], traj[:-1, face]])
        hits = np.nonzero((pre - init) * (traj[:, face] - init) <= 0)[0]
        # the loop tests cross > 0 after each step, with the length bound
        length = step * (hits + 1)
        hits = hits[length < lmax][:ncross]
        assert found[i] == len(hits)
        assert np.array_equal(xo[i, 1:1 + len(hits)], traj[hits, 0])
        assert np.array_equal(zo[i, 1:1 + len(hits)], traj[hits, 2])
        assert np.all(yo[i, 1 + len(hits):] == 2 * d.ymax)
        assert xo[i, 0] == seeds[i, 0]


def test_field_file_records_restated():
    """The reference's binary readers store float(data * B0) with the product
    in double (src/magnetic_field.c:458-474); the fixture made by them agrees
    with that restatement bit for bit."""
    f = load("fields")
    c = f["comps"]
    b0, e0 = f["scale"]
    rb = (c[:3].T.astype(np.float64) * b0).astype(np.float32).ravel()
    re_ = (c[3:].T.astype(np.float64) * e0).astype(np.float32).ravel()
    assert np.array_equal(rb, f["records_b"]) and np.array_equal(re_, f["records_e"])
