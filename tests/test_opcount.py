"""The per-push operation count of the FP64 path (oracle/opcount.py): its
restatement of the Wirz push reproduces the oracle bit for bit on plain
floats, and the counts are pinned."""
import numpy as np

import make_golden as mg
from oracle import opcount as oc
from oracle import pyoracle as po

SC = mg.scenarios()


def test_restatement_matches_oracle_bitexact():
    s = SC["abc111"]
    A, B, C = s["abc"]
    f = mg.field_from(s)
    p0 = mg.particles_for(s, np.random.default_rng(2), 16)
    dt = 0.02
    ref, _ = po.wirz_steps(f, p0, dt, 1)
    for i in range(len(p0)):
        q = [float(p0[k][i]) for k in ("x", "y", "z", "ux", "uy", "uz", "t")]
        got = oc.wirz(q, dt, s["charge_mass"],
                      lambda x, y, z, t: oc.abc_field(x, y, z, A, B, C, s["B0"], s["lambda0"]))
        # or_wirz_steps applies the periodic boundary after the push
        for k, v in zip(("ux", "uy", "uz", "t"), got[3:]):
            assert v == ref[k][i], k
        for k, v, sh in zip(("x", "y", "z"), got[:3], ("xshift", "yshift", "zshift")):
            assert v == ref[k][i] + ref[sh][i] - p0[sh][i], k


def test_counts_pinned():
    """One push: 90 add/sub + 154 mul + 12 div + 8 sqrt + 8 sin + 8 cos, of
    which two ABC field evaluations take 2 x (3 add + 15 mul + 3 sin + 3 cos);
    the Wirz step alone is 84 add + 124 mul + 12 div + 8 sqrt + 2 sin + 2 cos."""
    push, field = oc.count_abc_push()
    assert field == {"add": 3, "mul": 15, "div": 0, "sqrt": 0, "sin": 3, "cos": 3}
    assert push == {"add": 90, "mul": 154, "div": 12, "sqrt": 8, "sin": 8, "cos": 8}
