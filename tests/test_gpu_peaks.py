"""The FMA-chain microbenchmark behind the compute-bound rooflines
(tp_measure_fma_peak): plausible rates for a 152-SM part at boost clock
(FP32: 152 SMs x 128 lanes x 2 FLOP x ~2 GHz ~ 80 TFLOP/s; FP64 far below
it on this part), packed FP32 pairs no slower than scalar FP32, bad kinds
rejected."""
import ctypes as C

import pytest

pytestmark = pytest.mark.gpu
tp = pytest.importorskip("test_particle_gb300")


def test_fma_peaks_are_plausible():
    pk = tp.measure_fma_peaks()
    assert 20e12 < pk["fp32"] < 200e12, pk
    assert 0.05e12 < pk["fp64"] < pk["fp32"], pk
    assert pk["fp32x2"] > 0.8 * pk["fp32"], pk


def test_bad_kind_is_an_error():
    v = C.c_double()
    assert tp.lib().tp_measure_fma_peak(C.c_int(3), C.byref(v)) == -1
    tp.lib().tp_clear_status()
