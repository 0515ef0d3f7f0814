"""The tensor-core building blocks (tcgen05.mma with BF16 operands in
128-byte-swizzled shared memory, FP32 accumulation in tensor memory) against
an FP64 product of the same BF16 values, through tp_tc_gemm_bf16."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
tp = pytest.importorskip("test_particle_gb300")


def bf16_bits(a):
    u = np.asarray(a, dtype=np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) >> 16
    return u.astype(np.uint16)


def bits_to_f64(b):
    return (b.astype(np.uint32) << 16).view(np.float32).astype(np.float64)


@pytest.mark.parametrize("n,k", [(256, 256), (16, 256), (256, 128), (64, 64), (128, 192)])
def test_tile_gemm_matches_fp64(n, k):
    rng = np.random.default_rng(n * 1000 + k)
    a = bf16_bits(rng.uniform(-1, 1, size=(128, k)))
    b = bf16_bits(rng.uniform(-1, 1, size=(n, k)))
    d = np.zeros((128, n), dtype=np.float32)
    L = tp.lib()
    L.tp_tc_gemm_bf16.restype = C.c_int
    u16 = C.POINTER(C.c_uint16)
    rc = L.tp_tc_gemm_bf16(n, k, a.ctypes.data_as(u16), b.ctypes.data_as(u16),
                           d.ctypes.data_as(C.POINTER(C.c_float)))
    assert rc == 0
    ref = bits_to_f64(a) @ bits_to_f64(b).T
    # FP32 accumulation of k products of BF16 values
    assert np.abs(d - ref).max() <= 1e-5 * np.abs(ref).max(), np.abs(d - ref).max()
    assert tp.device_status() == 0


@pytest.mark.parametrize("m,n,k", [(128, 256, 256), (256, 16, 256), (384, 128, 640), (256, 256, 64),
                                   (128, 48, 4096), (640 * 128, 256, 256), (1024, 256, 128)])
def test_training_gemm_matches_fp64(m, n, k):
    """The training GEMM kernels: the ring of k-atoms through shared memory
    with one tcgen05.mma chain per 128-row tile (several tiles, long K), and,
    for N = 256 and K <= 256, the persistent warp-specialised kernel (B
    resident, two accumulators in tensor memory; 640 tiles: several per
    block, both accumulators reused)."""
    rng = np.random.default_rng(m * 7 + n * 1000 + k)
    a = bf16_bits(rng.uniform(-1, 1, size=(m, k)))
    b = bf16_bits(rng.uniform(-1, 1, size=(n, k)))
    d = np.zeros((m, n), dtype=np.float32)
    L = tp.lib()
    L.tp_tc_gemm_train_bf16.restype = C.c_int
    u16 = C.POINTER(C.c_uint16)
    rc = L.tp_tc_gemm_train_bf16(m, n, k, a.ctypes.data_as(u16), b.ctypes.data_as(u16),
                                 d.ctypes.data_as(C.POINTER(C.c_float)))
    assert rc == 0
    ref = bits_to_f64(a) @ bits_to_f64(b).T
    # FP32 accumulation of k products of BF16 values: |error| <= k 2^-24 sum |a b|
    bound = k * 2.0 ** -24 * (np.abs(bits_to_f64(a)) @ np.abs(bits_to_f64(b)).T)
    assert np.all(np.abs(d - ref) <= bound + 1e-30), np.abs(d - ref).max()
    assert tp.device_status() == 0


def test_training_gemm_rejects_bad_shapes():
    L = tp.lib()
    L.tp_tc_gemm_train_bf16.restype = C.c_int
    z = np.zeros(1, dtype=np.uint16).ctypes.data_as(C.POINTER(C.c_uint16))
    d = np.zeros(1, dtype=np.float32).ctypes.data_as(C.POINTER(C.c_float))
    for m, n, k in ((100, 16, 64), (128, 8, 64), (128, 272, 64), (128, 16, 96)):
        assert L.tp_tc_gemm_train_bf16(m, n, k, z, z, d) != 0
    tp.lib().tp_clear_status()
