"""Build libtpgpu.so (CUDA for sm_103a + host C ABI) in-tree.

nvcc cross-compiles without a GPU; the translation units compile in parallel.
The FP64 tracking unit is compiled twice: without FMA contraction (the parity
path, reference arithmetic) and with it (the fast FP64 path).
"""
import concurrent.futures as cf
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libtpgpu.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC = os.environ.get("NVCC", shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc")
COMMON = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall",
                 "--expt-relaxed-constexpr"]

# (output object, source, extra flags)
UNITS = [
    ("track_fp64.o", "track_fp64.cu", ["-fmad=false"]),
    ("track_fp64fast.o", "track_fp64.cu", ["-fmad=true", "-DTP_FP64_NS=fp64fast"]),
    ("track_mixed.o", "track_mixed.cu", ["-fmad=true", "-ftz=true"]),
    ("mixed_host.o", "mixed_host.cu", []),
    ("capi.o", "capi.cu", []),
    ("session.o", "session.cu", []),
    ("ref_api.o", "ref_api.cu", []),
    ("bs.o", "bs.cu", []),
    ("synth.o", "synth.cu", []),
    ("mlp.o", "mlp.cu", []),
    ("track_surrogate.o", "track_surrogate.cu", ["-fmad=true", "-ftz=true"]),
    ("host_config.o", "host_config.cpp", ["-x", "cu"]),
    ("noalloc.o", "noalloc.cu", []),
    ("tc_gemm.o", "tc_gemm.cu", []),
    ("tc_train.o", "tc_train.cu", []),
    ("poincare.o", "poincare.cu", []),
    ("loaders.o", "loaders.cu", []),
    ("h5lite.o", "h5lite.cpp", []),
    ("h5io.o", "h5io.cu", []),
    ("peaks.o", "peaks.cu", []),
]


def _sources_mtime():
    m = 0.0
    for fn in os.listdir(CSRC):
        m = max(m, os.path.getmtime(os.path.join(CSRC, fn)))
    inc = os.path.join(os.path.dirname(HERE), "include")
    for fn in os.listdir(inc):
        m = max(m, os.path.getmtime(os.path.join(inc, fn)))
    return max(m, os.path.getmtime(__file__))


def _compile(unit):
    obj, src, extra = unit
    out = os.path.join(BUILD, obj)
    cmd = [NVCC] + COMMON + extra + ["-c", os.path.join(CSRC, src), "-o", out]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, " ".join(cmd), r.stderr))
    return out


def build(force=False, verbose=False):
    """Compile every CUDA unit for sm_103a and link libtpgpu.so; returns its path."""
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= _sources_mtime():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=min(len(UNITS), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(_compile, UNITS))
    tmp = LIB + ".%d.tmp" % os.getpid()
    cmd = [NVCC] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart_static", "-ldl"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s\n%s" % (" ".join(cmd), r.stderr))
    os.replace(tmp, LIB)
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    build(force=True, verbose=True)
