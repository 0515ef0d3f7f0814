"""The reference's own program links against libtpgpu.so in place of its
tracking, emfields, interpolation, force_free, wlcs, poincare_map and data_io objects
(test_particle_gb300/link_reference.sh).  Needs the reference tree (read only)
and a compiler; linking needs no GPU."""
import os
import shutil
import subprocess

import pytest

from oracle import pyoracle as po

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = po.reference_dir()


@pytest.mark.skipif(REF is None, reason="reference tree absent: set TP_REFERENCE_DIR to it, or build "
                                         "oracle/_ref from it first (oracle/build_ref.sh)")
@pytest.mark.skipif(shutil.which("gcc") is None or shutil.which("objcopy") is None,
                    reason="gcc/objcopy absent")
def test_reference_program_links_against_library(tmp_path):
    from test_particle_gb300 import build as b
    lib = b.build()
    env = dict(os.environ, REF=REF, CC="gcc", OUT=str(tmp_path),
               CFLAGS="-I" + os.path.join(ROOT, "oracle", "stubs"))
    r = subprocess.run([os.path.join(ROOT, "test_particle_gb300", "link_reference.sh")],
                       env=env, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    exe = tmp_path / "test_particle"
    assert exe.exists()
    und = subprocess.run(["nm", "-D", "--undefined-only", str(exe)], capture_output=True,
                         text=True).stdout.split("\n")
    need = {ln.split()[-1] for ln in und if ln.strip() and "@" not in ln and " w " not in ln}
    exported = set()
    for ln in subprocess.run(["nm", "-D", "--defined-only", lib], capture_output=True,
                             text=True).stdout.split("\n"):
        parts = ln.split()
        if len(parts) == 3:
            exported.add(parts[2])
    # every hot-path function the reference's program calls comes from the library
    for name in ("particle_tracking_hybrid", "set_variables_tracking", "set_ptl_params_tracking",
                 "set_variables_emfields", "get_emf", "getemf_ff",
                 "getemf_wlcs", "get_trilinar_parameters", "get_param_ff", "read_wlcs",
                 "free_config", "adjust_dt_normI", "get_tracking_time_interval", "poincare_map",
                 "read_data_serial_float_h5", "read_data_serial_double_h5", "read_data_serial_float_binary",
                 "read_data_serial_double_binary"):
        assert name in need, name
    assert need <= exported, sorted(need - exported)
