"""The onika plugin's host logic (exastamp_gb300/onika/gb300_bridge.h) on the
CPU, over a stand-in of the libgbmd entry points it calls
(tests/onika_bridge/bridge_cpu_check.cpp, compiled here with g++): the box
and coordinates of a domain with a diagonal xform, layout-change detection,
the resident mode's write-back, a rescale between calls (synced back with
the old scale, uploaded again with the new one), and device errors
stopping a call.  The same logic runs over the real library on the GPU in
test_gpu_onika_bridge.py."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_bridge_host_logic_over_a_stand_in_library(tmp_path):
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("g++ not found")
    exe = str(tmp_path / "bridge_cpu_check")
    subprocess.run([gxx, "-std=c++17", "-O1", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"), "-I",
                    os.path.join(ROOT, "exastamp_gb300", "onika"),
                    os.path.join(ROOT, "tests", "onika_bridge", "bridge_cpu_check.cpp"), "-o", exe], check=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.strip() == "ok"
