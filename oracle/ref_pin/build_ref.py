"""Recipe for oracle/_ref/libref.so: the reference's own per-pair code,
compiled from the exaStamp sources where they lie, for pinning the oracle.

Compiled from the exaStamp tree (EXASTAMP_ROOT, default /root/reference):
  src/potential/eam_potentials/eam_alloy/eam_alloy.cpp       (setfl reader, splines)
and, through oracle/ref_pin/ref_shim.cpp (this build's C entry points):
  src/potential/pair_potentials/lennard_jones/include/.../lennard_jones.h
  src/potential/pair_potential_template/force_op_impl2.hxx
  src/potential/eam_potentials/eam_alloy/eam_alloy.h
  include/exaStamp/unit_system.h
The onika / exaNBody / yaml-cpp headers they include are replaced by the
stand-ins in oracle/ref_pin/stubs (nothing else of the reference's build is
used: no CMake, no generated code).  g++ -O2 -ffp-contract=off, so the
reference arithmetic is evaluated as written, like the oracle's.

Test infrastructure only: the output goes to oracle/_ref/ (not committed),
the library is loaded by tests/test_ref_pin.py and tests/golden/make_ref_pin.py
and never by the product.

    python oracle/ref_pin/build_ref.py [--force]
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE = os.path.dirname(HERE)
OUT_DIR = os.path.join(ORACLE, "_ref")
LIB = os.path.join(OUT_DIR, "libref.so")


def reference_root() -> str:
    return os.environ.get("EXASTAMP_ROOT", "/root/reference")


def sources(root: str):
    return [os.path.join(HERE, "ref_shim.cpp"),
            os.path.join(root, "src", "potential", "eam_potentials", "eam_alloy", "eam_alloy.cpp")]


def includes(root: str):
    return [os.path.join(HERE, "stubs"),
            os.path.join(root, "include"),
            os.path.join(root, "src", "potential", "pair_potentials", "lennard_jones", "include"),
            os.path.join(root, "src", "potential", "eam_potentials", "eam_alloy"),
            os.path.join(root, "src", "potential", "pair_potential_template")]


def available(root: str | None = None) -> bool:
    root = root or reference_root()
    return all(os.path.exists(s) for s in sources(root)) and shutil.which("g++") is not None


def build(force: bool = False) -> str | None:
    """Build oracle/_ref/libref.so when the exaStamp sources are readable;
    returns its path, or None when they are not (nothing to pin against)."""
    root = reference_root()
    if not available(root):
        return None
    srcs = sources(root)
    stubs = [os.path.join(dp, f) for dp, _, fs in os.walk(os.path.join(HERE, "stubs")) for f in fs]
    if (not force and os.path.exists(LIB)
            and os.path.getmtime(LIB) >= max(os.path.getmtime(p) for p in srcs + stubs + [__file__])):
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = ["g++", "-O2", "-ffp-contract=off", "-std=c++17", "-fPIC", "-shared", "-w"]
    for inc in includes(root):
        cmd += ["-I", inc]
    cmd += srcs + ["-o", tmp]
    subprocess.check_call(cmd)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    p = build(force="--force" in sys.argv)
    print(p if p else "exaStamp sources not found: nothing built")
