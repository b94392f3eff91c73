"""The onika plugin source compiled on the CPU against stand-in headers of
the onika / exaNBody / exaStamp / yaml-cpp API it uses (tests/onika_stub):
every operator template is instantiated over a grid with and one without a
virial field, and every libgbmd function it calls is one include/gbmd.h
declares and libgbmd.so exports.  (The operators' host logic runs on the
GPU in test_gpu_onika_bridge.py.)"""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PLUGIN = os.path.join(ROOT, "exastamp_gb300", "onika", "gb300_md_ops.cpp")

OPERATORS = ("gb300_force", "gb300_lj_force", "gb300_lj_force_symetric", "gb300_lj_multi_force",
             "gb300_eam_alloy_force", "gb300_johnson_force", "gb300_sutton_chen_force", "gb300_push_f_v_r",
             "gb300_push_f_v",
             "gb300_neighbors", "gb300_sync_grid")


@pytest.fixture(scope="module")
def plugin_object(tmp_path_factory):
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("g++ not found")
    obj = str(tmp_path_factory.mktemp("plugin") / "gb300_md_ops.o")
    r = subprocess.run([gxx, "-std=c++17", "-c", "-Wall", "-Werror=return-type", "-I",
                        os.path.join(ROOT, "tests", "onika_stub"), "-I", os.path.join(ROOT, "include"), PLUGIN,
                        "-o", obj], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]
    return obj


def _symbols(obj):
    out = subprocess.run(["nm", "-C", obj], capture_output=True, text=True, check=True).stdout
    return out.splitlines()


def test_every_operator_instantiated_for_both_grid_flavours(plugin_object):
    lines = _symbols(plugin_object)
    text = "\n".join(lines)
    for cls in ("Gb300ForceNode", "Gb300LJForceNode", "Gb300LJMultiForceNode", "Gb300EamAlloyForceNode",
                "Gb300JohnsonForceNode", "Gb300SuttonChenForceNode", "Gb300PushNode", "Gb300NeighborsNode",
                "Gb300SyncGridNode"):
        for flavour in ("StubGrid<false>", "StubGrid<true>"):
            assert any(cls + "<exanb::" + flavour in ln and "::execute()" in ln for ln in lines), (cls, flavour)
    src = open(PLUGIN).read()
    for op in OPERATORS:
        assert 'register_factory("%s"' % op in src, op
    assert "gbmd_" in text


def test_plugin_calls_only_declared_and_exported_entry_points(plugin_object, gbmd_lib):
    undef = {ln.split()[-1] for ln in _symbols(plugin_object) if " U gbmd_" in ln}
    assert {"gbmd_update_neighbors", "gbmd_push_f_v_r", "gbmd_compute_forces", "gbmd_upload_atoms"} <= undef
    declared = set(gbmd_lib.declared_symbols())
    assert undef <= declared, undef - declared
    out = subprocess.run(["nm", "-D", "--defined-only", gbmd_lib.LIB_PATH], capture_output=True, text=True).stdout
    exported = {ln.split()[-1] for ln in out.splitlines() if " T " in ln}
    assert undef <= exported
