"""CPU checks of the C ABI library: it builds for sm_103a, loads without a GPU
and exports every entry point include/gbmd.h declares; operator-layer slot
validation that needs no device."""
import ctypes
import os
import subprocess

import pytest

from exastamp_gb300 import operators as OP


def test_library_exports_every_declared_symbol(gbmd_lib):
    declared = gbmd_lib.declared_symbols()
    assert len(declared) >= 30
    L = ctypes.CDLL(gbmd_lib.LIB_PATH)
    missing = [s for s in declared if not hasattr(L, s)]
    assert not missing, missing
    out = subprocess.run(["nm", "-D", "--defined-only", gbmd_lib.LIB_PATH], capture_output=True, text=True).stdout
    exported = {ln.split()[-1] for ln in out.splitlines() if " T " in ln}
    assert set(declared) <= exported


def test_abi_version(gbmd_lib):
    assert gbmd_lib.lib().gbmd_abi_version() == 1


def test_no_fallback_without_device(gbmd_lib):
    """On a machine without a GPU the library refuses to create a context
    (there is no CPU path behind the ABI)."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("GPU present")
    h = ctypes.c_void_p()
    rc = gbmd_lib.lib().gbmd_create(ctypes.byref(h), 0, None)
    assert rc in (2, 3)


def test_quantity_units():
    assert OP.quantity("5 ang") == 5.0
    assert abs(OP.quantity("1 eV") - 1.602176634e-19 / 1.66053906660e-23) < 1e-9
    assert OP.quantity(2.5) == 2.5
    with pytest.raises(OP.OperatorError):
        OP.quantity("3 furlong")


def test_required_slots_raise():
    with pytest.raises(OP.OperatorError):
        OP.lj_compute_force(parameters={"epsilon": 1.0, "sigma": 1.0})
    with pytest.raises(OP.OperatorError):
        OP.eam_alloy_force(rcut=5.0)
    with pytest.raises(OP.OperatorError):
        OP.compute_force_from_config({"compute_force": "nop"})
    op = OP.compute_force_from_config({"compute_force": "lj_compute_force",
                                       "lj_compute_force": {"rcut": "2.5 ang",
                                                            "parameters": {"epsilon": 1.0, "sigma": 1.0}}})
    assert isinstance(op, OP.lj_compute_force)


def test_header_is_plain_c():
    """include/gbmd.h compiles as C (no torch or C++ types in the ABI)."""
    hdr = os.path.join(os.path.dirname(os.path.dirname(__file__)), "include", "gbmd.h")
    r = subprocess.run(["gcc", "-std=c99", "-fsyntax-only", "-x", "c", hdr], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
