"""CPU checks of the C ABI library: it builds for sm_103a, loads without a GPU
and exports every entry point include/gbmd.h declares; operator-layer slot
validation that needs no device."""
import ctypes
import os
import subprocess

import numpy as np
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


def test_entry_points_refuse_a_null_context(gbmd_lib):
    """Argument checks that need no device: every setter and getter of the
    list buffer, the Newton-3 switch and the error check answer
    GBMD_ERR_INVALID (1) for a null context, before any CUDA call."""
    L = gbmd_lib.lib()
    d, k = ctypes.c_double(), ctypes.c_int64()
    assert L.gbmd_set_list_buffer(None, ctypes.c_double(1.0)) == 1
    assert L.gbmd_get_list_buffer(None, ctypes.byref(d), ctypes.byref(k)) == 1
    assert L.gbmd_check_errors(None) == 1
    assert L.gbmd_set_newton3(None, 1) == 1
    assert L.gbmd_set_eam_sutton_chen(None, None, ctypes.c_double(5.0)) == 1


def test_quantity_units():
    assert OP.quantity("5 ang") == 5.0
    assert abs(OP.quantity("1 eV") - 1.602176634e-19 / 1.66053906660e-23) < 1e-9
    assert OP.quantity(2.5) == 2.5
    with pytest.raises(OP.OperatorError):
        OP.quantity("3 furlong")


def test_sutton_chen_regression_parameters_in_internal_units():
    """The run file's quantities (single_specy.msp L8-13) convert to the
    parameter vector the tests use; a missing parameter is refused."""
    from exastamp_gb300 import systems as S
    got = [OP.quantity(v) for v in (3.317e01, "3.605e-21 J", "0.327e-09 m", 9.050, 5.005)]
    assert np.allclose(got, S.sutton_chen_cu_params(), rtol=1e-15, atol=0.0)
    assert S.SUTTON_CHEN_PARAM_NAMES == ("c", "epsilon", "a0", "n", "m")
    op = OP.compute_force_from_config({"compute_force": "sutton_chen_force",
                                       "sutton_chen_force": {"rcut": "7.29 ang",
                                                             "parameters": {"c": 1.0, "epsilon": 1.0}}})
    assert isinstance(op, OP.sutton_chen_force)
    with pytest.raises(OP.OperatorError):
        op.bind(None)


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
    op = OP.compute_force_from_config({"compute_force": "lj_compute_force_symetric",
                                       "lj_compute_force_symetric": {"rcut": 2.5}})
    assert isinstance(op, OP.lj_compute_force_symetric) and op.name == "lj_compute_force_symetric"


def test_header_is_plain_c():
    """include/gbmd.h compiles as C (no torch or C++ types in the ABI)."""
    hdr = os.path.join(os.path.dirname(os.path.dirname(__file__)), "include", "gbmd.h")
    r = subprocess.run(["gcc", "-std=c99", "-fsyntax-only", "-x", "c", hdr], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_dump_thermodynamic_state_columns(oracle, tmp_path):
    """The thermo CSV line: 21 columns in the reference's order and formats,
    total = kinetic + potential per particle, temperature from the kinetic
    energy without the centre-of-mass term, cubic-box geometry."""
    import types

    import numpy as np

    from exastamp_gb300 import operators as O
    from exastamp_gb300 import systems as S

    s = S.eam_cu_fcc(ncell=3, T=300.0, seed=5)
    th = oracle.thermo(s.vx, s.vy, s.vz, np.full(s.n, -3.0 * S.EV), np.zeros((s.n, 9)), s.type, s.masses)
    vol = float(np.prod(s.hi - s.lo))
    st = O.ThermodynamicState(th, vol)
    sim = types.SimpleNamespace(lo=s.lo, hi=s.hi, volume=vol)
    op = O.dump_thermodynamic_state(thermostate_file=str(tmp_path / "thermo.csv"))
    line = op.execute(sim, st, timestep=10, physical_time=0.01)
    text = (tmp_path / "thermo.csv").read_text().splitlines()
    assert text[0] == O.THERMO_HEADER and text[1] == line
    cols = [float(v) for v in line.split()]
    assert len(cols) == 21 and cols[0] == 10 and cols[2] == s.n
    assert abs(cols[3] - (cols[4] + cols[5])) < 1e-9 * abs(cols[3])
    assert abs(cols[5] + 3.0) < 1e-9
    assert abs(cols[6] - 300.0) < 30.0  # Maxwell-Boltzmann draw of 108 atoms
    assert cols[13:16] == [float(s.hi[0] - s.lo[0])] * 3 and cols[16:19] == [90.0] * 3
    assert abs(cols[20] - O.THERMO_CONV_DENSITY * s.masses[0] * s.n / vol) < 1e-9
