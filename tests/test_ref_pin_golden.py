"""The oracle against vectors the reference's own code produced
(tests/golden/ref_pin_vectors.json, written by tests/golden/make_ref_pin.py
from oracle/_ref/libref.so, which is compiled from the exaStamp sources):
lj_compute_energy (lennard_jones.h L41-50), the per-atom loop of
lj_compute_force (force_op_impl2.hxx L22-78), the setfl spline
(eam_alloy.cpp L29-278) and the eam_alloy lookups (eam_alloy.h L198-313),
all bit for bit.  Needs neither the exaStamp tree nor a GPU."""
import hashlib
import json
import os

import numpy as np
import pytest

from exastamp_gb300 import setfl as SF

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def vec():
    with open(os.path.join(HERE, "golden", "ref_pin_vectors.json")) as fh:
        return json.load(fh)


def dx(v):
    return np.array([float.fromhex(s) for s in v])


def test_lj_pair_matches_reference_vectors(oracle, vec):
    assert len(vec["lj_pair"]) >= 100
    for row in vec["lj_pair"]:
        eps, sig, r, e, de = dx(row)
        assert oracle.lj_pair(eps, sig, r) == (e, de)


def test_lj_per_atom_loop_matches_reference_vectors(oracle, vec):
    for case in vec["lj_atom"]:
        eps, sig, ecut = dx(case["params"])
        got = oracle.lj_atom_buffer(eps, sig, ecut, dx(case["drx"]), dx(case["dry"]), dx(case["drz"]), dx(case["d2"]))
        assert np.array_equal(got, dx(case["out"]))


def test_eam_spline_and_lookups_match_reference_vectors(oracle, vec, tmp_path):
    e = vec["eam"]
    path = str(tmp_path / "cu_analytic.eam.alloy")
    SF.write_setfl(SF.tabulate(SF.load_cu_params()), path)
    with open(path, "rb") as fh:
        if hashlib.sha256(fh.read()).hexdigest() != e["setfl_text_sha256"]:
            pytest.skip("this platform's libm tabulates the analytic functions differently")
    sf = SF.read_setfl(path)
    cz, cf = dx(e["conversions"])
    tab = oracle.EamOracleTables.from_setfl(sf, cz, cf)
    for name, arr in (("frho", tab.frho), ("rhor", tab.rhor), ("z2r", tab.z2r)):
        got = hashlib.sha256(np.ascontiguousarray(arr, "<f8").tobytes()).hexdigest()
        assert got == e["spline_sha256"][name], name
    for row in e["samples"]:
        r, fpi, fpj, ddx, ddy, ddz, rho, rho_r, fx, fy, fz, phi, F, Fp = dx(row)
        assert oracle.eam_rho(tab, r) == rho_r
        fpair, ph = oracle.eam_pair_force(tab, r, fpi, fpj)
        assert ph == phi
        assert np.array_equal(np.array([ddx, ddy, ddz]) * fpair, np.array([fx, fy, fz]))
        assert oracle.eam_embed_one(tab, rho) == (F, Fp)


def test_golden_check_detects_a_planted_change(oracle, vec):
    """A one-ulp change planted in the oracle's result (on the CPU) fails."""
    eps, sig, r, e, de = dx(vec["lj_pair"][0])
    got = oracle.lj_pair(eps, sig, r)
    assert got == (e, de)
    assert (np.nextafter(got[0], np.inf), got[1]) != (e, de)
