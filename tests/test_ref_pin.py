"""The oracle pinned to the reference's own code, bit for bit.

oracle/ref_pin/build_ref.py compiles the exaStamp sources of the hot path's
per-pair arithmetic -- lj_compute_energy (lennard_jones.h L41-50), the
per-atom loop of lj_compute_force (force_op_impl2.hxx L22-78), the setfl
reader and spline (eam_alloy.cpp L29-278) and the eam_alloy lookups
(eam_alloy.h L198-313) -- into oracle/_ref/libref.so.  These tests feed the
same seeded inputs to it and to the oracle (oracle/gbmd_oracle.c) and
require identical doubles.  The GPU kernels are checked against the oracle
elsewhere, so this closes the chain reference -> oracle -> GPU.

Where the exaStamp sources are not readable the live library cannot be
built and the tests of this file skip; tests/test_ref_pin_golden.py then
checks the oracle against vectors this library produced
(tests/golden/ref_pin_vectors.json).
"""
import os

import numpy as np
import pytest

from exastamp_gb300 import setfl as SF

import ref_pin_lib as R


@pytest.fixture(scope="module")
def ref():
    L = R.load()
    if L is None:
        pytest.skip("exaStamp sources not readable here: the pin library is not built")
    return L


def test_lj_pair_function_bit_exact(ref, oracle):
    rng = np.random.default_rng(11)
    for _ in range(3000):
        eps, sig = rng.uniform(0.1, 3.0), rng.uniform(0.5, 2.0)
        r = rng.uniform(0.6, 3.2) * sig
        assert oracle.lj_pair(eps, sig, r) == R.lj_pair(ref, eps, sig, r)


def _pair_buffer(rng, n, rc):
    u = rng.normal(size=(n, 3))
    u /= np.linalg.norm(u, axis=1)[:, None]
    r = rng.uniform(0.85, rc, n)
    d = u * r[:, None]
    d2 = d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1] + d[:, 2] * d[:, 2]
    return d[:, 0].copy(), d[:, 1].copy(), d[:, 2].copy(), d2


@pytest.mark.parametrize("n", [0, 1, 7, 54, 90])
def test_lj_per_atom_loop_bit_exact(ref, oracle, n):
    rng = np.random.default_rng(100 + n)
    for _ in range(40):
        eps, sig = rng.uniform(0.5, 2.0), rng.uniform(0.8, 1.2)
        rc = 2.5 * sig
        ecut = oracle.lj_energy_cut(eps, sig, rc)
        buf = _pair_buffer(rng, n, rc)
        a = oracle.lj_atom_buffer(eps, sig, ecut, *buf)
        b = R.lj_force_atom(ref, eps, sig, ecut, *buf)
        assert np.array_equal(a, b), (a, b)


def _setfl_cases(tmp_path):
    """(label, path): two of exaStamp's own setfl fixtures and the build's
    copper-like analytic table (5,000-point grids) written as a setfl file."""
    cu = str(tmp_path / "cu_analytic.eam.alloy")
    SF.write_setfl(SF.tabulate(SF.load_cu_params()), cu)
    return [("Ta1_Ravelo_2013", R.exastamp_file("data", "potentials", "Ta1_Ravelo_2013.eam.alloy")),
            ("AlCu", R.exastamp_file("data", "potentials", "AlCu.eam.alloy")),
            ("cu_analytic", cu)]


def _oracle_tables(oracle, ref, path):
    sf = SF.read_setfl(path)
    cz, cf = R.eam_conversions(ref)
    return sf, oracle.EamOracleTables.from_setfl(sf, cz, cf)


def test_eam_setfl_splines_bit_exact(ref, oracle, tmp_path):
    for label, path in _setfl_cases(tmp_path):
        if not os.path.exists(path):
            pytest.skip("missing %s" % path)
        nel, nr, nrho = R.eam_load(ref, path)
        sf, tab = _oracle_tables(oracle, ref, path)
        assert (nel, nr, nrho) == (sf.nelements, sf.nr, sf.nrho), label
        for which, mine in enumerate((tab.frho, tab.rhor, tab.z2r)):
            theirs = R.eam_spline(ref, which)
            assert np.array_equal(mine.ravel(), theirs), (label, which)


def test_eam_pair_and_embedding_functions_bit_exact(ref, oracle, tmp_path):
    rng = np.random.default_rng(12)
    for label, path in _setfl_cases(tmp_path):
        if not os.path.exists(path):
            pytest.skip("missing %s" % path)
        R.eam_load(ref, path)
        sf, tab = _oracle_tables(oracle, ref, path)
        nel = sf.nelements
        rhomax = (sf.nrho - 1) * sf.drho
        for _ in range(1500):
            it, jt = int(rng.integers(nel)), int(rng.integers(nel))
            # beyond the table too, where both clamp the knot index
            r = rng.uniform(0.5, sf.rcut * 1.08)
            assert oracle.eam_rho(tab, r, it, jt) == ref.ref_eam_rho(r, it, jt), label
            fpi, fpj = rng.normal(0.0, 2.0, 2)
            dr = rng.normal(0.0, 1.0, 3)
            fpair, phi = oracle.eam_pair_force(tab, r, fpi, fpj, it, jt)
            v, phi_ref = R.eam_mm_force(ref, r, fpi, fpj, it, jt, dr)
            assert phi == phi_ref, label
            assert np.array_equal(dr * fpair, v), label
            rho = rng.uniform(0.0, 1.3 * rhomax)
            assert oracle.eam_embed_one(tab, rho, it) == R.eam_fembed(ref, rho, it), label


def test_eam_conversion_factors_match_the_build_units(ref):
    """The stand-in units give the reference's conversion factors the values
    the build uses for eV (CODATA 2018, Da A^2 / ps^2)."""
    from exastamp_gb300 import systems as S
    cz, cf = R.eam_conversions(ref)
    assert cz == S.EV and cf == S.EV
