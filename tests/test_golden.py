"""The oracle pinned against exaStamp's own EAM fixtures.

tests/golden/eam_setfl_lattice.json holds windows of the setfl files in
exaStamp's data/potentials (Ta1/Ta2 Ravelo 2013, AlCu Cai-Ye), written by
tests/golden/make_golden.py.  Known answers: each file's header lattice
constant is the zero-pressure lattice constant of its element, and the
Ravelo Ta models give their fitted cohesive energy, 8.1 eV per atom, on the
perfect BCC lattice (PRB 88, 134101).  These pin the setfl reader, the
spline (eam_alloy.cpp L29-58), the lookups (eam_alloy.h L198-313) and the
three EAM passes (eam_force_op_multimat.h L114-343) of the oracle; the GPU
side is checked against the same fixture in test_gpu_golden.py.
"""
import os

import numpy as np
import pytest

from exastamp_gb300 import setfl

import golden_setfl as G

# the exaStamp source tree, when readable (set EXASTAMP_ROOT to check the
# fixture against the original files)
REF = os.environ.get("EXASTAMP_ROOT", "")


def oracle_lattice(oracle, sf, case, a):
    s = G.lattice_system(case, a)
    tab = oracle.EamOracleTables.from_setfl(sf, 1.0, 1.0)
    nl = oracle.build_neighbors(s.x, s.y, s.z, s.id, s.lo, s.hi, sf.rcut)
    fx, fy, fz, ep, vir, _, _ = oracle.eam_forces(s.x, s.y, s.z, s.type, nl, s.L, tab, sf.rcut)
    vol = float(np.prod(s.L))
    pressure = -vir[:, [0, 4, 8]].sum() / (3.0 * vol)  # eV / A^3 (virial = -1/2 f x dr)
    return ep.mean(), pressure, max(np.abs(fx).max(), np.abs(fy).max(), np.abs(fz).max())


@pytest.mark.parametrize("k", range(4))
def test_oracle_lattice_known_answers(oracle, k):
    fx = G.load()
    case = fx["cases"][k]
    sf = G.setfl_for(case, fx)
    a0 = case["a0"]
    E0, P0, fmax = oracle_lattice(oracle, sf, case, a0)
    assert fmax < 1e-10  # perfect lattice: every force cancels
    # zero pressure at the header's lattice constant: E(a) is minimal there
    da = np.array(case["lattice_offsets"])
    E = np.array([oracle_lattice(oracle, sf, case, a0 + d)[0] for d in da])
    c = np.polyfit(da, E, 2)
    assert abs(-c[1] / (2 * c[0])) < 1e-3, (case["file"], -c[1] / (2 * c[0]))
    if case["cohesive_energy_eV"] is not None:
        assert abs(E0 - case["cohesive_energy_eV"]) < 1e-9, E0
        assert abs(P0) < 1e-8, P0


@pytest.mark.skipif(not REF or not os.path.isdir(os.path.join(REF, "data", "potentials")),
                    reason="exaStamp sources not present")
def test_fixture_matches_exastamp_files(oracle):
    """The committed windows are the files' own values, and a lattice
    evaluation with the windowed tables equals the full tables bit for bit."""
    fx = G.load()
    for name, p in fx["potentials"].items():
        sf = setfl.read_setfl(os.path.join(REF, "data", "potentials", name + ".eam.alloy"))
        assert (sf.nrho, sf.drho, sf.nr, sf.dr, sf.rcut) == (p["nrho"], p["drho"], p["nr"], p["dr"], p["rcut"])
        assert sf.elements == p["elements"] and sf.a0 == p["a0"] and sf.masses == p["masses"]
        for key, tabs in (("frho", sf.frho), ("rhor", sf.rhor), ("z2r", sf.z2r)):
            for k, wl in p[key].items():
                for lo, vals in wl:
                    assert np.array_equal(tabs[int(k)][lo:lo + len(vals)], np.array(vals)), (name, key, k, lo)
    for case in fx["cases"]:
        full = setfl.read_setfl(os.path.join(REF, "data", "potentials", case["file"] + ".eam.alloy"))
        e, kz = case["element"], case["z2r_index"]
        one = setfl.Setfl([full.elements[e]], [full.Z[e]], [full.masses[e]], [full.a0[e]], [full.structs[e]],
                          full.nrho, full.drho, full.nr, full.dr, full.rcut, [full.frho[e]], [full.rhor[e]],
                          [full.z2r[kz]])
        win = G.setfl_for(case, fx)
        for d in case["lattice_offsets"]:
            a = case["a0"] + d
            assert oracle_lattice(oracle, one, case, a) == oracle_lattice(oracle, win, case, a)
