"""GPU path against exaStamp's own EAM fixtures (tests/golden, windows of
data/potentials/*.eam.alloy): on the perfect lattice at the header's lattice
constant, every force cancels, the Ravelo Ta models give their fitted
cohesive energy of 8.1 eV per atom, and the virial vanishes.  FP64 agrees
with the oracle on the same tables to 1e-12; mixed precision within its
stated tolerances."""
import numpy as np
import pytest

import golden_setfl as G

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("k", range(4))
@pytest.mark.parametrize("mixed", [False, True])
def test_lattice_known_answers_on_gpu(gpu, oracle, k, mixed):
    fx = G.load()
    case = fx["cases"][k]
    sf = G.setfl_for(case, fx)
    s = G.lattice_system(case, case["a0"], ncell=7)
    tab = oracle.EamOracleTables.from_setfl(sf, 1.0, 1.0)
    nl = oracle.build_neighbors(s.x, s.y, s.z, s.id, s.lo, s.hi, sf.rcut + 0.3)
    ofx, ofy, ofz, oep, ovir, _, _ = oracle.eam_forces(s.x, s.y, s.z, s.type, nl, s.L, tab, sf.rcut)
    with gpu.Context(0) as ctx:
        ctx.upload_system(s)
        ctx.set_eam_alloy(sf, sf.rcut, 1.0, 1.0)  # eV, eV*A: energies in eV, masses 1
        ctx.set_skin(0.3)
        ctx.set_precision(mixed)
        ctx.compute_forces(energy=True, virial=True)
        d = ctx.download(virial=True)
    e = d["ep"].mean()
    fmax = max(np.abs(d[c]).max() for c in ("ax", "ay", "az"))
    vir = d["vir"].reshape(-1, 9)
    p = -vir[:, [0, 4, 8]].sum() / (3.0 * float(np.prod(s.L)))
    if not mixed:
        assert abs(e - oep.mean()) < 1e-12 * abs(oep.mean())
        # per-atom virials vanish up to the rounding of O(1 eV) pair terms
        assert np.abs(vir - ovir).max() < 1e-12
        assert fmax < 1e-10
    else:
        assert abs(e - oep.mean()) < 1e-6 * abs(oep.mean())
        assert fmax < 1e-4  # FP32 sums of O(1 eV/A) terms that cancel
    if case["cohesive_energy_eV"] is not None:
        assert abs(e - case["cohesive_energy_eV"]) < (1e-9 if not mixed else 1e-5), e
        assert abs(p) < (1e-8 if not mixed else 1e-5), p
