"""sutton_chen_force (analytic single-element EAM, sutton_chen.h L30-67 with
the mono-material two-pass template) on the GPU against the oracle, on the
Cu FCC system of the reference's regression case (eam_sutton_chen/
single_specy.msp: c 33.17, epsilon 3.605e-21 J, a0 0.327 nm, n 9.05,
m 5.005, rcut 7.29 A, lattice 3.6 A, noise 0.1 A, skin 1.0 A).
Tolerances: FP64 1e-12 relative RMS force, mixed 1e-5."""
import numpy as np
import pytest

from exastamp_gb300 import operators as OP
from exastamp_gb300 import systems as S

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12
MIXED_TOL = 1e-5
RCUT, SKIN = 7.29, 1.0


def _rel(a, b):
    return float(np.sqrt(((a - b) ** 2).sum() / (b ** 2).sum()))


def _system(ncell, seed):
    # the regression case's box: FCC 3.6 A, Gaussian noise of 0.1 A
    return S.eam_cu_fcc(ncell=ncell, a=3.6, T=300.0, seed=seed, displace=0.1)


def _oracle_forces(oracle, s, pot):
    x, y, z = s.x.copy(), s.y.copy(), s.z.copy()
    oracle.wrap(x, y, z, s.lo, s.hi)
    nl = oracle.build_neighbors(x, y, z, s.id, s.lo, s.hi, RCUT + SKIN)
    fx, fy, fz, ep, vir, fp = oracle.sc_forces(x, y, z, nl, s.L, pot)
    return np.stack([fx, fy, fz], 1) / s.masses[0], ep, vir


@pytest.mark.parametrize("tpa,vec", [(1, 1), (1, 4), (4, 1)])
def test_sutton_chen_forces_match_oracle(gpu, oracle, tpa, vec):
    s = _system(8, 31)
    params = S.sutton_chen_cu_params()
    pot = oracle.SuttonChen(params, RCUT)
    F, ep, vir = _oracle_forces(oracle, s, pot)
    for mixed, tol in ((False, FP64_TOL), (True, MIXED_TOL)):
        with gpu.Context(0) as ctx:
            ctx.upload_system(s)
            ctx.set_eam_sutton_chen(params, RCUT)
            ctx.set_skin(SKIN)
            ctx.set_precision(mixed)
            ctx.set_launch(tpa, 128, vec)
            ctx.compute_forces(energy=True, virial=True)
            d = ctx.download(virial=True)
        G = np.stack([d["ax"], d["ay"], d["az"]], 1)
        assert _rel(G, F) < tol, (mixed, _rel(G, F))
        assert abs(d["ep"].sum() - ep.sum()) < (FP64_TOL if not mixed else 1e-6) * abs(ep.sum())
        assert _rel(d["vir"], vir) < (FP64_TOL if not mixed else MIXED_TOL)


def test_sutton_chen_nve_tracks_oracle(gpu, oracle):
    s = _system(7, 32)
    params = S.sutton_chen_cu_params()
    pot = oracle.SuttonChen(params, RCUT)
    st = s.state()
    th_ref = oracle.run_nve(st, s.masses, s.lo, s.hi, oracle.POT_EAM_SUTTON_CHEN, pot, SKIN, 1e-3, 20, 10)
    with gpu.Context(0) as ctx:
        ctx.upload_system(s)
        ctx.set_eam_sutton_chen(params, RCUT)
        ctx.set_skin(SKIN)
        ctx.set_precision(False)
        th = ctx.run_nve(20, 1e-3, rebuild_every=10, thermo_every=1)
        d = ctx.download(("x", "y", "z"))
    assert np.allclose(th, th_ref, rtol=1e-10, atol=1e-10 * np.abs(th_ref).max())
    for k in ("x", "y", "z"):
        dd = np.abs(d[k] - st[k])
        assert np.minimum(dd, s.L[0] - dd).max() < 1e-10, k


def test_sutton_chen_operator_with_the_regression_units(gpu, oracle):
    """The operator mirror reads the run file's quantities (J, m) as the
    reference's YAML decoder does and gives the oracle's forces."""
    s = _system(7, 33)
    slots = {"rcut": "7.29 ang",
             "parameters": {"c": 3.317e01, "epsilon": "3.605e-21 J", "a0": "0.327e-09 m", "n": 9.050,
                            "m": 5.005}}
    op = OP.compute_force_from_config({"compute_force": "sutton_chen_force", "sutton_chen_force": slots})
    assert isinstance(op, OP.sutton_chen_force)
    sim = OP.Simulation(s)
    try:
        op.bind(sim)
        OP.chunk_neighbors().bind(sim, SKIN)
        op.execute(sim, energy=True)
        d = sim.ctx.download()
    finally:
        sim.ctx.close()
    F, ep, _ = _oracle_forces(oracle, s, oracle.SuttonChen(S.sutton_chen_cu_params(), RCUT))
    G = np.stack([d["ax"], d["ay"], d["az"]], 1)
    assert _rel(G, F) < 1e-12
    assert np.abs(d["ep"] - ep).max() < 1e-12 * np.abs(ep).max()
