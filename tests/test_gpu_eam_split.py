"""Split EAM passes (eam_alloy_force with eam_rho / eam_rho2emb / eam_force
set per call, as in the reference's split run-file form), called through
the C ABI and through the operator mirror.

Bars: density pass then force pass gives the fused result bit for bit (the
same kernels in the same order); a force pass without a density pass on the
same positions, or energies the density pass did not store, is refused with
GBMD_ERR_INVALID.
"""
import numpy as np
import pytest

from exastamp_gb300 import operators as OP
from exastamp_gb300 import setfl as SF
from exastamp_gb300 import systems as S

from test_gpu_parity import gpu_ctx

pytestmark = pytest.mark.gpu

INVALID = 1  # GBMD_ERR_INVALID
FIELDS = ("ax", "ay", "az", "ep", "vir")


def _eam():
    return SF.tabulate(SF.load_cu_params())


def _same(a, b):
    for k in FIELDS:
        assert np.array_equal(a[k], b[k]), k


@pytest.mark.parametrize("mixed", [False, True])
@pytest.mark.parametrize("pot", ["eam_alloy", "johnson"])
def test_split_passes_bit_identical_to_fused(gpu, mixed, pot):
    if pot == "eam_alloy":
        sf = _eam()
        s = S.eam_cu_fcc(ncell=5, displace=0.08, seed=4)
        setpot = lambda c: c.set_eam_alloy(sf, 5.0, S.EV, S.EV)  # noqa: E731
    else:
        params = S.johnson_ta_params()
        s = S.ta_bcc(ncell=6, seed=5)
        setpot = lambda c: c.set_eam_johnson(params, 6.1)  # noqa: E731
    with gpu_ctx(gpu, s, setpot, 0.3, mixed=mixed) as ctx:
        ctx.compute_forces(energy=True, virial=True)
        fused = ctx.download(virial=True)
        ctx.compute_forces(energy=True, virial=True, passes="density")
        ctx.compute_forces(energy=True, virial=True, passes="force")
        split = ctx.download(virial=True)
        _same(split, fused)
        # the force pass may run again from the same density pass
        ctx.compute_forces(energy=True, virial=True, passes="force")
        _same(ctx.download(virial=True), fused)


def test_force_pass_needs_its_density_pass(gpu):
    sf = _eam()
    s = S.eam_cu_fcc(ncell=4, displace=0.05, seed=3)
    with gpu_ctx(gpu, s, lambda c: c.set_eam_alloy(sf, 5.0, S.EV, S.EV), 0.3, mixed=True) as ctx:
        with pytest.raises(gpu.GbmdError) as e:
            ctx.compute_forces(passes="force")
        assert e.value.code == INVALID
        ctx.compute_forces(energy=False, passes="density")
        with pytest.raises(gpu.GbmdError) as e:  # energies not stored by that density pass
            ctx.compute_forces(energy=True, passes="force")
        assert e.value.code == INVALID
        ctx.compute_forces(energy=False, passes="force")
        ctx.push_f_v_r(1e-3, 1.0)  # positions moved: the kept F'(rho) is stale
        with pytest.raises(gpu.GbmdError) as e:
            ctx.compute_forces(energy=False, passes="force")
        assert e.value.code == INVALID
        ctx.compute_forces(energy=False)  # the fused call always works


def test_lj_pass_flags(gpu):
    s = S.lj_fcc(ncell=4, seed=2)
    with gpu_ctx(gpu, s, lambda c: c.set_lj(1.0, 1.0, 2.5), 0.3, mixed=True) as ctx:
        ctx.compute_forces(energy=True)
        full = ctx.download()
        ctx.compute_forces(energy=True, passes="force")
        again = ctx.download()
        for k in ("ax", "ay", "az", "ep"):
            assert np.array_equal(again[k], full[k]), k


def test_split_run_file_form(gpu):
    """Three eam_alloy_force operators with the per-pass flags of the
    reference's split form (eam_rho / eam_rho2emb / eam_force, each alone)
    executed in order give the one-call result bit for bit."""
    sf = _eam()
    s = S.eam_cu_fcc(ncell=5, displace=0.06, seed=8)
    common = {"rcut": 5.0, "parameters": sf, "eam_ghost": False, "eam_symmetry": False}
    flags = [dict(eam_rho=True, eam_rho2emb=False, eam_force=False),
             dict(eam_rho=False, eam_rho2emb=True, eam_force=False),
             dict(eam_rho=False, eam_rho2emb=False, eam_force=True)]
    out = []
    for split in (False, True):
        sim = OP.Simulation(s)
        try:
            sim.set_precision(True)
            ops = [OP.eam_alloy_force(**common, **f) for f in flags] if split else [OP.eam_alloy_force(**common)]
            for op in ops:
                op.bind(sim)
            OP.chunk_neighbors().bind(sim, 0.3)
            for op in ops:
                op.execute(sim, energy=True)
            out.append(sim.ctx.download())
        finally:
            sim.ctx.close()
    for k in ("ax", "ay", "az", "ep"):
        assert np.array_equal(out[0][k], out[1][k]), k
    with pytest.raises(OP.OperatorError):
        OP.eam_alloy_force(**common, eam_rho=True, eam_rho2emb=False, eam_force=True).bind(OP.Simulation(s))


def test_eam_symmetry_runs_the_full_list(gpu, oracle):
    """eam_symmetry: true (the reference's Newton-3 scatter) gives the
    full-list result bit for bit, and that result matches the oracle."""
    sf = _eam()
    s = S.eam_cu_fcc(ncell=5, displace=0.06, seed=9)
    out = []
    for sym in (False, True):
        sim = OP.Simulation(s)
        try:
            sim.set_precision(False)
            op = OP.eam_alloy_force(rcut=5.0, parameters=sf, eam_symmetry=sym)
            op.bind(sim)
            OP.chunk_neighbors().bind(sim, 0.3)
            op.execute(sim, energy=True, virial=True)
            out.append(sim.ctx.download(virial=True))
        finally:
            sim.ctx.close()
    for k in ("ax", "ay", "az", "ep", "vir"):
        assert np.array_equal(out[0][k], out[1][k]), k
    tab = oracle.EamOracleTables.from_setfl(sf, S.EV, S.EV, rcut=5.0)
    x, y, z = s.x.copy(), s.y.copy(), s.z.copy()
    oracle.wrap(x, y, z, s.lo, s.hi)
    nl = oracle.build_neighbors(x, y, z, s.id, s.lo, s.hi, 5.3)
    fx, fy, fz, ep, vir, _, _ = oracle.eam_forces(x, y, z, s.type, nl, s.L, tab, 5.0)
    F = np.stack([fx, fy, fz], 1) / s.masses[0]
    G = np.stack([out[1]["ax"], out[1]["ay"], out[1]["az"]], 1)
    assert np.abs(G - F).max() < 1e-11 * np.abs(F).max()
    assert np.abs(out[1]["ep"] - ep).max() < 1e-12 * np.abs(ep).max()


def test_eam_symmetry_half_list_operator(gpu, oracle):
    """eam_symmetry with half_list: the operator mirror switches the context
    to the Newton-3 half list (mixed precision, fixed-point scatter); the
    forces, energies and virials match the oracle at the mixed tolerances."""
    sf = _eam()
    s = S.eam_cu_fcc(ncell=5, displace=0.06, seed=10)
    sim = OP.Simulation(s)
    try:
        op = OP.eam_alloy_force(rcut=5.0, parameters=sf, eam_symmetry=True, half_list=True)
        op.bind(sim)
        OP.chunk_neighbors().bind(sim, 0.3)
        assert sim.ctx.get_newton3()
        op.execute(sim, energy=True, virial=True)
        sim.ctx.check_errors()
        d = sim.ctx.download(virial=True)
    finally:
        sim.ctx.close()
    tab = oracle.EamOracleTables.from_setfl(sf, S.EV, S.EV, rcut=5.0)
    x, y, z = s.x.copy(), s.y.copy(), s.z.copy()
    oracle.wrap(x, y, z, s.lo, s.hi)
    nl = oracle.build_neighbors(x, y, z, s.id, s.lo, s.hi, 5.3)
    fx, fy, fz, ep, vir, _, _ = oracle.eam_forces(x, y, z, s.type, nl, s.L, tab, 5.0)
    F = np.stack([fx, fy, fz], 1) / s.masses[0]
    G = np.stack([d["ax"], d["ay"], d["az"]], 1)
    assert np.sqrt(((G - F) ** 2).sum() / (F ** 2).sum()) < 1e-5
    assert abs(d["ep"].sum() - ep.sum()) < 1e-6 * abs(ep.sum())
    assert np.sqrt(((d["vir"] - vir) ** 2).sum() / (vir ** 2).sum()) < 1e-5
