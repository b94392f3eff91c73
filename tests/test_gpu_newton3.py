"""Newton-3 mode (lj_compute_force_symetric): half list + reaction forces
scattered through 64-bit fixed-point atomics, called through the C ABI,
against the FP64 oracle.

Bars: the half list holds each pair of the full list exactly once (bit-exact
pair set after mirroring); forces within 1e-5 relative RMS (the mixed
tolerance), total energy within 1e-6 relative, virial within 1e-5 relative
RMS; two runs are bit-identical (the integer sums do not depend on the
order of the atomics); an NVE run stays close to the full-list run; a pair
force beyond the fixed-point range answers GBMD_ERR_TOO_LARGE; the set-ups
without a Newton-3 kernel answer GBMD_ERR_UNSUPPORTED.
"""
import numpy as np
import pytest

from exastamp_gb300 import systems as S
from exastamp_gb300 import setfl as SF

from test_gpu_parity import LJ, _jitter, _lj_oracle, _two_element_setfl, gpu_ctx, oracle_lists, rel_rms

pytestmark = pytest.mark.gpu

MIXED_FORCE_TOL = 1e-5
UNSUPPORTED = 8  # GBMD_ERR_UNSUPPORTED
TOO_LARGE = 9    # GBMD_ERR_TOO_LARGE


def _n3_ctx(gpu, s, pot, skin=0.3):
    ctx = gpu_ctx(gpu, s, pot, skin, mixed=True, tpa=1, block=256, vec=4)
    ctx.set_newton3(True)
    assert ctx.get_newton3()
    return ctx


@pytest.mark.parametrize("ncell,sig", [(3, 0.05), (6, 0.1), (2, 0.1)])
def test_half_list_mirrors_to_full_list(gpu, ncell, sig):
    s = _jitter(S.lj_fcc(ncell=ncell, seed=ncell), sig, ncell)
    with gpu_ctx(gpu, s, LJ, 0.3, mixed=True, tpa=1, block=256, vec=4) as ctx:
        ctx.build_neighbors()
        full = {tuple(int(v) for v in r) for r in ctx.export_pairs()}
    with _n3_ctx(gpu, s, LJ) as ctx:
        ctx.build_neighbors()
        rows = [tuple(int(v) for v in r) for r in ctx.export_pairs()]
    half = set(rows)
    assert len(half) == len(rows)
    mirror = {(j, i, -a, -b, -c) for (i, j, a, b, c) in half}
    assert not (half & mirror)
    assert half | mirror == full
    assert 2 * len(half) == len(full)


@pytest.mark.parametrize("ncell,sig", [(8, 0.06), (3, 0.08)])
def test_lj_newton3_matches_oracle(gpu, oracle, ncell, sig):
    s = _jitter(S.lj_fcc(ncell=ncell, seed=2), sig, 2)
    F, ep, vir = _lj_oracle(oracle, s)
    with _n3_ctx(gpu, s, LJ) as ctx:
        for _ in range(2):  # the second call sees the accumulators cleared by the first
            ctx.compute_forces(energy=True, virial=True)
            d = ctx.download(virial=True)
            G = np.stack([d["ax"], d["ay"], d["az"]], 1)
            assert rel_rms(G, F) < MIXED_FORCE_TOL
            assert abs(d["ep"].sum() - ep.sum()) < 1e-6 * abs(ep.sum())
            assert rel_rms(d["ep"], ep) < 1e-5
            assert rel_rms(d["vir"], vir) < 1e-5
        ctx.compute_forces()  # no energy: forces only
        d = ctx.download()
        assert rel_rms(np.stack([d["ax"], d["ay"], d["az"]], 1), F) < MIXED_FORCE_TOL


def test_lj_multi_newton3_matches_oracle(gpu, oracle):
    s = _jitter(S.lj_fcc(ncell=6, seed=3), 0.05, 3)
    rng = np.random.default_rng(3)
    s.type = (rng.random(s.n) < 0.2).astype(np.uint8)
    s.masses = np.array([1.0, 2.0])
    eps, sig, rc = S.kob_andersen_tables()
    rcmax = float(rc.max())
    x, y, z = s.x.copy(), s.y.copy(), s.z.copy()
    oracle.wrap(x, y, z, s.lo, s.hi)
    nl = oracle.build_neighbors(x, y, z, s.id, s.lo, s.hi, rcmax + 0.3)
    fx, fy, fz, ep, vir = oracle.lj_multi_force(x, y, z, s.type, nl, s.L, eps, sig, rc, rcmax)
    F = np.stack([fx, fy, fz], 1) / s.masses[s.type][:, None]
    with _n3_ctx(gpu, s, lambda c: c.set_lj_multi(eps, sig, rc, 0.0)) as ctx:
        ctx.compute_forces(energy=True, virial=True)
        d = ctx.download(virial=True)
    G = np.stack([d["ax"], d["ay"], d["az"]], 1)
    assert rel_rms(G, F) < MIXED_FORCE_TOL
    assert abs(d["ep"].sum() - ep.sum()) < 1e-6 * abs(ep.sum())
    assert rel_rms(d["vir"], vir) < 1e-5


@pytest.mark.parametrize("use_graph", [False, True])
def test_newton3_nve_tracks_full_list(gpu, use_graph):
    """40 NVE steps with rebuilds every 10 (fused Verlet epilogue, graph
    replay): positions stay within 1e-6 of the full-list run, the energy is
    conserved as well, and the momentum stays ~0 (pairwise equal and opposite
    forces up to FP32 rounding)."""
    s = S.lj_fcc(ncell=6, seed=8)
    out = {}
    for n3 in (False, True):
        with gpu_ctx(gpu, s, LJ, 0.3, mixed=True, tpa=1, block=256, vec=4) as ctx:
            ctx.set_newton3(n3)
            th = ctx.run_nve(40, 0.005, rebuild_every=10, thermo_every=20 if use_graph else 10,
                             use_graph=use_graph)
            out[n3] = (th, ctx.download())
    (th0, d0), (th1, d1) = out[False], out[True]
    for k in ("x", "y", "z", "vx"):
        assert np.abs(d1[k] - d0[k]).max() < 1e-6, k
    e0 = th0[:, 21:24].sum(1) + th0[:, 24]
    e1 = th1[:, 21:24].sum(1) + th1[:, 24]
    assert np.abs(e1 - e0).max() < 1e-6 * np.abs(e0).max()
    assert np.abs(th1[:, 18:21]).max() < 1e-5


def test_newton3_displacement_trigger(gpu):
    s = S.lj_fcc(ncell=6, seed=9)
    with gpu_ctx(gpu, s, LJ, 0.3, mixed=True, tpa=1, block=256, vec=4) as ctx:
        ctx.set_newton3(True)
        ctx.run_nve(30, 0.005, rebuild_every=-1, thermo_every=10)
        d1 = ctx.download()
    with gpu_ctx(gpu, s, LJ, 0.3, mixed=True, tpa=1, block=256, vec=4) as ctx:
        ctx.run_nve(30, 0.005, rebuild_every=-1, thermo_every=10)
        d0 = ctx.download()
    assert np.abs(d1["x"] - d0["x"]).max() < 1e-6


def test_newton3_unsupported_setups(gpu):
    s = _jitter(S.lj_fcc(ncell=4, seed=5), 0.05, 5)
    # FP64 precision
    with gpu_ctx(gpu, s, LJ, 0.3, mixed=False, tpa=1, block=256, vec=4) as ctx:
        ctx.set_newton3(True)
        with pytest.raises(gpu.GbmdError) as e:
            ctx.compute_forces()
        assert e.value.code == UNSUPPORTED
    # another launch layout
    with gpu_ctx(gpu, s, LJ, 0.3, mixed=True, tpa=4, block=128, vec=1) as ctx:
        ctx.set_newton3(True)
        with pytest.raises(gpu.GbmdError) as e:
            ctx.compute_forces()
        assert e.value.code == UNSUPPORTED
    # eam_alloy in FP64, and the analytic EAM operators
    sf = SF.tabulate(SF.load_cu_params())
    c = S.eam_cu_fcc(ncell=4, displace=0.05, seed=4)
    with gpu_ctx(gpu, c, lambda k: k.set_eam_alloy(sf, 5.0, S.EV, S.EV), 0.3, mixed=False, tpa=1, block=256,
                 vec=4) as ctx:
        ctx.set_newton3(True)
        with pytest.raises(gpu.GbmdError) as e:
            ctx.compute_forces()
        assert e.value.code == UNSUPPORTED
    ta = S.ta_bcc(ncell=5, seed=4)
    with gpu_ctx(gpu, ta, lambda k: k.set_eam_johnson(S.johnson_ta_params(), 6.1), 0.3, mixed=True, tpa=1,
                 block=256, vec=4) as ctx:
        ctx.set_newton3(True)
        with pytest.raises(gpu.GbmdError) as e:
            ctx.compute_forces()
        assert e.value.code == UNSUPPORTED
    # switching back gives the full-list result again
    with _n3_ctx(gpu, s, LJ) as ctx:
        ctx.compute_forces(energy=True)
        d1 = ctx.download()
        ctx.set_newton3(False)
        ctx.compute_forces(energy=True)
        d0 = ctx.download()
    assert rel_rms(d1["ax"], d0["ax"]) < MIXED_FORCE_TOL


@pytest.mark.parametrize("half_list", [False, True])
def test_symetric_operator_matches_lj_compute_force(gpu, oracle, half_list):
    """The operator mirror: a run file binding lj_compute_force_symetric to
    compute_force gives the lj_compute_force result: on the full list by
    default (FP64, 1e-12), on the Newton-3 half list with half_list (mixed
    tolerance)."""
    from exastamp_gb300 import operators as OP
    s = _jitter(S.lj_fcc(ncell=5, seed=6), 0.05, 6)
    F, ep, _ = _lj_oracle(oracle, s)
    par = {"rcut": 2.5, "parameters": {"epsilon": 1.0, "sigma": 1.0}}
    if half_list:
        par["half_list"] = True
    cfg = {"compute_force": "lj_compute_force_symetric", "lj_compute_force_symetric": par}
    sim = OP.Simulation(s)
    try:
        op = OP.compute_force_from_config(cfg)
        assert isinstance(op, OP.lj_compute_force_symetric)
        op.bind(sim)
        OP.chunk_neighbors().bind(sim, 0.3)
        op.execute(sim, energy=True)
        assert sim.ctx.get_newton3() == half_list
        d = sim.ctx.download()
    finally:
        sim.ctx.close()
    G = np.stack([d["ax"], d["ay"], d["az"]], 1)
    if half_list:
        assert rel_rms(G, F) < MIXED_FORCE_TOL
        assert abs(d["ep"].sum() - ep.sum()) < 1e-6 * abs(ep.sum())
    else:
        assert np.abs(G - F).max() < 1e-12 * np.abs(F).max()
        assert np.abs(d["ep"] - ep).max() < 1e-12 * np.abs(ep).max()


@pytest.mark.parametrize("use_graph", [False, True])
def test_newton3_runs_are_bit_reproducible(gpu, use_graph):
    """The same 40 steps twice (LJ mixture types, energies and virials on
    thermo steps): every array equal bit for bit."""
    s = _jitter(S.lj_fcc(ncell=8, seed=21), 0.05, 21)
    rng = np.random.default_rng(21)
    s.type = (rng.random(s.n) < 0.2).astype(np.uint8)
    s.masses = np.array([1.0, 2.0])
    eps, sig, rc = S.kob_andersen_tables()
    out = []
    for _ in range(2):
        with _n3_ctx(gpu, s, lambda c: c.set_lj_multi(eps, sig, rc, 0.0)) as ctx:
            th = ctx.run_nve(40, 0.002, rebuild_every=10, thermo_every=20, use_graph=use_graph)
            ctx.compute_forces(energy=True, virial=True)
            out.append((th, ctx.download(virial=True)))
    assert np.array_equal(out[0][0], out[1][0])
    for k in ("x", "y", "z", "vx", "vy", "vz", "ax", "ay", "az", "ep", "vir"):
        assert np.array_equal(out[0][1][k], out[1][1][k]), k


def test_newton3_force_beyond_the_fixed_point_range(gpu):
    """Two atoms 0.4 sigma apart: a pair force of ~7e6 (beyond 2^16 x 24
    eps/sigma) is refused on the half list; the full list computes it."""
    s = S.lj_fcc(ncell=4, seed=22)
    s.x[1], s.y[1], s.z[1] = s.x[0] + 0.4, s.y[0], s.z[0]
    with _n3_ctx(gpu, s, LJ) as ctx:
        ctx.compute_forces()
        with pytest.raises(gpu.GbmdError) as e:
            ctx.check_errors()
        assert e.value.code == TOO_LARGE
        ctx.check_errors()  # cleared once reported
        with pytest.raises(gpu.GbmdError) as e:
            ctx.run_nve(1, 0.001, rebuild_every=0)
        assert e.value.code == TOO_LARGE
        ctx.set_newton3(False)
        ctx.compute_forces()
        ctx.check_errors()
        d = ctx.download()
    assert np.isfinite(d["ax"]).all() and abs(d["ax"][0]) > 1e6


def _eam_case(kind):
    if kind == "cu":
        sf = SF.tabulate(SF.load_cu_params())
        s = S.eam_cu_fcc(ncell=5, displace=0.08, seed=23)
    else:
        sf = _two_element_setfl()
        s = S.eam_cu_fcc(ncell=5, displace=0.08, seed=24)
        rng = np.random.default_rng(24)
        s.type = (rng.random(s.n) < 0.3).astype(np.uint8)
        s.masses = np.array(sf.masses)
    return sf, s


@pytest.mark.parametrize("kind", ["cu", "two_elements"])
def test_eam_newton3_matches_oracle(gpu, oracle, kind):
    """eam_symmetry on the half list: rho_j and the reaction force scattered
    through fixed-point atomics; forces, energies and virials against the
    FP64 oracle at the mixed tolerances."""
    sf, s = _eam_case(kind)
    tab = oracle.EamOracleTables.from_setfl(sf, S.EV, S.EV, rcut=5.0)
    _, (x, y, z), nl = oracle_lists(oracle, s, 5.3)
    fx, fy, fz, ep, vir, fp, rho = oracle.eam_forces(x, y, z, s.type, nl, s.L, tab, 5.0)
    F = np.stack([fx, fy, fz], 1) / s.masses[s.type][:, None]
    with _n3_ctx(gpu, s, lambda c: c.set_eam_alloy(sf, 5.0, S.EV, S.EV)) as ctx:
        for _ in range(2):  # the second call sees the planes cleared by the first
            ctx.compute_forces(energy=True, virial=True)
            ctx.check_errors()
            d = ctx.download(virial=True)
            G = np.stack([d["ax"], d["ay"], d["az"]], 1)
            assert rel_rms(G, F) < MIXED_FORCE_TOL, rel_rms(G, F)
            assert abs(d["ep"].sum() - ep.sum()) < 1e-6 * abs(ep.sum())
            assert rel_rms(d["ep"], ep) < 1e-5
            assert rel_rms(d["vir"], vir) < 1e-5
        ctx.compute_forces()
        d = ctx.download()
        assert rel_rms(np.stack([d["ax"], d["ay"], d["az"]], 1), F) < MIXED_FORCE_TOL


def test_eam_newton3_split_passes_and_reruns(gpu):
    """The density pass then the force pass give the fused pass bit for bit;
    two 40-step runs are bit-identical and stay within 1e-6 of the
    full-list run."""
    sf, s = _eam_case("cu")
    setpot = lambda c: c.set_eam_alloy(sf, 5.0, S.EV, S.EV)  # noqa: E731
    with _n3_ctx(gpu, s, setpot) as ctx:
        ctx.compute_forces(energy=True, virial=True)
        fused = ctx.download(virial=True)
        ctx.compute_forces(energy=True, virial=True, passes="density")
        ctx.compute_forces(energy=True, virial=True, passes="force")
        split = ctx.download(virial=True)
    for k in ("ax", "ay", "az", "ep", "vir"):
        assert np.array_equal(split[k], fused[k]), k
    out = []
    for n3 in (True, True, False):
        with gpu_ctx(gpu, s, setpot, 0.3, mixed=True, tpa=1, block=256, vec=4) as ctx:
            ctx.set_newton3(n3)
            th = ctx.run_nve(40, 1e-3, rebuild_every=10, thermo_every=20, use_graph=True)
            out.append((th, ctx.download()))
    assert np.array_equal(out[0][0], out[1][0])
    for k in ("x", "y", "z", "vx", "vy", "vz", "ax"):
        assert np.array_equal(out[0][1][k], out[1][1][k]), k
        if k in ("x", "y", "z"):
            dd = np.abs(out[0][1][k] - out[2][1][k])
            assert np.minimum(dd, s.L[0] - dd).max() < 1e-6, k
    e0 = out[2][0][:, 21:24].sum(1) + out[2][0][:, 24]
    e1 = out[0][0][:, 21:24].sum(1) + out[0][0][:, 24]
    assert np.abs(e1 - e0).max() < 1e-6 * np.abs(e0).max()
