"""GPU parity tests: the sm_103a kernels, called through the C ABI, against
the FP64 oracle on the same seeded inputs.

Bars (stated per test):
  * neighbour pair set inside rcut+skin: bit-exact, in the same per-atom order;
  * FP64 path: forces / energies / virials within 1e-12 relative of the oracle
    (same formulas; the GPU contracts multiply-adds in the pair function);
  * mixed path: force error <= 1e-5 relative RMS, energy <= 1e-6 relative;
  * standalone push operators: bit-exact.
"""
import numpy as np
import pytest

from exastamp_gb300 import setfl as SF
from exastamp_gb300 import systems as S

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12
MIXED_FORCE_TOL = 1e-5


def _jitter(s, sig, seed):
    rng = np.random.default_rng(seed)
    for a in (s.x, s.y, s.z):
        a += rng.normal(0.0, sig, s.n)
    return s


def rel_rms(a, b):
    return float(np.sqrt(((a - b) ** 2).sum() / max((b ** 2).sum(), 1e-300)))


def per_atom_lists(rows):
    out = {}
    for r in rows:
        out.setdefault(int(r[0]), []).append((int(r[1]), int(r[2]), int(r[3]), int(r[4])))
    return out


def oracle_lists(oracle, s, R):
    x, y, z = s.x.copy(), s.y.copy(), s.z.copy()
    oracle.wrap(x, y, z, s.lo, s.hi)
    nl = oracle.build_neighbors(x, y, z, s.id, s.lo, s.hi, R)
    return per_atom_lists(nl.pairs_with_ids(s.id)), (x, y, z), nl


def gpu_ctx(gpu, s, pot, skin, mixed=False, tpa=None, block=None, vec=1):
    ctx = gpu.Context(0)
    ctx.upload_system(s)
    pot(ctx)
    ctx.set_skin(skin)
    ctx.set_precision(mixed)
    if tpa:
        ctx.set_launch(tpa, block or 128, vec)
    return ctx


LJ = lambda ctx: ctx.set_lj(1.0, 1.0, 2.5)  # noqa: E731


@pytest.mark.parametrize("ncell,sig,tpa,vec", [(3, 0.05, 1, 1), (5, 0.1, 4, 1), (8, 0.02, 8, 1), (2, 0.1, 2, 1),
                                               (5, 0.1, 1, 4), (4, 0.05, 2, 4), (6, 0.08, 4, 4)])
def test_pair_set_bit_exact_lj(gpu, oracle, ncell, sig, tpa, vec):
    s = _jitter(S.lj_fcc(ncell=ncell, seed=ncell), sig, ncell)
    ref, _, _ = oracle_lists(oracle, s, 2.8)
    with gpu_ctx(gpu, s, LJ, 0.3, tpa=tpa, vec=vec) as ctx:
        ctx.build_neighbors()
        got = per_atom_lists(ctx.export_pairs())
    assert got.keys() == ref.keys() or (len(ref) < s.n)
    assert got == ref


def test_pair_set_bit_exact_random_gas_and_small_boxes(gpu, oracle):
    rng = np.random.default_rng(8)
    for n, L, R in ((400, 9.0, 2.8), (60, 5.7, 2.8), (12, 3.0, 2.9), (2000, 12.0, 2.8)):
        x, y, z = (rng.uniform(0, L, n) for _ in range(3))
        s = S.System(x, y, z, np.zeros(n), np.zeros(n), np.zeros(n), np.zeros(n, np.uint8),
                     rng.permutation(n).astype(np.uint64), np.zeros(3), np.full(3, L), np.array([1.0]))
        ref, _, _ = oracle_lists(oracle, s, R)
        with gpu_ctx(gpu, s, lambda c: c.set_lj(1.0, 1.0, R - 0.3), 0.3) as ctx:
            ctx.build_neighbors()
            got = per_atom_lists(ctx.export_pairs())
        assert got == ref, (n, L)


def test_empty_and_single_atom(gpu):
    for n in (0, 1):
        s = S.System(*(np.full(n, 3.0) for _ in range(6)), np.zeros(n, np.uint8), np.arange(n, dtype=np.uint64),
                     np.zeros(3), np.full(3, 10.0), np.array([1.0]))
        with gpu_ctx(gpu, s, LJ, 0.3) as ctx:
            ctx.compute_forces()
            d = ctx.download()
            assert all(len(v) == n for v in d.values())
            if n:
                assert d["ax"][0] == 0.0 and d["ep"][0] == 0.0
            th = ctx.thermo()
            assert th[26] == n


def _lj_oracle(oracle, s):
    ref, (x, y, z), nl = oracle_lists(oracle, s, 2.8)
    fx, fy, fz, ep, vir = oracle.lj_force(x, y, z, nl, s.L, 1.0, 1.0, 2.5)
    return np.stack([fx, fy, fz], 1), ep, vir


@pytest.mark.parametrize("tpa,vec", [(1, 1), (2, 1), (4, 1), (8, 1), (16, 1), (1, 4), (4, 4)])
def test_lj_fp64_matches_oracle(gpu, oracle, tpa, vec):
    s = _jitter(S.lj_fcc(ncell=6, seed=1), 0.04, 1)
    F, ep, vir = _lj_oracle(oracle, s)
    with gpu_ctx(gpu, s, LJ, 0.3, tpa=tpa, vec=vec) as ctx:
        ctx.compute_forces(energy=True, virial=True)
        d = ctx.download(virial=True)
    G = np.stack([d["ax"], d["ay"], d["az"]], 1)
    assert rel_rms(G, F) < FP64_TOL
    assert np.abs(G - F).max() < 1e-11 * np.abs(F).max()
    assert np.abs(d["ep"] - ep).max() < FP64_TOL * np.abs(ep).max()
    assert np.abs(d["vir"] - vir).max() < FP64_TOL * np.abs(vir).max()


@pytest.mark.parametrize("tpa,vec", [(1, 1), (4, 1), (8, 1), (1, 4), (2, 4), (4, 4)])
def test_lj_mixed_within_tolerance(gpu, oracle, tpa, vec):
    s = _jitter(S.lj_fcc(ncell=8, seed=2), 0.06, 2)
    F, ep, vir = _lj_oracle(oracle, s)
    with gpu_ctx(gpu, s, LJ, 0.3, mixed=True, tpa=tpa, vec=vec) as ctx:
        ctx.compute_forces(energy=True, virial=True)
        d = ctx.download(virial=True)
    G = np.stack([d["ax"], d["ay"], d["az"]], 1)
    assert rel_rms(G, F) < MIXED_FORCE_TOL
    assert abs(d["ep"].sum() - ep.sum()) < 1e-6 * abs(ep.sum())
    assert rel_rms(d["vir"], vir) < 1e-5


@pytest.mark.parametrize("vec", [1, 4])
def test_lj_multi_matches_oracle(gpu, oracle, vec):
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
    for mixed, tol in ((False, FP64_TOL), (True, MIXED_FORCE_TOL)):
        with gpu_ctx(gpu, s, lambda c: c.set_lj_multi(eps, sig, rc, 0.0), 0.3, mixed=mixed, tpa=1, vec=vec) as ctx:
            ctx.compute_forces(energy=True)
            d = ctx.download()
        G = np.stack([d["ax"], d["ay"], d["az"]], 1)
        assert rel_rms(G, F) < tol, mixed
        assert abs(d["ep"].sum() - ep.sum()) < (1e-12 if not mixed else 1e-6) * abs(ep.sum())


def _eam_setup(oracle, ncell=5, displace=0.08, seed=4):
    cfg = SF.load_cu_params()
    sf = SF.tabulate(cfg)
    tab = oracle.EamOracleTables.from_setfl(sf, S.EV, S.EV, rcut=5.0)
    s = S.eam_cu_fcc(ncell=ncell, displace=displace, seed=seed)
    return sf, tab, s


@pytest.mark.parametrize("tpa,vec", [(1, 1), (4, 1), (8, 1), (1, 4), (2, 4)])
def test_eam_fp64_and_mixed_match_oracle(gpu, oracle, tpa, vec):
    sf, tab, s = _eam_setup(oracle)
    ref, (x, y, z), nl = oracle_lists(oracle, s, 5.3)
    fx, fy, fz, ep, vir, fp, rho = oracle.eam_forces(x, y, z, s.type, nl, s.L, tab, 5.0)
    F = np.stack([fx, fy, fz], 1) / s.masses[0]
    for mixed, tol in ((False, FP64_TOL), (True, MIXED_FORCE_TOL)):
        with gpu_ctx(gpu, s, lambda c: c.set_eam_alloy(sf, 5.0, S.EV, S.EV), 0.3, mixed=mixed, tpa=tpa,
                     vec=vec) as ctx:
            ctx.compute_forces(energy=True, virial=True)
            d = ctx.download(virial=True)
            if not mixed:
                got = per_atom_lists(ctx.export_pairs())
                assert got == ref
        G = np.stack([d["ax"], d["ay"], d["az"]], 1)
        assert rel_rms(G, F) < tol, (mixed, rel_rms(G, F))
        etol = FP64_TOL if not mixed else 1e-6
        assert abs(d["ep"].sum() - ep.sum()) < etol * abs(ep.sum())
        assert rel_rms(d["vir"], vir) < (FP64_TOL if not mixed else 1e-5)


def _two_element_setfl():
    """Cu-like element 0 and a stiffer, larger element 1 (A x1.1, re x1.03),
    cross pair z2r = mean of the two; same knot grids."""
    cfg = SF.load_cu_params()
    a = SF.tabulate(cfg)
    b = SF.tabulate(cfg, {"A": cfg["params"]["A"] * 1.1, "re": cfg["params"]["re"] * 1.03})
    return SF.Setfl(["Cu", "Xx"], [29, 30], [a.masses[0], 1.1 * a.masses[0]], [a.a0[0], a.a0[0]],
                    [a.structs[0], a.structs[0]], a.nrho, a.drho, a.nr, a.dr, a.rcut,
                    [a.frho[0], b.frho[0]], [a.rhor[0], b.rhor[0]],
                    [a.z2r[0], 0.5 * (a.z2r[0] + b.z2r[0]), b.z2r[0]])


@pytest.mark.parametrize("vec", [1, 4])
def test_eam_two_elements_match_oracle(gpu, oracle, vec):
    sf = _two_element_setfl()
    tab = oracle.EamOracleTables.from_setfl(sf, S.EV, S.EV, rcut=5.0)
    s = S.eam_cu_fcc(ncell=5, displace=0.08, seed=14)
    rng = np.random.default_rng(14)
    s.type = (rng.random(s.n) < 0.3).astype(np.uint8)
    s.masses = np.array(sf.masses)
    _, (x, y, z), nl = oracle_lists(oracle, s, 5.3)
    fx, fy, fz, ep, vir, fp, rho = oracle.eam_forces(x, y, z, s.type, nl, s.L, tab, 5.0)
    F = np.stack([fx, fy, fz], 1) / s.masses[s.type][:, None]
    for mixed, tol in ((False, FP64_TOL), (True, MIXED_FORCE_TOL)):
        with gpu_ctx(gpu, s, lambda c: c.set_eam_alloy(sf, 5.0, S.EV, S.EV), 0.3, mixed=mixed, tpa=1,
                     vec=vec) as ctx:
            ctx.compute_forces(energy=True, virial=True)
            d = ctx.download(virial=True)
        G = np.stack([d["ax"], d["ay"], d["az"]], 1)
        assert rel_rms(G, F) < tol, (mixed, rel_rms(G, F))
        assert abs(d["ep"].sum() - ep.sum()) < (FP64_TOL if not mixed else 1e-6) * abs(ep.sum())
        assert rel_rms(d["vir"], vir) < (FP64_TOL if not mixed else 1e-5)


def test_eam_setfl_file_path(gpu, oracle, tmp_path):
    sf, tab, s = _eam_setup(oracle, ncell=4)
    p = str(tmp_path / "cu.eam.alloy")
    SF.write_setfl(sf, p)
    sf2 = SF.read_setfl(p)
    with gpu_ctx(gpu, s, lambda c: c.load_setfl(p, 5.0, S.EV, S.EV), 0.3) as c1, \
            gpu_ctx(gpu, s, lambda c: c.set_eam_alloy(sf2, 5.0, S.EV, S.EV), 0.3) as c2:
        c1.compute_forces()
        c2.compute_forces()
        a, b = c1.download(), c2.download()
    assert np.array_equal(a["ax"], b["ax"]) and np.array_equal(a["ep"], b["ep"])


def test_push_operators_bit_exact(gpu, oracle):
    s = _jitter(S.lj_fcc(ncell=4, seed=5), 0.03, 5)
    with gpu_ctx(gpu, s, LJ, 0.3) as ctx:
        ctx.compute_forces()
        d0 = ctx.download()
        ctx.push_f_v_r(0.005, 1.0)
        ctx.push_f_v(0.005, 0.5)
        d1 = ctx.download()
        ctx.push_min(0.01, 1.0, 0.5)
        d2 = ctx.download()
    st = {k: d0[k].copy() for k in d0}
    oracle.push_f_v_r(st["x"], st["y"], st["z"], st["vx"], st["vy"], st["vz"], st["ax"], st["ay"], st["az"], 0.005, 1.0)
    oracle.push_f_v(st["vx"], st["vy"], st["vz"], st["ax"], st["ay"], st["az"], 0.005, 0.5)
    for k in ("x", "y", "z", "vx", "vy", "vz"):
        assert np.array_equal(d1[k], st[k]), k
    oracle.push_min(st["x"], st["y"], st["z"], st["ax"], st["ay"], st["az"], 0.01, 1.0, 0.5)
    for k in ("x", "y", "z", "ax", "ay", "az"):
        assert np.array_equal(d2[k], st[k]), k


def test_thermo_matches_oracle(gpu, oracle):
    s = _jitter(S.lj_fcc(ncell=7, seed=6), 0.03, 6)
    with gpu_ctx(gpu, s, LJ, 0.3) as ctx:
        ctx.compute_forces(energy=True, virial=True)
        d = ctx.download(virial=True)
        th = ctx.thermo()
    ref = oracle.thermo(d["vx"], d["vy"], d["vz"], d["ep"], d["vir"], s.type, s.masses)
    assert np.allclose(th, ref, rtol=1e-12, atol=1e-12 * np.abs(ref).max())


def _nve_compare(gpu, oracle, s, pot_gpu, pot_kind, pot_orc, skin, dt, nsteps, R, mixed, use_graph=False):
    st = s.state()
    th_ref = oracle.run_nve(st, s.masses, s.lo, s.hi, pot_kind, pot_orc, skin, dt, nsteps, R)
    with gpu_ctx(gpu, s, pot_gpu, skin, mixed=mixed) as ctx:
        th = ctx.run_nve(nsteps, dt, rebuild_every=R, thermo_every=1 if not use_graph else 2 * R,
                         use_graph=use_graph)
        d = ctx.download()
    return th_ref, th, st, d


def test_lj_nve_fp64_tracks_oracle(gpu, oracle):
    """20 NVE steps, rebuild every 10: FP64 GPU state stays within 1e-10 of
    the oracle's (rounding differences grow slowly in a chaotic system)."""
    s = S.lj_fcc(ncell=5, seed=7)
    th_ref, th, st, d = _nve_compare(gpu, oracle, s, LJ, oracle.POT_LJ, oracle.LJParams(1.0, 1.0, 2.5), 0.3,
                                     0.005, 20, 10, mixed=False)
    for k in ("x", "vx", "ax"):
        assert np.abs(d[k] - st[k]).max() < 1e-10, k
    assert np.allclose(th, th_ref, rtol=1e-9, atol=1e-9)


def test_eam_nve_fp64_tracks_oracle(gpu, oracle):
    sf, tab, s = _eam_setup(oracle, ncell=4, displace=0.02)
    th_ref, th, st, d = _nve_compare(gpu, oracle, s, lambda c: c.set_eam_alloy(sf, 5.0, S.EV, S.EV),
                                     oracle.POT_EAM, tab, 0.3, 1e-3, 20, 10, mixed=False)
    assert np.abs(d["x"] - st["x"]).max() < 1e-10
    assert np.allclose(th, th_ref, rtol=1e-9, atol=1e-9 * np.abs(th_ref).max())


def test_mixed_nve_energy_drift_lj(gpu, oracle):
    s = S.lj_fcc(ncell=6, seed=8)
    with gpu_ctx(gpu, s, LJ, 0.3, mixed=True) as ctx:
        th = ctx.run_nve(400, 0.005, rebuild_every=10, thermo_every=10)
    etot = th[:, 21:24].sum(1) + th[:, 24]
    drift_per_atom = abs(etot[-1] - etot[0]) / s.n
    assert drift_per_atom < 2e-3
    # FP32 pair forces do not cancel exactly: net momentum stays ~1e-9 of sum m|v|
    assert np.abs(th[:, 18:21]).max() < 1e-5


def test_graph_with_thermo_equals_stepwise_run(gpu):
    s = S.lj_fcc(ncell=5, seed=13)
    outs, ths = [], []
    for use_graph in (False, True):
        with gpu_ctx(gpu, s, LJ, 0.3, mixed=True) as ctx:
            ths.append(ctx.run_nve(85, 0.005, rebuild_every=10, thermo_every=20, use_graph=use_graph))
            outs.append(ctx.download())
    assert np.array_equal(ths[0], ths[1])
    for k in outs[0]:
        assert np.array_equal(outs[0][k], outs[1][k]), k


@pytest.mark.parametrize("pot", ["lj", "eam"])
def test_consecutive_graph_runs_equal_stepwise_runs(gpu, pot):
    """Runs whose last chunk is a whole graph (the tail graph), one after
    another: each run flips the parity of the double buffers, so the graphs
    are kept per parity and replayed only from the buffers they were captured
    on.  Thermo rows and the final state equal the stepwise runs bit for bit."""
    if pot == "lj":
        s, setpot, dt = _jitter(S.lj_fcc(ncell=5, seed=14), 0.03, 14), LJ, 0.005
    else:
        sf = SF.tabulate(SF.load_cu_params())
        s = S.eam_cu_fcc(ncell=5, displace=0.05, seed=15)
        setpot, dt = (lambda c: c.set_eam_alloy(sf, 5.0, S.EV, S.EV)), 1e-3
    runs = (40, 20, 20, 20, 60, 20)
    outs, ths = [], []
    for use_graph in (False, True):
        with gpu_ctx(gpu, s, setpot, 0.3, mixed=True) as ctx:
            ths.append([ctx.run_nve(k, dt, rebuild_every=10, thermo_every=20, use_graph=use_graph) for k in runs])
            outs.append(ctx.download())
    for a, b in zip(*ths):
        assert np.array_equal(a, b)
    for k in outs[0]:
        assert np.array_equal(outs[0][k], outs[1][k]), k


def test_graph_run_equals_stepwise_run(gpu, oracle):
    s = S.lj_fcc(ncell=5, seed=9)
    outs = []
    for use_graph in (False, True):
        with gpu_ctx(gpu, s, LJ, 0.3, mixed=True) as ctx:
            ctx.run_nve(65, 0.005, rebuild_every=10, use_graph=use_graph)
            outs.append(ctx.download())
    for k in outs[0]:
        assert np.array_equal(outs[0][k], outs[1][k]), k


def test_runs_are_bit_reproducible(gpu):
    s = S.lj_fcc(ncell=6, seed=10)
    outs = []
    for _ in range(2):
        with gpu_ctx(gpu, s, LJ, 0.3, mixed=True, tpa=4) as ctx:
            ctx.run_nve(30, 0.005, rebuild_every=10)
            outs.append(ctx.download())
    for k in outs[0]:
        assert np.array_equal(outs[0][k], outs[1][k]), k


def test_upload_positions_triggers_rebuild(gpu, oracle):
    s = _jitter(S.lj_fcc(ncell=5, seed=11), 0.02, 11)
    with gpu_ctx(gpu, s, LJ, 0.3) as ctx:
        ctx.compute_forces()
        # move every atom by 0.2 (> skin/2): the list must be rebuilt
        x2 = s.x + 0.2
        ctx.upload_positions(x2, s.y, s.z)
        ctx.compute_forces()
        d = ctx.download()
        got = per_atom_lists(ctx.export_pairs())
    s2 = s.copy()
    s2.x = x2
    F, ep, _ = _lj_oracle(oracle, s2)
    G = np.stack([d["ax"], d["ay"], d["az"]], 1)
    assert rel_rms(G, F) < FP64_TOL
    ref, _, _ = oracle_lists(oracle, s2, 2.8)
    assert got == ref


def test_nonfinite_force_reported(gpu):
    """Two atoms at the same position: the FP64 path divides by r = 0 and
    the context reports GBMD_ERR_NONFINITE (no device trap)."""
    s = S.lj_fcc(ncell=3, seed=12)
    s.x[1], s.y[1], s.z[1] = s.x[0], s.y[0], s.z[0]
    with gpu_ctx(gpu, s, LJ, 0.3) as ctx:
        with pytest.raises(gpu.GbmdError) as e:
            ctx.run_nve(1, 0.001, rebuild_every=0)
        assert e.value.code == 6


def test_upload_state_download_round_trip(gpu):
    """r, v, a through gbmd_upload_state and back through gbmd_download, in
    the caller's order, bit for bit (batched staging copies + permutation)."""
    s = _jitter(S.lj_fcc(ncell=7, seed=31), 0.05, 31)
    rng = np.random.default_rng(31)
    with gpu_ctx(gpu, s, LJ, 0.3, mixed=True) as ctx:
        ctx.run_nve(12, 0.005, rebuild_every=5)
        d = ctx.download(("x", "y", "z", "vx", "vy", "vz", "ax", "ay", "az"))
        new = {k: d[k] + (rng.normal(0.0, 1e-3, s.n) if k[0] != "x" and k[0] != "y" and k[0] != "z" else 0.0)
               for k in d}
        ctx.upload_state(*(new[k] for k in ("x", "y", "z", "vx", "vy", "vz", "ax", "ay", "az")))
        back = ctx.download(("x", "y", "z", "vx", "vy", "vz", "ax", "ay", "az"))
    for k in new:
        assert np.array_equal(back[k], new[k]), k


@pytest.mark.parametrize("case", ["eam", "lj", "lj_multi", "eam_small_box"])
def test_staged_positions_bit_identical(gpu, oracle, case):
    """Neighbour positions from the block's shared-memory staging give the
    same forces, energies and virials, bit for bit, as the global gathers
    (same list, same arithmetic, same summation order)."""
    if case.startswith("eam"):
        sf, tab, s = _eam_setup(oracle, ncell=3 if case == "eam_small_box" else 9, displace=0.08, seed=41)
        pot = lambda c: c.set_eam_alloy(sf, 5.0, S.EV, S.EV)  # noqa: E731
        skin = 0.3
    elif case == "lj":
        s = _jitter(S.lj_fcc(ncell=12, seed=42), 0.05, 42)
        pot, skin = LJ, 0.3
    else:
        s = _jitter(S.lj_fcc(ncell=10, seed=43), 0.05, 43)
        rng = np.random.default_rng(43)
        s.type = (rng.random(s.n) < 0.2).astype(np.uint8)
        s.masses = np.array([1.0, 2.0])
        eps, sig, rc = S.kob_andersen_tables()
        pot, skin = (lambda c: c.set_lj_multi(eps, sig, rc, 0.0)), 0.3
    out = []
    for staged in (False, True):
        with gpu_ctx(gpu, s, pot, skin, mixed=True, tpa=1, block=256, vec=4) as ctx:
            ctx.set_neighbor_staging(staged)
            ctx.compute_forces(energy=True, virial=True)
            d = ctx.download(virial=True)
            th = ctx.run_nve(30, 1e-3 if case.startswith("eam") else 0.004, rebuild_every=10, thermo_every=10,
                             use_graph=True)
            out.append((d, th))
    (d0, t0), (d1, t1) = out
    for k in ("ax", "ay", "az", "ep", "vir"):
        assert np.array_equal(d0[k], d1[k]), k
    assert np.array_equal(t0, t1)


def test_pinned_host_arrays_round_trip(gpu):
    """Page-locked caller arrays take the direct path (the kernel reads and
    writes host memory in the caller's order): same values as the staged
    copies of pageable arrays, bit for bit."""
    torch = pytest.importorskip("torch")
    s = _jitter(S.lj_fcc(ncell=7, seed=32), 0.05, 32)
    keys = ("x", "y", "z", "vx", "vy", "vz", "ax", "ay", "az")
    with gpu_ctx(gpu, s, LJ, 0.3, mixed=True) as ctx:
        ctx.run_nve(12, 0.005, rebuild_every=5)
        ref = ctx.download(keys)
        pinned = {k: torch.empty(s.n, dtype=torch.float64, pin_memory=True).numpy() for k in keys}
        for k in keys:
            pinned[k][:] = ref[k] * (1.0 + 1e-9)
        ctx.upload_state(*(pinned[k] for k in keys))
        out = {k: torch.empty(s.n, dtype=torch.float64, pin_memory=True).numpy() for k in keys}
        ctx._chk(ctx._L.gbmd_download(ctx.h, *[out[k].ctypes.data for k in keys], None, None))
        back = ctx.download(keys)
    for k in keys:
        assert np.array_equal(out[k], pinned[k]), k
        assert np.array_equal(back[k], pinned[k]), k


@pytest.mark.parametrize("pinned,nsteps,R", [(True, 1, 10), (True, 5, 1), (False, 3, 2)])
def test_run_nve_host_matches_separate_calls(gpu, pinned, nsteps, R):
    """gbmd_run_nve_host (positions copied back during the last force pass)
    gives the state of upload_state + run_nve + download bit for bit, also
    when the last step rebuilds the list (R = 1) and for pageable arrays."""
    torch = pytest.importorskip("torch")
    s = _jitter(S.lj_fcc(ncell=7, seed=33), 0.05, 33)
    keys = ("x", "y", "z", "vx", "vy", "vz", "ax", "ay", "az")
    # two contexts with the same history, so the same rebuild decisions
    with gpu_ctx(gpu, s, LJ, 0.3, mixed=True) as ctx:
        ctx.run_nve(7, 0.005, rebuild_every=5)
        start = ctx.download(keys)
        ctx.upload_state(*(start[k] for k in keys))
        ctx.run_nve(nsteps, 0.005, rebuild_every=R)
        ref = ctx.download(keys)
    with gpu_ctx(gpu, s, LJ, 0.3, mixed=True) as ctx:
        ctx.run_nve(7, 0.005, rebuild_every=5)
        st = {}
        for k in keys:
            st[k] = torch.empty(s.n, dtype=torch.float64, pin_memory=True).numpy() if pinned else np.empty(s.n)
            st[k][:] = start[k]
        ctx.run_nve_host(st, nsteps, 0.005, rebuild_every=R)
    for k in keys:
        assert np.array_equal(st[k], ref[k]), k


def test_upload_argument_errors(gpu):
    """The reference aborts on bad input; the ABI returns a status and the
    context stays usable: too many atoms (checked before any array is read),
    a type outside the species table, a negative count."""
    x = np.zeros(4)
    with gpu.Context(0) as ctx:
        ctx.set_box(np.zeros(3), np.full(3, 10.0))
        ctx.set_species(np.array([1.0]))
        L, h, p = ctx._L, ctx.h, x.ctypes.data
        assert L.gbmd_upload_atoms(h, (1 << 26) + 1, p, p, p, None, None, None, None, None) == 9
        bad = np.array([0, 1, 0, 0], np.uint8)
        assert L.gbmd_upload_atoms(h, 4, p, p, p, None, None, None, bad.ctypes.data, None) == 1
        assert L.gbmd_upload_atoms(h, -1, p, p, p, None, None, None, None, None) == 1
        s = _jitter(S.lj_fcc(ncell=3, seed=2), 0.05, 2)
        ctx.upload_system(s)
        ctx.set_lj(1.0, 1.0, 2.5)
        ctx.set_skin(0.3)
        ctx.compute_forces()
        assert np.isfinite(ctx.download(("ax",))["ax"]).all()


@pytest.mark.parametrize("mixed", [False, True])
def test_list_regrows_for_a_dense_cluster(gpu, oracle, mixed):
    """A dense FCC cluster in a dilute gas: the first per-atom capacity is
    sized from the mean density, the cluster's atoms overflow it, the list is
    regrown and rebuilt; the pair set stays bit-exact and the forces match."""
    rng = np.random.default_rng(21)
    L = 24.0
    pos, _, _ = S.lattice(5, 5, 5, 1.5874, S.FCC_BASIS)   # 500 atoms at rho ~1.0
    pos = pos + 8.0
    gas = rng.uniform(0, L, (300, 3))
    gas = gas[np.any((gas < 6.5) | (gas > 17.5), axis=1)]   # outside the cluster's cube
    P = np.concatenate([pos, gas])
    n = len(P)
    s = S.System(*(np.ascontiguousarray(P[:, k]) for k in range(3)), np.zeros(n), np.zeros(n), np.zeros(n),
                 np.zeros(n, np.uint8), rng.permutation(n).astype(np.uint64), np.zeros(3), np.full(3, L),
                 np.array([1.0]))
    s = _jitter(s, 0.03, 21)
    ref, (x, y, z), nl = oracle_lists(oracle, s, 2.8)
    assert max(len(v) for v in ref.values()) > 1.35 * 4.18879 * 2.8 ** 3 * n / L ** 3 + 16
    fx, fy, fz, ep, _ = oracle.lj_force(x, y, z, nl, s.L, 1.0, 1.0, 2.5)
    F = np.stack([fx, fy, fz], 1)
    with gpu_ctx(gpu, s, LJ, 0.3, mixed=mixed) as ctx:
        ctx.compute_forces(energy=True)
        got = per_atom_lists(ctx.export_pairs())
        d = ctx.download(("ax", "ay", "az"))
    assert got == ref
    G = np.stack([d["ax"], d["ay"], d["az"]], 1)
    assert rel_rms(G, F) < (FP64_TOL if not mixed else MIXED_FORCE_TOL)


def test_consecutive_runs_reuse_current_energies(gpu, oracle):
    """A run that ended on a thermo step leaves its energies and virials
    current: the next run's step-0 row reuses them (only the reduction runs)
    and must equal the same row of one long run, bit for bit; a change of
    velocities (push_f_v) in between is seen by that row."""
    s = _jitter(S.lj_fcc(ncell=6, seed=51), 0.03, 51)
    with gpu_ctx(gpu, s, LJ, 0.3, mixed=True) as ctx:
        long_rows = ctx.run_nve(60, 0.005, rebuild_every=10, thermo_every=20)
        long_state = ctx.download(("x", "y", "z", "vx", "vy", "vz"))
    with gpu_ctx(gpu, s, LJ, 0.3, mixed=True) as ctx:
        a = ctx.run_nve(40, 0.005, rebuild_every=10, thermo_every=20)
        b = ctx.run_nve(20, 0.005, rebuild_every=10, thermo_every=20)
        st = ctx.download(("x", "y", "z", "vx", "vy", "vz"))
        assert np.array_equal(a, long_rows[:3])
        assert np.array_equal(b, long_rows[2:])
        for k in st:
            assert np.array_equal(st[k], long_state[k]), k
        # velocities changed after a thermo step: the kinetic terms follow
        ctx.push_f_v(0.005, 1.0)
        c = ctx.run_nve(0, 0.005, rebuild_every=10, thermo_every=20)
        v = ctx.download(("vx", "vy", "vz"))
        ke = 0.5 * sum((v[k] ** 2).sum() for k in ("vx", "vy", "vz"))
        assert abs(c[0, 21:24].sum() - ke) < 1e-12 * ke
        assert c[0, 24] == b[-1, 24]  # same positions: same potential energy
