"""Two-level neighbour list (gbmd_set_list_buffer), called through the C ABI.

A full build also makes an outer list of radius rcut + skin + d with the sort
into cells; every later rebuild filters the list the pair kernels read from
it and runs the outer build again only when some atom moved more than d/2
since it was built.

Bars:
  * after rebuilds without an outer build, the filtered list holds exactly
    the pairs of a fresh build at the same positions (pair ids and
    separations; the rows keep the outer build's cell order);
  * FP64 trajectories track the oracle's fixed-interval rebuilds within
    1e-10 (positions modulo the box: between outer builds the coordinates
    run on past the box faces);
  * the outer build runs again when atoms moved more than d/2 (small d) and
    not otherwise (large d);
  * graph replays equal step-by-step runs bit for bit, with fixed-interval
    rebuilds and with the displacement trigger;
  * an explicit build is a full one (wrap, rebin, outer list);
  * a box edge shorter than the outer radius is refused.
"""
import numpy as np
import pytest

from exastamp_gb300 import setfl as SF
from exastamp_gb300 import systems as S

from pairset_compare import assert_same_pair_sets
from test_gpu_parity import LJ, _jitter, gpu_ctx, rel_rms

pytestmark = pytest.mark.gpu

INVALID = 1  # GBMD_ERR_INVALID
MIXED_FORCE_TOL = 1e-5


def _pair_table(rows, pos, ids, L):
    """(sorted keys id_i * n + id_j, separations) of an exported pair list,
    separations from the given positions (upload order) and the images."""
    a, b, img = rows
    n = len(ids)
    where = np.empty(n, np.int64)
    where[ids] = np.arange(n)
    ia, ib = where[a.astype(np.int64)], where[b.astype(np.int64)]
    sep = np.stack([pos[d][ib] + img[:, d] * L[d] - pos[d][ia] for d in range(3)], 1)
    key = a.astype(np.int64) * n + b.astype(np.int64)
    o = np.argsort(key, kind="stable")
    return key[o], sep[o]


def _fresh_rows(oracle, pos, s, R):
    x, y, z = (p.copy() for p in pos)
    oracle.wrap(x, y, z, s.lo, s.hi)
    nl = oracle.build_neighbors(x, y, z, s.id, s.lo, s.hi, R)
    pairs = nl.pairs_with_ids(s.id)
    rows = (pairs[:, 0].astype(np.uint64), pairs[:, 1].astype(np.uint64), pairs[:, 2:5].astype(np.int8))
    return rows, (x, y, z)


def _min_image(d, L):
    return np.abs(d - L * np.round(d / L))


@pytest.mark.parametrize("mixed", [False, True])
def test_filtered_list_holds_the_pairs_of_a_fresh_build(gpu, oracle, mixed):
    s = _jitter(S.lj_fcc(ncell=10, T=0.1, seed=11), 0.03, 11)
    with gpu_ctx(gpu, s, LJ, 0.3, mixed=mixed) as ctx:
        ctx.set_list_buffer(1.0)
        ctx.run_nve(30, 0.005, rebuild_every=10)
        buf, outer = ctx.list_buffer()
        builds = ctx.list_builds()
        rows = ctx.export_pairs_raw()
        d = ctx.download(("x", "y", "z"))
    assert buf == 1.0 and outer == 1 and builds == 4  # one full build, three filtered
    pos = (d["x"], d["y"], d["z"])
    fresh, wrapped = _fresh_rows(oracle, pos, s, 2.8)
    kg, sg = _pair_table(rows, pos, s.id, s.L)
    ko, so = _pair_table(fresh, wrapped, s.id, s.L)
    assert np.array_equal(kg, ko)
    assert np.abs(sg - so).max() < 1e-9


def test_fp64_nve_tracks_the_oracle(gpu, oracle):
    """Fixed rebuilds every 10 steps; d = 0.4 sigma at T* = 1: some rebuilds
    filter, some rebuild the outer list."""
    s = S.lj_fcc(ncell=8, seed=12)
    st = s.state()
    th_ref = oracle.run_nve(st, s.masses, s.lo, s.hi, oracle.POT_LJ, oracle.LJParams(1.0, 1.0, 2.5), 0.3, 0.005,
                            60, 10)
    with gpu_ctx(gpu, s, LJ, 0.3, mixed=False) as ctx:
        ctx.set_list_buffer(0.4)
        th = ctx.run_nve(60, 0.005, rebuild_every=10, thermo_every=1)
        _, outer = ctx.list_buffer()
        d = ctx.download()
    assert 1 < outer < 7, outer
    for k in ("x", "y", "z"):
        assert _min_image(d[k] - st[k], s.L[0]).max() < 1e-10, k
    for k in ("vx", "ax"):
        assert np.abs(d[k] - st[k]).max() < 1e-10, k
    assert np.allclose(th, th_ref, rtol=1e-9, atol=1e-9)


@pytest.mark.parametrize("buffer,expect", [(0.05, "every"), (2.0, "once")])
def test_outer_build_runs_when_atoms_moved_half_the_buffer(gpu, buffer, expect):
    """T* = 1: in 10 steps of 0.005 the fastest atoms move ~0.2 sigma (more
    than 0.025), in 20 steps less than 1.0."""
    s = S.lj_fcc(ncell=10, seed=13)
    with gpu_ctx(gpu, s, LJ, 0.3, mixed=True) as ctx:
        ctx.set_list_buffer(buffer)
        ctx.run_nve(20, 0.005, rebuild_every=10)
        _, outer = ctx.list_buffer()
        builds = ctx.list_builds()
    assert builds == 3
    assert outer == (3 if expect == "every" else 1), outer


@pytest.mark.parametrize("rebuild_every", [10, -1])
def test_graph_replay_equals_stepwise_run(gpu, rebuild_every):
    """EAM Cu, mixed precision: the captured rebuilds (the outer build in a
    conditional node, the displacement trigger's in another) give the
    arrays of the step-by-step run bit for bit."""
    sf = SF.tabulate(SF.load_cu_params())
    s = S.eam_cu_fcc(ncell=10, T=600.0, seed=14)
    out = []
    for use_graph in (False, True):
        with gpu_ctx(gpu, s, lambda c: c.set_eam_alloy(sf, 5.0, S.EV, S.EV), 0.3, mixed=True) as ctx:
            ctx.set_list_buffer(0.3)
            th = ctx.run_nve(80, 1e-3, rebuild_every=rebuild_every, thermo_every=20, use_graph=use_graph)
            out.append((th, ctx.download(), ctx.list_builds(), ctx.list_buffer()[1]))
    (t0, d0, b0, o0), (t1, d1, b1, o1) = out
    assert b0 == b1 and o0 == o1 and o0 >= 2, (b0, b1, o0, o1)
    assert np.array_equal(t0, t1)
    for k in ("x", "y", "z", "vx", "vy", "vz", "ax", "ay", "az"):
        assert np.array_equal(d0[k], d1[k]), k


def test_trigger_run_tracks_single_level_run(gpu):
    """Displacement-triggered rebuilds, FP64: the two-level run and the
    plain one rebuild on the same steps and stay within 1e-10."""
    s = S.lj_fcc(ncell=8, seed=15)
    out = []
    for buffer in (0.0, 0.4):
        with gpu_ctx(gpu, s, LJ, 0.3, mixed=False) as ctx:
            ctx.set_list_buffer(buffer)
            th = ctx.run_nve(60, 0.005, rebuild_every=-1, thermo_every=10)
            out.append((th, ctx.download(), ctx.list_builds()))
    (t0, d0, b0), (t1, d1, b1) = out
    assert b0 == b1 and b0 >= 3
    assert np.allclose(t0, t1, rtol=1e-10, atol=1e-10)
    for k in ("x", "y", "z"):
        assert _min_image(d1[k] - d0[k], s.L[0]).max() < 1e-10, k


def test_eam_forces_after_filtered_rebuilds_match_oracle(gpu, oracle):
    sf = SF.tabulate(SF.load_cu_params())
    tab = oracle.EamOracleTables.from_setfl(sf, S.EV, S.EV, rcut=5.0)
    s = S.eam_cu_fcc(ncell=10, seed=16)
    with gpu_ctx(gpu, s, lambda c: c.set_eam_alloy(sf, 5.0, S.EV, S.EV), 0.3, mixed=True) as ctx:
        ctx.set_list_buffer(0.6)
        ctx.run_nve(30, 1e-3, rebuild_every=10, use_graph=True)
        assert ctx.list_buffer()[1] == 1
        d = ctx.download(("x", "y", "z"))
        ctx.compute_forces(energy=True)
        dm = ctx.download(("ax", "ay", "az", "ep"))
        ctx.set_precision(False)
        ctx.compute_forces(energy=True)
        d64 = ctx.download(("ax", "ay", "az", "ep"))
    x, y, z = d["x"].copy(), d["y"].copy(), d["z"].copy()
    oracle.wrap(x, y, z, s.lo, s.hi)
    nl = oracle.build_neighbors(x, y, z, s.id, s.lo, s.hi, 5.3)
    fx, fy, fz, ep, _, _, _ = oracle.eam_forces(x, y, z, s.type, nl, s.L, tab, 5.0)
    F = np.stack([fx, fy, fz], 1) / s.masses[0]
    G64 = np.stack([d64["ax"], d64["ay"], d64["az"]], 1)
    assert rel_rms(G64, F) < 1e-12
    assert np.abs(d64["ep"] - ep).max() < 1e-12 * np.abs(ep).max()
    G = np.stack([dm["ax"], dm["ay"], dm["az"]], 1)
    assert rel_rms(G, F) < MIXED_FORCE_TOL


def test_explicit_build_is_a_full_build(gpu, oracle):
    """gbmd_build_neighbors wraps, rebins and builds the outer list again
    (the positions come back inside the box) and its filtered list is the
    pair set of a fresh build; with the buffer off again the rows are in the
    oracle's canonical order."""
    s = S.lj_fcc(ncell=8, seed=17)
    with gpu_ctx(gpu, s, LJ, 0.3, mixed=True) as ctx:
        ctx.set_list_buffer(0.5)
        ctx.run_nve(20, 0.005, rebuild_every=10)
        outer = ctx.list_buffer()[1]
        ctx.build_neighbors()
        assert ctx.list_buffer()[1] == outer + 1
        rows = ctx.export_pairs_raw()
        d = ctx.download(("x", "y", "z"))
        ctx.set_list_buffer(0.0)
        ctx.build_neighbors()
        rows0 = ctx.export_pairs_raw()
    pos = (d["x"], d["y"], d["z"])
    for k in range(3):
        assert (pos[k] >= s.lo[k]).all() and (pos[k] < s.hi[k]).all()
    fresh, wrapped = _fresh_rows(oracle, pos, s, 2.8)
    kg, sg = _pair_table(rows, pos, s.id, s.L)
    ko, so = _pair_table(fresh, wrapped, s.id, s.L)
    assert np.array_equal(kg, ko)
    assert np.abs(sg - so).max() < 1e-9
    nl = oracle.build_neighbors(*wrapped, s.id, s.lo, s.hi, 2.8)
    assert_same_pair_sets(rows0, nl, s.id)


def test_box_shorter_than_the_outer_radius_is_refused(gpu):
    s = S.lj_fcc(ncell=2, seed=18)  # box edge 3.36 sigma
    with gpu_ctx(gpu, s, LJ, 0.3) as ctx:
        ctx.set_list_buffer(0.6)      # outer radius 3.4
        with pytest.raises(gpu.GbmdError) as e:
            ctx.build_neighbors()
        assert e.value.code == INVALID
        ctx.set_list_buffer(0.0)
        ctx.build_neighbors()
    with gpu.Context(0) as ctx:
        for bad in (-1.0, float("nan"), float("inf")):
            with pytest.raises(gpu.GbmdError):
                ctx.set_list_buffer(bad)


def test_newton3_half_list_filtered(gpu):
    """Newton-3 half lists (each unordered pair once, j after i in the outer
    build's cell order) filtered from a half outer list: 40 NVE steps stay
    within 1e-6 of the same run on the one-level half list."""
    s = S.lj_fcc(ncell=8, seed=19)
    out = []
    for buffer in (0.0, 0.5):
        with gpu_ctx(gpu, s, LJ, 0.3, mixed=True, tpa=1, block=256, vec=4) as ctx:
            ctx.set_newton3(True)
            ctx.set_list_buffer(buffer)
            th = ctx.run_nve(40, 0.005, rebuild_every=10, thermo_every=10)
            out.append((th, ctx.download(), ctx.list_builds()))
    (t0, d0, b0), (t1, d1, b1) = out
    assert b0 == b1
    for k in ("x", "y", "z"):
        assert _min_image(d1[k] - d0[k], s.L[0]).max() < 1e-6, k
    e0 = t0[:, 21:24].sum(1) + t0[:, 24]
    e1 = t1[:, 21:24].sum(1) + t1[:, 24]
    assert np.abs(e1 - e0).max() < 1e-6 * np.abs(e0).max()


@pytest.mark.parametrize("mixed", [False, True])
def test_split_eam_passes_on_the_filtered_list(gpu, mixed):
    """eam_rho then eam_force on a filtered list give the fused pass bit for
    bit; after more steps (ending with a filtered rebuild) a force pass
    needs a new density pass."""
    sf = SF.tabulate(SF.load_cu_params())
    s = S.eam_cu_fcc(ncell=8, seed=20)
    with gpu_ctx(gpu, s, lambda c: c.set_eam_alloy(sf, 5.0, S.EV, S.EV), 0.3, mixed=mixed) as ctx:
        ctx.set_list_buffer(0.6)
        ctx.run_nve(30, 1e-3, rebuild_every=10)
        assert ctx.list_buffer()[1] == 1
        ctx.compute_forces(energy=True, virial=True)
        fused = ctx.download(virial=True)
        ctx.compute_forces(energy=True, virial=True, passes="density")
        ctx.compute_forces(energy=True, virial=True, passes="force")
        split = ctx.download(virial=True)
        for k in ("ax", "ay", "az", "ep", "vir"):
            assert np.array_equal(split[k], fused[k]), k
        ctx.compute_forces(passes="density")
        ctx.run_nve(10, 1e-3, rebuild_every=10)   # ends with a filtered rebuild
        assert ctx.list_buffer()[1] == 1
        with pytest.raises(gpu.GbmdError) as e:
            ctx.compute_forces(passes="force")
        assert e.value.code == INVALID
