"""Displacement-triggered neighbour-list rebuild (particle_displ_over,
config_move_particles.msp L19-22, L116-118) on the GPU.

The trigger is evaluated on the device every step and gates the rebuild
kernels, so it runs inside CUDA graphs too.  Checked against the oracle's
trigger (same FP64 test, same skin/2 threshold): thermo rows and the number
of list builds; graph replay against step-by-step launches bit for bit.
"""
import numpy as np
import pytest

from exastamp_gb300 import setfl
from exastamp_gb300 import systems as S

pytestmark = pytest.mark.gpu

TRIGGER = -1


@pytest.mark.parametrize("use_graph", [False, True])
def test_trigger_fp64_lj_matches_oracle(gpu, oracle, use_graph):
    """Step by step (gated kernels) and in CUDA-graph chunks of 10 steps (the
    rebuild chain in a conditional node set on the device)."""
    s = S.lj_fcc(ncell=10, density=0.8442, T=1.5, seed=5)
    st = s.state()
    th_ref = oracle.run_nve(st, s.masses, s.lo, s.hi, oracle.POT_LJ, oracle.LJParams(1.0, 1.0, 2.5), 0.3, 0.005,
                            150, TRIGGER)
    builds_ref = oracle.last_list_builds()
    every = 10 if use_graph else 1
    with gpu.Context(0) as ctx:
        ctx.upload_system(s)
        ctx.set_lj(1.0, 1.0, 2.5)
        ctx.set_skin(0.3)
        ctx.set_precision(False)
        b0 = ctx.list_builds()
        th = ctx.run_nve(150, 0.005, rebuild_every=TRIGGER, thermo_every=every, use_graph=use_graph)
        builds = ctx.list_builds() - b0
        d = ctx.download(("x", "y", "z"))
    assert 2 < builds_ref < 60
    assert builds == builds_ref
    th_ref = th_ref[::every]
    assert np.allclose(th, th_ref, rtol=1e-9, atol=1e-9 * np.abs(th_ref).max())
    for k in ("x", "y", "z"):
        dd = np.abs(d[k] - st[k])
        assert np.minimum(dd, s.L[0] - dd).max() < 1e-9, k


def test_trigger_graph_matches_step_launches(gpu):
    cfg = setfl.load_cu_params()
    sf = setfl.tabulate(cfg)
    s = S.eam_cu_fcc(ncell=12, a=3.615, T=900.0, seed=8)
    out = []
    for use_graph in (False, True):
        with gpu.Context(0) as ctx:
            ctx.upload_system(s)
            ctx.set_eam_alloy(sf, 5.0, S.EV, S.EV)
            ctx.set_skin(0.3)
            ctx.set_precision(True)
            th = ctx.run_nve(120, 1e-3, rebuild_every=TRIGGER, thermo_every=10, use_graph=use_graph)
            out.append((th, ctx.download(("x", "y", "z", "vx")), ctx.list_builds()))
    (th0, d0, n0), (th1, d1, n1) = out
    assert n0 == n1 and n0 > 2
    assert np.array_equal(th0, th1)
    for k in d0:
        assert np.array_equal(d0[k], d1[k]), k


def test_trigger_minimiser_matches_oracle(gpu, oracle):
    s = S.lj_binary_voids(n=6000, density=1.2, frac_a=0.8, nvoids=1, void_r=2.5, seed=12)
    eps, sig, rc = S.kob_andersen_tables()
    st = s.state()
    oracle.run_minimize(st, s.masses, s.lo, s.hi, oracle.POT_LJ_MULTI,
                        oracle.multi_params(eps, sig, rc, float(rc.max())), 0.3, 0.02, 100.0, 40, TRIGGER)
    builds_ref = oracle.last_list_builds()
    with gpu.Context(0) as ctx:
        ctx.upload_system(s)
        ctx.set_lj_multi(eps, sig, rc, 0.0)
        ctx.set_skin(0.3)
        ctx.set_precision(False)
        ctx.run_minimize(40, 0.02, tolF=100.0, rebuild_every=TRIGGER)
        builds = ctx.list_builds()
        d = ctx.download(("x", "y", "z"))
    assert builds == builds_ref and builds > 2
    for k in ("x", "y", "z"):
        dd = np.abs(d[k] - st[k])
        assert np.minimum(dd, s.L[0] - dd).max() < 1e-8, k


@pytest.mark.parametrize("use_graph", [False, True])
def test_fixed_interval_build_count(gpu, use_graph):
    s = S.lj_fcc(ncell=8, density=0.8442, T=1.0, seed=6)
    with gpu.Context(0) as ctx:
        ctx.upload_system(s)
        ctx.set_lj(1.0, 1.0, 2.5)
        ctx.set_skin(0.3)
        ctx.set_precision(True)
        ctx.build_neighbors()
        b0 = ctx.list_builds()
        ctx.run_nve(101, 0.005, rebuild_every=10, thermo_every=20, use_graph=use_graph)
        assert ctx.list_builds() - b0 == 10


def test_operator_graph_with_check_and_update_particles(gpu, oracle):
    """The verlet_nve operator sequence (config_numerical_schemes.msp L44-52)
    through the operator mirror -- push_f_v_r, push_f_v,
    check_and_update_particles (gbmd_update_neighbors), forces, push_f_v --
    against the oracle's verlet_nve with the displacement trigger: same final
    state within 1e-10 and the same number of list builds."""
    from exastamp_gb300 import operators as OP
    s = S.lj_fcc(ncell=6, T=1.0, seed=41)
    st = s.state()
    nsteps, dt = 60, 0.005
    oracle.run_nve(st, s.masses, s.lo, s.hi, oracle.POT_LJ, oracle.LJParams(1.0, 1.0, 2.5), 0.3, dt, nsteps, -1,
                   thermo=False)
    orc_builds = oracle.last_list_builds()
    sim = OP.Simulation(s)
    force = OP.lj_compute_force(rcut=2.5, parameters={"epsilon": 1.0, "sigma": 1.0})
    force.bind(sim)
    OP.chunk_neighbors().bind(sim, 0.3)
    sim.set_precision(False)
    check = OP.check_and_update_particles()
    p1, p2 = OP.push_f_v_r(dt_scale=1.0), OP.push_f_v(dt_scale=0.5)
    b0 = sim.ctx.list_builds()
    force.execute(sim, energy=False)
    fired = 0
    for _ in range(nsteps):
        p1.execute(sim, dt)
        p2.execute(sim, dt)
        fired += int(check.execute(sim))
        force.execute(sim, energy=False)
        p2.execute(sim, dt)
    d = sim.ctx.download(("x", "y", "z", "vx", "vy", "vz"))
    assert sim.ctx.list_builds() - b0 == orc_builds
    assert fired == orc_builds - 1 and fired > 0
    for k in ("vx", "vy", "vz"):
        assert np.abs(d[k] - st[k]).max() < 1e-10
    for k, dd in (("x", 0), ("y", 1), ("z", 2)):
        diff = d[k] - st[k]
        diff -= np.round(diff / s.L[dd]) * s.L[dd]
        assert np.abs(diff).max() < 1e-10
