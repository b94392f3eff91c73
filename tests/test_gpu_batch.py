"""Batched periodic replicas (persistent launch) against the FP64 oracle.

Bars: forces within 1e-5 relative RMS and per-atom energies within 1e-6 of
the oracle (mixed precision, eV units); per-replica virial within 1e-5;
parameter gradient within 1e-4 relative of the FP64 oracle adjoint (itself
checked against finite differences in tests/test_oracle.py); persistent,
one-launch-per-replica and CUDA-graph runs bit-identical.
"""
import numpy as np
import pytest

from exastamp_gb300 import setfl as SF
from exastamp_gb300 import systems as S

pytestmark = pytest.mark.gpu


def _replicas(nrep, seed, nmax=400):
    reps = S.replica_set(nrep=nrep, nmin=32, nmax=nmax, seed=seed)
    return reps


def _oracle_forward(oracle, reps, tab):
    F, E, V = [], [], []
    for s in reps:
        x, y, z = s.x.copy(), s.y.copy(), s.z.copy()
        oracle.wrap(x, y, z, s.lo, s.hi)
        nl = oracle.build_neighbors(x, y, z, s.id, s.lo, s.hi, 5.0)
        fx, fy, fz, ep, vir, _, _ = oracle.eam_forces(x, y, z, s.type, nl, s.L, tab, 5.0)
        F.append(np.stack([fx, fy, fz], 1))
        E.append(ep)
        V.append(vir.sum(0))
    return np.concatenate(F), np.concatenate(E), np.stack(V)


@pytest.fixture(scope="module")
def cu():
    cfg = SF.load_cu_params()
    return cfg, SF.tabulate(cfg)


@pytest.mark.parametrize("stencil,nmax", [(1, 400), (2, 400), (1, 1500), (2, 1500)])
def test_batch_forward_matches_oracle(gpu, oracle, cu, stencil, nmax):
    """nmax 400: only the small-replica kernel; 1500: both kernels."""
    cfg, sf = cu
    reps = _replicas(24, seed=31, nmax=nmax)
    if nmax > 512:
        assert any(s.n > 512 for s in reps) and any(s.n <= 512 for s in reps)
    tab = oracle.EamOracleTables.from_setfl(sf, 1.0, 1.0, rcut=5.0)
    F, E, V = _oracle_forward(oracle, reps, tab)
    with gpu.Batch(0) as b:
        b.set_eam_alloy(sf, 5.0)
        b.upload(reps)
        b.set_launch(256, stencil)
        b.run()
        d = b.download()
    err = np.sqrt(((d["F"] - F) ** 2).sum() / (F ** 2).sum())
    assert err < 1e-5, err
    assert np.abs(d["ep"] - E).max() < 1e-6 * np.abs(E).max()
    assert np.allclose(d["e_rep"], [e.sum() for e in np.split(E, np.cumsum([s.n for s in reps])[:-1])],
                       rtol=1e-6)
    assert np.sqrt(((d["vir_rep"] - V) ** 2).sum() / (V ** 2).sum()) < 1e-5


def test_batch_dense_replica_walks_the_cells(gpu, oracle, cu):
    """A replica compressed so far that its atoms have more pairs than the
    per-atom list holds (128) is evaluated from the cells instead; both kinds
    of replica in one launch match the oracle."""
    cfg, sf = cu
    reps = _replicas(6, seed=35)
    pos, lo, hi = S.lattice(4, 4, 4, 2.45, S.FCC_BASIS)
    rng = np.random.default_rng(35)
    pos = pos + rng.normal(0.0, 0.03, pos.shape)
    reps.insert(2, S._make(pos, lo, hi, np.zeros(len(pos)), np.array([63.546]), np.zeros_like(pos), {}))
    tab = oracle.EamOracleTables.from_setfl(sf, 1.0, 1.0, rcut=5.0)
    F, E, V = _oracle_forward(oracle, reps, tab)
    x, y, z = reps[2].x.copy(), reps[2].y.copy(), reps[2].z.copy()
    oracle.wrap(x, y, z, reps[2].lo, reps[2].hi)
    nl = oracle.build_neighbors(x, y, z, reps[2].id, reps[2].lo, reps[2].hi, 5.0)
    assert np.diff(nl.off).max() > 128
    with gpu.Batch(0) as b:
        b.set_eam_alloy(sf, 5.0)
        b.upload(reps)
        b.run()
        d = b.download()
    err = np.sqrt(((d["F"] - F) ** 2).sum() / (F ** 2).sum())
    assert err < 1e-5, err
    # the dense replica sums ~140 strongly repulsive pair energies per atom
    # (+15 eV per atom) in FP32: 2e-6 relative
    assert np.abs(d["ep"] - E).max() < 2e-6 * np.abs(E).max()


def test_batch_launch_modes_are_identical(gpu, cu):
    cfg, sf = cu
    reps = _replicas(40, seed=32, nmax=800)
    outs = []
    for per_replica, graph in ((False, False), (True, False), (False, True)):
        with gpu.Batch(0) as b:
            b.set_eam_alloy(sf, 5.0)
            b.upload(reps)
            b.run(per_replica=per_replica, use_graph=graph)
            if graph:
                b.run(use_graph=True)   # replay
            outs.append(b.download())
    for o in outs[1:]:
        assert np.array_equal(o["F"], outs[0]["F"]) and np.array_equal(o["ep"], outs[0]["ep"])
        assert np.array_equal(o["vir_rep"], outs[0]["vir_rep"])


def _adjoint_problem(oracle, cfg, nconf=6, seed=4, ncell=4):
    confs = S.adjoint_training_set(nconf=nconf, ncell=ncell, seed=seed)
    rng = np.random.default_rng(5)
    pert = {k: v * rng.uniform(0.9, 1.1) for k, v in cfg["params"].items()}
    tab_t = oracle.EamOracleTables.from_setfl(SF.tabulate(cfg, pert), 1.0, 1.0, rcut=5.0)
    Ft, Et, _ = _oracle_forward(oracle, confs, tab_t)
    return confs, Ft, Et


@pytest.mark.parametrize("ncell", [4, 6])
def test_batch_adjoint_matches_fp64_oracle_gradient(gpu, oracle, cu, ncell):
    """ncell 4: 243-atom configurations (small-replica kernel); 6: ~820 atoms
    (large-replica kernel)."""
    cfg, sf = cu
    confs, Ft, Et = _adjoint_problem(oracle, cfg, nconf=6 if ncell == 4 else 3, ncell=ncell)
    assert all((c.n > 512) == (ncell == 6) for c in confs)
    ntot = sum(c.n for c in confs)
    wF, wE = 1.0 / ntot, 0.1 / ntot
    # FP64 oracle loss and gradient
    tab = oracle.EamOracleTables.from_setfl(sf, 1.0, 1.0, rcut=5.0)
    dsp = oracle.EamDerivativeSplines(cfg)
    loss_ref, grad_ref, o = 0.0, np.zeros(9), 0
    for c in confs:
        x, y, z = c.x.copy(), c.y.copy(), c.z.copy()
        oracle.wrap(x, y, z, c.lo, c.hi)
        nl = oracle.build_neighbors(x, y, z, c.id, c.lo, c.hi, 5.0)
        l, g, _, _ = oracle.eam_loss_grad(x, y, z, nl, c.L, tab, 5.0, dsp, Ft[o:o + c.n], Et[o:o + c.n], wF, wE)
        loss_ref += l
        grad_ref += g
        o += c.n
    J_F, J_f, J_z = SF.table_param_jacobian(cfg)
    with gpu.Batch(0) as b:
        b.set_eam_alloy(sf, 5.0)
        b.set_param_derivatives(J_F, J_f, J_z)
        b.upload(confs)
        b.set_targets(Ft, Et, wF, wE)
        b.run(adjoint=True)
        d = b.download()
    assert abs(d["loss"] - loss_ref) < 1e-5 * abs(loss_ref)
    rel = np.abs(d["grad"] - grad_ref) / np.maximum(np.abs(grad_ref), 1e-3 * np.abs(grad_ref).max())
    assert rel.max() < 1e-4, (rel, d["grad"], grad_ref)


def test_batch_rejects_oversized_replica(gpu, cu):
    cfg, sf = cu
    big = S.eam_cu_fcc(ncell=9)   # 2916 atoms > 2048
    with gpu.Batch(0) as b:
        b.set_eam_alloy(sf, 5.0)
        with pytest.raises(gpu.GbmdError) as e:
            b.upload([big])
        assert e.value.code == 9
