"""Parameter adjoints through the torch.autograd.Function bindings:
gradients from backward() against central finite differences of the same
forward (relative 1e-4, the adjoint target) and against the FP64 oracle's
analytic gradients."""
import numpy as np
import pytest

from exastamp_gb300 import setfl as SF
from exastamp_gb300 import systems as S

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _lj_problem(oracle):
    s = S.lj_fcc(ncell=5, density=0.8442, T=1.0, seed=19)
    rng = np.random.default_rng(19)
    s.x, s.y, s.z = (a + rng.normal(0.0, 0.05, s.n) for a in (s.x, s.y, s.z))
    x, y, z = s.x.copy(), s.y.copy(), s.z.copy()
    oracle.wrap(x, y, z, s.lo, s.hi)
    nl = oracle.build_neighbors(x, y, z, s.id, s.lo, s.hi, 2.8)
    fx, fy, fz, ep, _ = oracle.lj_force(x, y, z, nl, s.L, 1.1, 0.97, 2.5)  # targets: perturbed parameters
    return s, (x, y, z, nl), np.stack([fx, fy, fz], 1), ep


@pytest.mark.parametrize("mixed", [False, True])
def test_lj_autograd_gradient(gpu, oracle, mixed):
    from exastamp_gb300.autograd import LJLoss
    s, (x, y, z, nl), Ft, Et = _lj_problem(oracle)
    wF, wE = 1.0 / s.n, 0.1 / s.n
    with gpu.Context(0) as ctx:
        ctx.upload_system(s)
        ctx.set_lj(1.0, 1.0, 2.5)
        ctx.set_skin(0.3)
        ctx.set_precision(mixed)
        p = torch.tensor([1.0, 1.0], dtype=torch.float64, requires_grad=True)
        loss = LJLoss.apply(p, ctx, 2.5, Ft, Et, wF, wE)
        loss.backward()
        g = p.grad.numpy().copy()
        h = 1e-4
        fd = np.zeros(2)
        for k in range(2):
            pp, pm = p.detach().clone(), p.detach().clone()
            pp[k] += h
            pm[k] -= h
            fd[k] = (float(LJLoss.apply(pp, ctx, 2.5, Ft, Et, wF, wE))
                     - float(LJLoss.apply(pm, ctx, 2.5, Ft, Et, wF, wE))) / (2 * h)
    loss_ref, g_ref = oracle.lj_loss_grad(x, y, z, nl, s.L, 1.0, 1.0, 2.5, Ft, Et, wF, wE)
    # FP64: 1e-4 (the adjoint target); mixed: the forward's FP32 forces put
    # ~1e-7 relative noise on the loss, i.e. ~1e-4 on differences over h = 1e-4
    fd_tol = 1e-4 if not mixed else 1e-3
    assert np.all(np.abs(g - fd) < fd_tol * np.abs(fd)), (g, fd)
    tol = 1e-9 if not mixed else 1e-4
    assert np.all(np.abs(g - g_ref) < tol * np.abs(g_ref)), (g, g_ref)
    assert abs(float(loss.detach()) - loss_ref) < (1e-9 if not mixed else 1e-4) * loss_ref


def test_eam_autograd_gradient(gpu, oracle):
    from exastamp_gb300.autograd import EamLoss
    cfg = SF.load_cu_params()
    names = SF.PARAM_NAMES
    confs = S.adjoint_training_set(nconf=12, ncell=4, seed=24)
    rng = np.random.default_rng(25)
    pert = {k: v * rng.uniform(0.95, 1.05) for k, v in cfg["params"].items()}
    ntot = sum(c.n for c in confs)
    with gpu.Batch(0) as b:
        b.upload(confs)
        b.set_eam_alloy(SF.tabulate(cfg, pert), 5.0)
        b.run()
        t = b.download()
        Ft, Et = t["F"], t["ep"]
        wF, wE = 1.0 / ntot, 0.1 / ntot
        p = torch.tensor([cfg["params"][k] for k in names], dtype=torch.float64, requires_grad=True)
        loss = EamLoss.apply(p, b, cfg, 5.0, Ft, Et, wF, wE)
        loss.backward()
        g = p.grad.numpy().copy()
        # central differences of the forward, on the three largest components
        fd = {}
        for k in np.argsort(-np.abs(g))[:3]:
            h = 1e-4 * abs(float(p.detach()[k]))
            pp, pm = p.detach().clone(), p.detach().clone()
            pp[k] += h
            pm[k] -= h
            fd[k] = (float(EamLoss.apply(pp, b, cfg, 5.0, Ft, Et, wF, wE))
                     - float(EamLoss.apply(pm, b, cfg, 5.0, Ft, Et, wF, wE))) / (2 * h)
    # the forward is mixed precision: its finite differences carry FP32 noise
    for k, v in fd.items():
        assert abs(g[k] - v) < 2e-3 * abs(v), (names[k], g[k], v)
    # FP64 oracle gradient (itself checked against finite differences)
    tab = oracle.EamOracleTables.from_setfl(SF.tabulate(cfg), 1.0, 1.0, rcut=5.0)
    dsp = oracle.EamDerivativeSplines(cfg)
    g_ref, o = np.zeros(9), 0
    for c in confs:
        x, y, z = c.x.copy(), c.y.copy(), c.z.copy()
        oracle.wrap(x, y, z, c.lo, c.hi)
        nl = oracle.build_neighbors(x, y, z, c.id, c.lo, c.hi, 5.0)
        _, gg, _, _ = oracle.eam_loss_grad(x, y, z, nl, c.L, tab, 5.0, dsp, Ft[o:o + c.n], Et[o:o + c.n], wF, wE)
        g_ref += gg
        o += c.n
    rel = np.abs(g - g_ref) / np.maximum(np.abs(g_ref), 1e-3 * np.abs(g_ref).max())
    assert rel.max() < 1e-4, (rel, g, g_ref)


def test_lj_multi_loss_gradient(gpu, oracle):
    """lj_multi_force adjoint (FP64 forward): each species pair's dL/deps and
    dL/dsigma within 1e-4 of central finite differences of the loss; with
    every pair given the same (eps, sigma, rc), the gradients summed over the
    pairs equal the single-species adjoint."""
    s = S.lj_fcc(ncell=4, seed=31)
    rng = np.random.default_rng(31)
    for a in (s.x, s.y, s.z):
        a += rng.normal(0.0, 0.05, s.n)
    s.type = (rng.random(s.n) < 0.3).astype(np.uint8)
    s.masses = np.array([1.0, 1.5])
    eps, sig, rc = S.kob_andersen_tables()
    wF, wE = 1.0 / s.n, 0.1 / s.n

    def run(ctx, e, g, r):
        ctx.set_lj_multi(e, g, r, 0.0)
        return ctx.lj_multi_loss_grad(Ft, Et, wF, wE)

    with gpu.Context(0) as ctx:
        ctx.upload_system(s)
        ctx.set_skin(0.3)
        ctx.set_precision(False)
        ctx.set_lj_multi(eps * 1.05, sig * 0.98, rc, 0.0)  # targets from perturbed tables
        ctx.compute_forces(energy=True)
        d = ctx.download()
        Ft = np.stack([d["ax"], d["ay"], d["az"]], 1) * s.masses[s.type][:, None]
        Et = d["ep"].copy()
        loss, ge, gs = run(ctx, eps, sig, rc)
        assert loss > 0 and np.allclose(ge, ge.T) and np.allclose(gs, gs.T)
        h = 1e-6
        for a, b in ((0, 0), (0, 1), (1, 1)):
            for tab, g in ((eps, ge), (sig, gs)):
                p, m = tab.copy(), tab.copy()
                p[a, b] += h; p[b, a] = p[a, b]
                m[a, b] -= h; m[b, a] = m[a, b]
                lp = run(ctx, p, sig, rc)[0] if tab is eps else run(ctx, eps, p, rc)[0]
                lm = run(ctx, m, sig, rc)[0] if tab is eps else run(ctx, eps, m, rc)[0]
                fd = (lp - lm) / (2 * h)
                assert abs(g[a, b] - fd) < 1e-4 * abs(fd) + 1e-12, (a, b, g[a, b], fd)
        # one species in disguise: the same parameters for every pair
        one = np.ones((2, 2))
        l2, ge2, gs2 = run(ctx, one, one, one * 2.5)
        ctx.set_lj(1.0, 1.0, 2.5)
        l1, g1 = ctx.lj_loss_grad(Ft, Et, wF, wE)
    assert abs(l2 - l1) < 1e-10 * abs(l1)
    su = lambda m: m[0, 0] + m[0, 1] + m[1, 1]  # noqa: E731  (one entry per unordered pair)
    assert abs(su(ge2) - g1[0]) < 1e-9 * abs(g1[0])
    assert abs(su(gs2) - g1[1]) < 1e-9 * abs(g1[1])


def test_lj_multi_autograd_symmetric_parametrisation(gpu):
    """LJMultiLoss through a symmetric parametrisation (upper triangle ->
    U + U.T - diag): torch's gradient equals the adjoint's per-pair one."""
    from exastamp_gb300.autograd import LJMultiLoss
    s = S.lj_fcc(ncell=4, seed=32)
    rng = np.random.default_rng(32)
    for a in (s.x, s.y, s.z):
        a += rng.normal(0.0, 0.05, s.n)
    s.type = (rng.random(s.n) < 0.3).astype(np.uint8)
    s.masses = np.array([1.0, 1.5])
    eps, sig, rc = S.kob_andersen_tables()
    wF, wE = 1.0 / s.n, 0.1 / s.n
    with gpu.Context(0) as ctx:
        ctx.upload_system(s)
        ctx.set_skin(0.3)
        ctx.set_precision(False)
        ctx.set_lj_multi(eps * 0.95, sig * 1.02, rc, 0.0)
        ctx.compute_forces(energy=True)
        d = ctx.download()
        Ft = np.stack([d["ax"], d["ay"], d["az"]], 1) * s.masses[s.type][:, None]
        Et = d["ep"].copy()
        iu = np.triu_indices(2)
        ue = torch.tensor(eps[iu], dtype=torch.float64, requires_grad=True)
        us = torch.tensor(sig[iu], dtype=torch.float64, requires_grad=True)

        def sym(u):
            m = torch.zeros(2, 2, dtype=torch.float64)
            m = m.index_put((torch.tensor(iu[0]), torch.tensor(iu[1])), u)
            return m + m.T - torch.diag(torch.diag(m))

        loss = LJMultiLoss.apply(sym(ue), sym(us), ctx, rc, Ft, Et, wF, wE)
        loss.backward()
        ref_loss, ge, gs = ctx.lj_multi_loss_grad(Ft, Et, wF, wE)
    assert abs(float(loss.detach()) - ref_loss) < 1e-12 * ref_loss
    assert np.allclose(ue.grad.numpy(), ge[iu], rtol=1e-12, atol=0)
    assert np.allclose(us.grad.numpy(), gs[iu], rtol=1e-12, atol=0)
