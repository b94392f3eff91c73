"""The Lennard-Jones workloads end to end on the GPU against the oracle.

* FCC 20^3 cells, 32,000 atoms, rho* 0.8442, rc 2.5, skin 0.3, T* 1, dt 0.005,
  100 NVE steps, rebuild every 10: FP64 GPU thermo rows within 1e-9 of the
  oracle's at every step, final positions within 1e-9, final pair set
  bit-exact; mixed precision within 1e-5 relative RMS force and its energy
  drift reported.
* Binary A/B mixture with voids (reduced size): lj_multi_force with per-pair
  cutoffs 2.5 sigma_ab, mixed vs FP64 forces, the clipped minimiser against
  the oracle's.
"""
import numpy as np
import pytest

from exastamp_gb300 import systems as S

pytestmark = pytest.mark.gpu


def _lists(rows):
    out = {}
    for r in rows:
        out.setdefault(int(r[0]), []).append(tuple(int(v) for v in r[1:]))
    return out


def test_lj_fcc_32000_atoms_100_steps(gpu, oracle):
    s = S.lj_fcc(ncell=20, density=0.8442, T=1.0, seed=1)
    st = s.state()
    th_ref = oracle.run_nve(st, s.masses, s.lo, s.hi, oracle.POT_LJ, oracle.LJParams(1.0, 1.0, 2.5), 0.3, 0.005,
                            100, 10)
    with gpu.Context(0) as ctx:
        ctx.upload_system(s)
        ctx.set_lj(1.0, 1.0, 2.5)
        ctx.set_skin(0.3)
        ctx.set_precision(False)
        th = ctx.run_nve(100, 0.005, rebuild_every=10, thermo_every=1)
        d = ctx.download()
        ctx.build_neighbors()
        got = _lists(ctx.export_pairs())
    assert np.allclose(th, th_ref, rtol=1e-9, atol=1e-9 * np.abs(th_ref).max())
    for k in ("x", "y", "z", "vx"):
        assert np.abs(d[k] - st[k]).max() < 1e-9, k
    x, y, z = st["x"].copy(), st["y"].copy(), st["z"].copy()
    oracle.wrap(x, y, z, s.lo, s.hi)
    ref = _lists(oracle.build_neighbors(x, y, z, s.id, s.lo, s.hi, 2.8).pairs_with_ids(s.id))
    assert got == ref
    # mixed precision on the same system: forces vs FP64 once the lattice has
    # thermalised (on the perfect lattice they vanish by symmetry), then the
    # energy drift of a mixed run
    with gpu.Context(0) as ctx:
        ctx.upload_system(s)
        ctx.set_lj(1.0, 1.0, 2.5)
        ctx.set_skin(0.3)
        ctx.set_precision(False)
        ctx.run_nve(20, 0.005, rebuild_every=10)
        ctx.set_precision(True)
        ctx.compute_forces()
        am = ctx.download(("ax", "ay", "az"))
        ctx.set_precision(False)
        ctx.compute_forces()
        a64 = ctx.download(("ax", "ay", "az"))
        ctx.set_precision(True)
        thm = ctx.run_nve(100, 0.005, rebuild_every=10, thermo_every=10, use_graph=True)
    A = np.stack([am[k] for k in ("ax", "ay", "az")], 1)
    B = np.stack([a64[k] for k in ("ax", "ay", "az")], 1)
    assert np.sqrt(((A - B) ** 2).sum() / (B ** 2).sum()) < 1e-5
    e = thm[:, 21:24].sum(1) + thm[:, 24]
    e64 = th[::10, 21:24].sum(1) + th[::10, 24]
    assert abs(e[-1] - e[0]) / s.n < 2e-3 and abs(e[-1] - e64[-1]) / s.n < 1e-3


def _binary(n=20000, seed=3):
    s = S.lj_binary_voids(n=n, density=1.2, frac_a=0.8, nvoids=2, void_r=3.0, seed=seed)
    return s


def test_lj_binary_mixture_mixed_vs_fp64_and_oracle(gpu, oracle):
    s = _binary()
    eps, sig, rc = S.kob_andersen_tables()
    st = s.state()
    oracle.run_minimize(st, s.masses, s.lo, s.hi, oracle.POT_LJ_MULTI,
                        oracle.multi_params(eps, sig, rc, float(rc.max())), 0.3, 0.02, 100.0, 30, 10)
    with gpu.Context(0) as ctx:
        ctx.upload_system(s)
        ctx.set_lj_multi(eps, sig, rc, 0.0)
        ctx.set_skin(0.3)
        # remove the worst overlaps first so FP32 forces stay finite
        ctx.set_precision(False)
        ctx.run_minimize(30, 0.02, tolF=100.0, rebuild_every=10)
        ctx.build_neighbors()
        d = ctx.download(("x", "y", "z"))
        ctx.compute_forces(energy=True)
        a64 = ctx.download(("ax", "ay", "az", "ep"))
        ctx.set_precision(True)
        ctx.compute_forces(energy=True)
        am = ctx.download(("ax", "ay", "az", "ep"))
    # minimiser trajectory: FP64 forces differ from the oracle's by summation
    # order only, the clipped push is the same arithmetic
    xo, yo, zo = st["x"].copy(), st["y"].copy(), st["z"].copy()
    oracle.wrap(xo, yo, zo, s.lo, s.hi)
    x, y, z = d["x"].copy(), d["y"].copy(), d["z"].copy()
    oracle.wrap(x, y, z, s.lo, s.hi)
    for a, b in ((x, xo), (y, yo), (z, zo)):
        dd = np.abs(a - b)
        dd = np.minimum(dd, s.L[0] - dd)
        assert dd.max() < 1e-8
    nl = oracle.build_neighbors(x, y, z, s.id, s.lo, s.hi, float(rc.max()) + 0.3)
    fx, fy, fz, ep, _ = oracle.lj_multi_force(x, y, z, s.type, nl, s.L, eps, sig, rc, float(rc.max()))
    F = np.stack([fx, fy, fz], 1) / s.masses[s.type][:, None]
    G64 = np.stack([a64[k] for k in ("ax", "ay", "az")], 1)
    Gm = np.stack([am[k] for k in ("ax", "ay", "az")], 1)
    assert np.sqrt(((G64 - F) ** 2).sum() / (F ** 2).sum()) < 1e-12
    assert np.sqrt(((Gm - F) ** 2).sum() / (F ** 2).sum()) < 1e-5
    assert abs(am["ep"].sum() - ep.sum()) < 1e-6 * abs(ep).sum()


def test_minimiser_push_matches_oracle(gpu, oracle):
    s = _binary(n=4000, seed=9)
    eps, sig, rc = S.kob_andersen_tables()
    with gpu.Context(0) as ctx:
        ctx.upload_system(s)
        ctx.set_lj_multi(eps, sig, rc, 0.0)
        ctx.set_skin(0.3)
        ctx.set_precision(False)
        ctx.compute_forces()
        d0 = ctx.download()
        ctx.push_min(0.002, 1.0, 50.0)
        d1 = ctx.download()
    st = {k: d0[k].copy() for k in d0}
    oracle.push_min(st["x"], st["y"], st["z"], st["ax"], st["ay"], st["az"], 0.002, 1.0, 50.0)
    for k in ("x", "y", "z", "ax"):
        assert np.array_equal(d1[k], st[k]), k
