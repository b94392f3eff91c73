"""CPU checks of the FP64 oracle (no GPU): pair set against an all-image
brute force, list forces against a direct sum and finite differences, the
EAM spline known answers, push / thermo formulas, setfl round trip."""
import numpy as np
import pytest

from exastamp_gb300 import setfl as SF
from exastamp_gb300 import systems as S


def _jitter(s, sig, seed):
    rng = np.random.default_rng(seed)
    for a in (s.x, s.y, s.z):
        a += rng.normal(0.0, sig, s.n)
    return s


def _pairset(rows):
    return set(map(tuple, np.asarray(rows).tolist()))


@pytest.mark.parametrize("ncell,R,seed", [(3, 2.8, 0), (2, 2.8, 1), (4, 3.3, 2), (5, 2.8, 3)])
def test_pairs_match_brute_force(oracle, ncell, R, seed):
    s = _jitter(S.lj_fcc(ncell=ncell, seed=seed), 0.08, seed)
    assert oracle.wrap(s.x, s.y, s.z, s.lo, s.hi) == 0
    nl = oracle.build_neighbors(s.x, s.y, s.z, s.id, s.lo, s.hi, R)
    pi, pj, img = oracle.brute_pairs(s.x, s.y, s.z, s.lo, s.hi, R)
    brute = set(zip(pi.tolist(), pj.tolist(), *img.T.tolist()))
    assert _pairset(nl.pairs_with_ids(s.id)) == brute
    # no duplicates in the list
    assert nl.npairs == len(brute)


def test_pairs_random_gas_small_box(oracle):
    rng = np.random.default_rng(5)
    n, L = 60, 5.7
    x, y, z = (rng.uniform(0, L, n) for _ in range(3))
    lo, hi = np.zeros(3), np.full(3, L)
    R = 2.8   # nc = 2 per dimension: every stencil cell is reached twice with different images
    nl = oracle.build_neighbors(x, y, z, np.arange(n, dtype=np.uint64), lo, hi, R)
    pi, pj, img = oracle.brute_pairs(x, y, z, lo, hi, R)
    assert _pairset(nl.pairs_with_ids(np.arange(n))) == set(zip(pi.tolist(), pj.tolist(), *img.T.tolist()))
    # nc = 1: self images appear when L is just above R
    L1 = 3.0
    x1, y1, z1 = (rng.uniform(0, L1, 10) for _ in range(3))
    nl1 = oracle.build_neighbors(x1, y1, z1, np.arange(10, dtype=np.uint64), np.zeros(3), np.full(3, L1), 2.9)
    pi, pj, img = oracle.brute_pairs(x1, y1, z1, np.zeros(3), np.full(3, L1), 2.9)
    assert _pairset(nl1.pairs_with_ids(np.arange(10))) == set(zip(pi.tolist(), pj.tolist(), *img.T.tolist()))


def test_empty_and_single_atom(oracle):
    lo, hi = np.zeros(3), np.full(3, 10.0)
    e = np.zeros(0)
    nl = oracle.build_neighbors(e, e.copy(), e.copy(), np.zeros(0, np.uint64), lo, hi, 2.8)
    assert nl.npairs == 0
    one = np.array([5.0])
    nl = oracle.build_neighbors(one, one.copy(), one.copy(), np.zeros(1, np.uint64), lo, hi, 2.8)
    assert nl.npairs == 0


def test_lj_list_matches_direct_sum(oracle):
    s = _jitter(S.lj_fcc(ncell=4, seed=7), 0.05, 7)
    oracle.wrap(s.x, s.y, s.z, s.lo, s.hi)
    nl = oracle.build_neighbors(s.x, s.y, s.z, s.id, s.lo, s.hi, 2.8)
    fx, fy, fz, ep, vir = oracle.lj_force(s.x, s.y, s.z, nl, s.L, 1.0, 1.0, 2.5)
    e, dfx, dfy, dfz = oracle.lj_direct(s.x, s.y, s.z, s.lo, s.hi, 1.0, 1.0, 2.5)
    assert abs(ep.sum() - e) < 1e-10 * abs(e)
    assert np.abs(fx - dfx).max() < 1e-11 and np.abs(fz - dfz).max() < 1e-11
    # Newton's third law: the full list still sums to zero net force
    assert abs(fx.sum()) < 1e-9 and abs(fy.sum()) < 1e-9
    # virial trace = -1/2 sum r.f over pairs (per-atom halves)
    assert vir.shape == (s.n, 9)


def test_lj_forces_are_energy_gradient(oracle):
    s = _jitter(S.lj_fcc(ncell=3, seed=9), 0.06, 9)
    oracle.wrap(s.x, s.y, s.z, s.lo, s.hi)
    prm = (1.0, 1.0, 2.5)
    _, fx, fy, fz = oracle.lj_direct(s.x, s.y, s.z, s.lo, s.hi, *prm)
    h = 1e-6
    for i in (0, 17, 55):
        xp, xm = s.x.copy(), s.x.copy()
        xp[i] += h
        xm[i] -= h
        ep = oracle.lj_direct(xp, s.y, s.z, s.lo, s.hi, *prm)[0]
        em = oracle.lj_direct(xm, s.y, s.z, s.lo, s.hi, *prm)[0]
        fd = -(ep - em) / (2 * h)
        assert abs(fd - fx[i]) < 2e-6 * max(1.0, abs(fx[i]))


def test_lj_pair_known_values(oracle):
    # e(2^(1/6) sigma) = -eps, de = 0 at the minimum; e(sigma) = 0
    e, de = oracle.lj_pair(1.0, 1.0, 2 ** (1 / 6))
    assert abs(e + 1.0) < 1e-15 and abs(de) < 1e-13
    e, de = oracle.lj_pair(2.0, 1.5, 1.5)
    assert abs(e) < 1e-15 and abs(de + 24 * 2.0 / 1.5) < 1e-12
    assert abs(oracle.lj_energy_cut(1.0, 1.0, 2.5) - (-0.016316891136)) < 1e-11


def test_lj_multi_reduces_to_single(oracle):
    s = _jitter(S.lj_fcc(ncell=3, seed=4), 0.05, 4)
    oracle.wrap(s.x, s.y, s.z, s.lo, s.hi)
    types = np.zeros(s.n, np.uint8)
    types[::3] = 1
    nl = oracle.build_neighbors(s.x, s.y, s.z, s.id, s.lo, s.hi, 2.8)
    one = oracle.lj_force(s.x, s.y, s.z, nl, s.L, 1.0, 1.0, 2.5)
    eps, sig, rc = np.ones((2, 2)), np.ones((2, 2)), np.full((2, 2), 2.5)
    multi = oracle.lj_multi_force(s.x, s.y, s.z, types, nl, s.L, eps, sig, rc, 2.5)
    for a, b in zip(one[:4], multi[:4]):
        assert np.array_equal(a, b)


def test_eam_spline_reproduces_cubics(oracle):
    # The 4th-order derivative estimate and Hermite cubic are exact for cubics
    # away from the two end knots on each side.
    n, d = 50, 0.1
    x = np.arange(n) * d
    f = 0.3 * x ** 3 - 2 * x ** 2 + x - 4
    sp = oracle.eam_spline(np.concatenate([[0.0], f]), d)
    for m in range(3, n - 3):
        c = sp[m]
        for p in (0.0, 0.25, 0.7):
            xx = (m - 1 + p) * d
            val = ((c[3] * p + c[4]) * p + c[5]) * p + c[6]
            der = (c[0] * p + c[1]) * p + c[2]
            assert abs(val - (0.3 * xx ** 3 - 2 * xx ** 2 + xx - 4)) < 1e-11
            assert abs(der - (0.9 * xx ** 2 - 4 * xx + 1)) < 1e-9


def _cu_tables(oracle, rcut=5.0):
    cfg = SF.load_cu_params()
    sf = SF.tabulate(cfg)
    return sf, oracle.EamOracleTables.from_setfl(sf, S.EV, S.EV, rcut=rcut)


def test_eam_lookups_match_analytic(oracle):
    cfg = SF.load_cu_params()
    sf, tab = _cu_tables(oracle)
    f, phi, F = SF.analytic_functions(cfg["params"], cfg["rho_e"])
    for r in (2.3, 2.556, 3.1, 4.4, 4.99):
        assert abs(oracle.eam_rho(tab, r) - f(r)) < 1e-9 * f(r)
    for rho in (5.0, 13.37, 20.0):
        e, fp = oracle.eam_embed_one(tab, rho)
        assert abs(e / S.EV - F(rho)) < 1e-8
    # above rhomax F is extended linearly with the end slope
    rhomax = (sf.nrho - 1) * sf.drho
    e1, fp1 = oracle.eam_embed_one(tab, rhomax)
    e2, fp2 = oracle.eam_embed_one(tab, rhomax + 1.0)
    assert abs((e2 - e1) - fp1) < 1e-6 * abs(fp1)


def test_eam_forces_are_energy_gradient(oracle):
    sf, tab = _cu_tables(oracle)
    s = S.eam_cu_fcc(ncell=3, displace=0.08, seed=3)
    nl = oracle.build_neighbors(s.x, s.y, s.z, s.id, s.lo, s.hi, 5.3)
    fx, fy, fz, ep, vir, _, _ = oracle.eam_forces(s.x, s.y, s.z, s.type, nl, s.L, tab, 5.0)
    h = 1e-5
    for i in (0, 31, 77):
        vals = []
        for sgn in (1, -1):
            x = s.x.copy()
            x[i] += sgn * h
            nl2 = oracle.build_neighbors(x, s.y, s.z, s.id, s.lo, s.hi, 5.3)
            vals.append(oracle.eam_forces(x, s.y, s.z, s.type, nl2, s.L, tab, 5.0)[3].sum())
        fd = -(vals[0] - vals[1]) / (2 * h)
        assert abs(fd - fx[i]) < 1e-6 * max(abs(fx[i]), 1e3)
    assert abs(fx.sum()) < 1e-7 * np.abs(fx).max() * s.n


def test_push_and_accel_formulas(oracle):
    rng = np.random.default_rng(1)
    n = 100
    arr = {k: rng.normal(size=n) for k in ("x", "y", "z", "vx", "vy", "vz", "ax", "ay", "az")}
    ref = {k: v.copy() for k, v in arr.items()}
    oracle.push_f_v_r(arr["x"], arr["y"], arr["z"], arr["vx"], arr["vy"], arr["vz"], arr["ax"], arr["ay"],
                      arr["az"], 0.01, 1.0)
    assert np.array_equal(arr["x"], ref["x"] + (ref["vx"] * 0.01 + ref["ax"] * (0.01 * 0.01 * 0.5)))
    oracle.push_f_v(arr["vx"], arr["vy"], arr["vz"], arr["ax"], arr["ay"], arr["az"], 0.01, 0.5)
    assert np.array_equal(arr["vx"], ref["vx"] + ref["ax"] * (0.01 * 0.5))
    f = rng.normal(size=(3, n))
    t = (np.arange(n) % 2).astype(np.uint8)
    m = np.array([2.0, 3.0])
    g = f.copy()
    oracle.force_to_accel(g[0], g[1], g[2], t, m)
    assert np.array_equal(g, f / m[t])
    x, ax = np.zeros(3), np.array([5.0, -0.5, 0.1])
    oracle.push_min(x, x.copy(), x.copy(), ax, ax.copy(), ax.copy(), 0.1, 1.0, tolF=1.0)
    assert np.allclose(x, np.array([1.0, -0.5, 0.1]) * 0.005)


def test_thermo_layout(oracle):
    rng = np.random.default_rng(2)
    n = 5000
    v = rng.normal(size=(3, n))
    ep = rng.normal(size=n)
    vir = rng.normal(size=(n, 9))
    t = (np.arange(n) % 2).astype(np.uint8)
    m = np.array([1.5, 2.5])
    out = oracle.thermo(v[0], v[1], v[2], ep, vir, t, m)
    mm = m[t]
    assert np.allclose(out[0:9], vir.sum(0))
    assert np.allclose(out[9:18].reshape(3, 3), 0.5 * np.einsum("i,ai,bi->ab", mm, v, v))
    assert np.allclose(out[18:21], (v * mm).sum(1))
    assert np.allclose(out[21:24], 0.5 * (v * v * mm).sum(1))
    assert np.isclose(out[24], ep.sum()) and np.isclose(out[25], mm.sum()) and out[26] == n


def test_setfl_round_trip(tmp_path):
    sf = SF.tabulate(SF.load_cu_params())
    p = tmp_path / "cu.eam.alloy"
    SF.write_setfl(sf, str(p))
    sf2 = SF.read_setfl(str(p))
    assert sf2.nrho == sf.nrho and sf2.nr == sf.nr and sf2.elements == ["Cu"]
    assert np.array_equal(sf2.frho[0], sf.frho[0]) and np.array_equal(sf2.z2r[0], sf.z2r[0])
    assert sf2.dr == sf.dr and sf2.rcut == sf.rcut


def test_param_jacobian_matches_finite_differences():
    cfg = SF.load_cu_params()
    J_F, J_f, J_z = SF.table_param_jacobian(cfg)
    base = SF.tabulate(cfg)
    for k, name in enumerate(SF.PARAM_NAMES):
        h = 1e-6 * max(1.0, abs(cfg["params"][name]))
        up = SF.tabulate(cfg, {name: cfg["params"][name] + h})
        dn = SF.tabulate(cfg, {name: cfg["params"][name] - h})
        for J, attr in ((J_F, "frho"), (J_f, "rhor"), (J_z, "z2r")):
            fd = (getattr(up, attr)[0] - getattr(dn, attr)[0]) / (2 * h)
            assert np.allclose(J[k], fd, rtol=1e-5, atol=1e-7 * (1 + np.abs(getattr(base, attr)[0]).max()))


def test_oracle_nve_conserves_energy(oracle):
    s = S.lj_fcc(ncell=4, seed=1)
    st = s.state()
    th = oracle.run_nve(st, s.masses, s.lo, s.hi, oracle.POT_LJ, oracle.LJParams(1.0, 1.0, 2.5), 0.3, 0.005, 200, 10)
    etot = th[:, 21:24].sum(1) + th[:, 24]
    drift = abs(etot[-1] - etot[0]) / s.n
    assert drift < 2e-3
    assert np.allclose(th[:, 18:21], 0.0, atol=1e-9)


def test_oracle_nve_continues_from_given_accelerations(oracle):
    """20 steps in one call equal 10 steps, then 10 more that start from the
    accelerations the first call left (orc_run_nve_from), bit for bit: the
    list is rebuilt from the same positions at step 10 in both."""
    s = S.lj_fcc(ncell=4, seed=2)
    pot = oracle.LJParams(1.0, 1.0, 2.5)
    one = s.state()
    oracle.run_nve(one, s.masses, s.lo, s.hi, oracle.POT_LJ, pot, 0.3, 0.005, 20, 10, thermo=False)
    two = s.state()
    oracle.run_nve(two, s.masses, s.lo, s.hi, oracle.POT_LJ, pot, 0.3, 0.005, 10, 10, thermo=False)
    oracle.run_nve(two, s.masses, s.lo, s.hi, oracle.POT_LJ, pot, 0.3, 0.005, 10, 10, thermo=False,
                   initial_forces=False)
    for k in ("x", "y", "z", "vx", "vy", "vz", "ax", "ay", "az"):
        assert np.array_equal(one[k], two[k]), k


def test_two_level_filter_is_complete(oracle):
    """The claim behind the two-level list (gbmd_set_list_buffer): filter an
    outer list of radius R + d, built at positions x0, by the distance at
    positions x1 that moved less than d/2, and the result is the pair set
    of a fresh radius-R build at x1.  Checked with the oracle's own builder
    (FP64) on a jittered LJ crystal: displacements uniform in a ball of
    radius 0.999 d/2, separations taken with the outer build's images."""
    s = _jitter_cpu(S.lj_fcc(ncell=7, seed=5), 0.04, 5)
    R, d = 2.8, 0.6
    x0, y0, z0 = s.x.copy(), s.y.copy(), s.z.copy()
    oracle.wrap(x0, y0, z0, s.lo, s.hi)
    outer = oracle.build_neighbors(x0, y0, z0, s.id, s.lo, s.hi, R + d)
    n = s.n
    ii = np.repeat(np.arange(n), np.diff(outer.off))
    jj = outer.nbr

    def filtered_and_fresh(reach, seed):
        rng = np.random.default_rng(seed)
        u = rng.normal(size=(n, 3))
        u *= (reach * rng.random(n) ** (1 / 3) / np.linalg.norm(u, axis=1))[:, None]
        x1, y1, z1 = x0 + u[:, 0], y0 + u[:, 1], z0 + u[:, 2]
        sep = np.stack([x1[jj] + outer.img[:, 0] * s.L[0] - x1[ii], y1[jj] + outer.img[:, 1] * s.L[1] - y1[ii],
                        z1[jj] + outer.img[:, 2] * s.L[2] - z1[ii]], 1)
        keep = ((sep[:, 0] * sep[:, 0] + sep[:, 1] * sep[:, 1]) + sep[:, 2] * sep[:, 2]) <= R * R
        xw, yw, zw = x1.copy(), y1.copy(), z1.copy()
        oracle.wrap(xw, yw, zw, s.lo, s.hi)
        fresh = oracle.build_neighbors(xw, yw, zw, s.id, s.lo, s.hi, R)
        fi = np.repeat(np.arange(n), np.diff(fresh.off))
        return set(zip(ii[keep].tolist(), jj[keep].tolist())), set(zip(fi.tolist(), fresh.nbr.tolist()))

    filtered, fresh = filtered_and_fresh(0.999 * 0.5 * d, 6)
    assert filtered == fresh
    assert 0 < len(filtered) < outer.npairs
    # moved farther than d/2 the filter misses pairs (the check is not vacuous)
    filtered, fresh = filtered_and_fresh(1.5 * d, 7)
    assert filtered < fresh


def _jitter_cpu(s, sig, seed):
    rng = np.random.default_rng(seed)
    for a in (s.x, s.y, s.z):
        a += rng.normal(0.0, sig, s.n)
    return s


def test_oracle_minimiser_lowers_energy_and_clips(oracle):
    """Clipped minimiser on an overlapping random binary mixture: the
    potential energy falls and no step moves an atom further than
    tolF*dt^2/2 per component."""
    s = S.lj_binary_voids(n=3000, density=1.2, frac_a=0.8, nvoids=1, void_r=2.0, seed=11)
    eps, sig, rc = S.kob_andersen_tables()
    prm = oracle.multi_params(eps, sig, rc, float(rc.max()))
    st = s.state()

    def epot(st):
        x, y, z = st["x"].copy(), st["y"].copy(), st["z"].copy()
        oracle.wrap(x, y, z, s.lo, s.hi)
        nl = oracle.build_neighbors(x, y, z, s.id, s.lo, s.hi, float(rc.max()) + 0.3)
        return oracle.lj_multi_force(x, y, z, s.type, nl, s.L, eps, sig, rc, float(rc.max()))[3].sum()

    e0 = epot(st)
    x0 = st["x"].copy()
    oracle.run_minimize(st, s.masses, s.lo, s.hi, oracle.POT_LJ_MULTI, prm, 0.3, 0.002, 1e3, 1, 0)
    step = np.abs(st["x"] - x0).max()
    assert step <= 1e3 * 0.002 ** 2 / 2 * (1 + 1e-12)
    oracle.run_minimize(st, s.masses, s.lo, s.hi, oracle.POT_LJ_MULTI, prm, 0.3, 0.002, 1e3, 40, 10)
    assert epot(st) < 0.5 * e0


def test_oracle_displacement_trigger(oracle):
    """Rebuilding on the skin/2 displacement trigger gives the trajectory of
    rebuilding every step (lists differ only by pairs beyond the cutoff),
    with far fewer builds."""
    s = S.lj_fcc(ncell=6, density=0.8442, T=1.5, seed=5)
    prm = oracle.LJParams(1.0, 1.0, 2.5)
    st1, st2 = s.state(), s.state()
    th1 = oracle.run_nve(st1, s.masses, s.lo, s.hi, oracle.POT_LJ, prm, 0.3, 0.005, 150, 1)
    n1 = oracle.last_list_builds()
    th2 = oracle.run_nve(st2, s.masses, s.lo, s.hi, oracle.POT_LJ, prm, 0.3, 0.005, 150, -1)
    n2 = oracle.last_list_builds()
    assert n1 == 151 and 2 < n2 < 40
    assert np.allclose(th1, th2, rtol=1e-9, atol=1e-9 * np.abs(th1).max())


def _ej(oracle):
    return oracle.Johnson(S.johnson_ta_params(), 6.1)


def test_johnson_functions_derivatives(oracle):
    """eam_johnson_phi / rho / fEmbed: the returned derivatives match central
    differences, the embedding in all three density branches."""
    pot = _ej(oracle)
    h = 1e-6
    for name, args in (("phi", [2.4, 2.86, 3.3, 4.1, 5.5]), ("rho", [2.4, 2.86, 3.3, 4.1, 5.5])):
        for r in args:
            v, dv = oracle.ej_function(name, pot, r)
            fd = (oracle.ej_function(name, pot, r + h)[0] - oracle.ej_function(name, pot, r - h)[0]) / (2 * h)
            assert abs(dv - fd) <= 1e-6 * max(1.0, abs(dv)), (name, r, dv, fd)
    rhoe = S.johnson_ta_params()[2]
    for frac in (0.5, 0.84, 1.0, 1.1, 1.3, 1.6):
        rho = frac * rhoe
        v, dv = oracle.ej_function("embed", pot, rho)
        hh = 1e-6 * rhoe
        fd = (oracle.ej_function("embed", pot, rho + hh)[0] - oracle.ej_function("embed", pot, rho - hh)[0]) / (2 * hh)
        assert abs(dv - fd) <= 1e-6 * max(1.0, abs(dv)), (frac, dv, fd)


def test_johnson_forces_are_energy_gradient(oracle):
    s = S.ta_bcc(ncell=4, noise=0.08, seed=3)
    pot = _ej(oracle)

    def energy_forces(x, y, z):
        x, y, z = x.copy(), y.copy(), z.copy()
        oracle.wrap(x, y, z, s.lo, s.hi)
        nl = oracle.build_neighbors(x, y, z, s.id, s.lo, s.hi, 7.1)
        fx, fy, fz, ep, _, _ = oracle.ej_forces(x, y, z, nl, s.L, pot)
        return ep.sum(), np.stack([fx, fy, fz], 1)

    E0, F = energy_forces(s.x, s.y, s.z)
    h = 1e-5
    for i in (0, 17, 63):
        for d, arr in enumerate((s.x, s.y, s.z)):
            p, m = arr.copy(), arr.copy()
            p[i] += h
            m[i] -= h
            args_p = [p if q == d else (s.x, s.y, s.z)[q] for q in range(3)]
            args_m = [m if q == d else (s.x, s.y, s.z)[q] for q in range(3)]
            fd = -(energy_forces(*args_p)[0] - energy_forces(*args_m)[0]) / (2 * h)
            assert abs(fd - F[i, d]) < 1e-6 * np.abs(F).max(), (i, d, fd, F[i, d])


def test_lj_loss_gradient_matches_finite_differences(oracle):
    """d(loss)/d(epsilon, sigma) of the force-matching + energy loss against
    central differences of the oracle's own loss (relative 1e-6)."""
    s = S.lj_fcc(ncell=4, density=0.8442, T=1.0, seed=9)
    rng = np.random.default_rng(9)
    x, y, z = (a + rng.normal(0.0, 0.05, s.n) for a in (s.x, s.y, s.z))
    oracle.wrap(x, y, z, s.lo, s.hi)
    nl = oracle.build_neighbors(x, y, z, s.id, s.lo, s.hi, 2.8)
    fx, fy, fz, ep, _ = oracle.lj_force(x, y, z, nl, s.L, 1.1, 0.97, 2.5)
    ft, et = np.stack([fx, fy, fz], 1), ep
    wF, wE = 1.0 / s.n, 0.1 / s.n
    loss, g = oracle.lj_loss_grad(x, y, z, nl, s.L, 1.0, 1.0, 2.5, ft, et, wF, wE)
    assert loss > 0
    h = 1e-6
    for k in range(2):
        p, m = [1.0, 1.0], [1.0, 1.0]
        p[k] += h
        m[k] -= h
        fd = (oracle.lj_loss_grad(x, y, z, nl, s.L, p[0], p[1], 2.5, ft, et, wF, wE)[0]
              - oracle.lj_loss_grad(x, y, z, nl, s.L, m[0], m[1], 2.5, ft, et, wF, wE)[0]) / (2 * h)
        assert abs(fd - g[k]) < 1e-6 * max(abs(fd), 1e-12), (k, fd, g[k])


def test_build_neighbors_first_matches_full_list(oracle):
    """The lists of the first m atoms (neighbours among all) are the full
    build's lists of those atoms, and the LJ-mixture forces of those atoms
    from them are the full evaluation's."""
    from exastamp_gb300 import systems as S
    s = S.lj_binary_voids(n=4000, seed=9, nvoids=1, void_r=2.0)
    eps, sig, rc = S.kob_andersen_tables()
    rcmax = float(rc.max())
    x, y, z = s.x.copy(), s.y.copy(), s.z.copy()
    oracle.wrap(x, y, z, s.lo, s.hi)
    full = oracle.build_neighbors(x, y, z, s.id, s.lo, s.hi, rcmax + 0.3)
    m = 700
    part = oracle.build_neighbors_first(x, y, z, s.id, s.lo, s.hi, rcmax + 0.3, m)
    assert np.array_equal(part.off, full.off[: m + 1])
    assert np.array_equal(part.nbr, full.nbr[: full.off[m]])
    assert np.array_equal(part.img, full.img[: full.off[m]])
    ff = oracle.lj_multi_force(x, y, z, s.type, full, s.L, eps, sig, rc, rcmax)
    fp = oracle.lj_multi_force(x, y, z, s.type, part, s.L, eps, sig, rc, rcmax)
    for a, b in zip(ff[:4], fp[:4]):
        assert np.array_equal(a[:m], b)
