"""The onika plugin's host logic (exastamp_gb300/onika/gb300_bridge.h) over a
fake exaNBody cell grid, through libgbmd on the GPU, against the FP64 oracle.

tests/onika_bridge/bridge_driver.cpp (compiled here with g++) puts a
Lennard-Jones system of two species into a grid of cells with a ghost
layer and runs the operators' calls:
  A  per-call forces (compute_force slot only), energies and virials on;
  B  new positions at the same particle layout (positions-only upload);
  C  move_particles-like reordering at constant count -- particles reversed
     inside each cell, every fifth moved to the next cell -- so the k-th
     gathered particle is another atom (the bridge must re-upload types
     and ids, or forces pair with stale species);
  D  the whole step on the device (push_f_v_r, push_f_v, check_and_update
     _particles, forces, push_f_v for 40 steps) and the state synced back.
Each phase's grid fields, matched by particle id, are checked against the
oracle: forces f = m a, per-atom energies and virials within 1e-12 (FP64
path), and the 40-step trajectory within 1e-10.
"""
import os
import shutil
import subprocess

import numpy as np
import pytest

from exastamp_gb300 import systems as S

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
NSTEPS = 40


@pytest.fixture(scope="module")
def driver(gbmd_lib, tmp_path_factory):
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("g++ not found")
    exe = str(tmp_path_factory.mktemp("bridge") / "bridge_driver")
    libdir = os.path.join(ROOT, "exastamp_gb300")
    subprocess.run([gxx, "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"), "-I",
                    os.path.join(ROOT, "exastamp_gb300", "onika"),
                    os.path.join(ROOT, "tests", "onika_bridge", "bridge_driver.cpp"), "-L", libdir, "-lgbmd",
                    "-Wl,-rpath," + libdir, "-o", exe], check=True)
    return exe


def _system():
    s = S.lj_fcc(ncell=6, seed=31)
    rng = np.random.default_rng(31)
    for a in (s.x, s.y, s.z):
        a += rng.normal(0.0, 0.04, s.n)
    s.type = (rng.random(s.n) < 0.3).astype(np.uint8)
    s.masses = np.array([1.0, 2.0])
    s.id = rng.permutation(s.n).astype(np.uint64) + 1000
    s.vx, s.vy, s.vz = (rng.normal(0.0, 0.5, s.n) / np.sqrt(s.masses[s.type]) for _ in range(3))
    return s


def _write_input(path, s, eps, sig, rcut, skin, dt, ncell):
    with open(path, "wb") as fh:
        np.array([s.n, len(s.masses), NSTEPS, ncell, ncell, ncell], np.int64).tofile(fh)
        np.concatenate([s.lo, s.hi, [eps, sig, rcut, skin, dt]]).astype(np.float64).tofile(fh)
        np.asarray(s.masses, np.float64).tofile(fh)
        for a in (s.x, s.y, s.z, s.vx, s.vy, s.vz):
            np.asarray(a, np.float64).tofile(fh)
        np.asarray(s.type, np.uint8).tofile(fh)
        np.asarray(s.id, np.uint64).tofile(fh)


def _read_phases(path, n):
    raw = open(path, "rb").read()
    out, off = [], 0
    for _ in range(4):
        cnt = np.frombuffer(raw, np.int64, 2, off)
        off += 16
        rec = np.frombuffer(raw, np.float64, 20 * n, off).reshape(n, 20)
        off += 160 * n
        ids = rec[:, 0].copy().view(np.uint64)
        order = np.argsort(ids)
        out.append({"counts": tuple(int(c) for c in cnt), "id": ids[order], "r": rec[order, 1:4],
                    "v": rec[order, 4:7], "f": rec[order, 7:10], "ep": rec[order, 10], "vir": rec[order, 11:20]})
    assert off == len(raw)
    return out


def _close(a, b, tol):
    return np.abs(a - b).max() <= tol * max(np.abs(b).max(), 1e-300)


def test_plugin_bridge_per_call_reorder_and_whole_step(driver, oracle, tmp_path):
    s = _system()
    eps, sig, rcut, skin, dt = 1.0, 1.0, 2.5, 0.3, 0.004
    inp, outp = str(tmp_path / "in.bin"), str(tmp_path / "out.bin")
    _write_input(inp, s, eps, sig, rcut, skin, dt, 3)
    subprocess.run([driver, inp, outp], check=True, timeout=300)
    ph = _read_phases(outp, s.n)
    order = np.argsort(s.id)
    types = s.type[order]
    ids = s.id[order]
    for k, p in enumerate(ph):
        assert np.array_equal(p["id"], ids), k
    # upload counters: A full, B positions only, C full again (new layout)
    assert ph[0]["counts"] == (1, 0)
    assert ph[1]["counts"] == (1, 1)
    assert ph[2]["counts"] == (2, 1)

    def oracle_forces(r):
        x, y, z = (np.ascontiguousarray(r[:, d]) for d in range(3))
        oracle.wrap(x, y, z, s.lo, s.hi)
        nl = oracle.build_neighbors(x, y, z, ids, s.lo, s.hi, rcut + skin)
        fx, fy, fz, ep, vir = oracle.lj_force(x, y, z, nl, s.L, eps, sig, rcut)
        return np.stack([fx, fy, fz], 1), ep, vir

    for k in range(3):
        F, ep, vir = oracle_forces(ph[k]["r"])
        assert _close(ph[k]["f"], F, 1e-12), k
        assert _close(ph[k]["ep"], ep, 1e-12), k
        assert _close(ph[k]["vir"], vir, 1e-12), k
    # D: the oracle's verlet_nve from C's state, rebuild on the skin/2 trigger
    st = {"x": ph[2]["r"][:, 0].copy(), "y": ph[2]["r"][:, 1].copy(), "z": ph[2]["r"][:, 2].copy(),
          "vx": ph[2]["v"][:, 0].copy(), "vy": ph[2]["v"][:, 1].copy(), "vz": ph[2]["v"][:, 2].copy(),
          "ax": np.zeros(s.n), "ay": np.zeros(s.n), "az": np.zeros(s.n), "ep": np.zeros(s.n),
          "type": np.ascontiguousarray(types), "id": np.ascontiguousarray(ids)}
    oracle.run_nve(st, s.masses, s.lo, s.hi, oracle.POT_LJ, oracle.LJParams(eps, sig, rcut), skin, dt, NSTEPS, -1,
                   thermo=False)
    d = ph[3]
    got = [np.ascontiguousarray(d["r"][:, q]) for q in range(3)]
    oracle.wrap(*got, s.lo, s.hi)
    ref = [st["x"].copy(), st["y"].copy(), st["z"].copy()]
    oracle.wrap(*ref, s.lo, s.hi)
    dr = np.stack(got, 1) - np.stack(ref, 1)
    dr -= np.round(dr / s.L) * s.L
    assert np.abs(dr).max() < 1e-10
    assert _close(d["v"], np.stack([st["vx"], st["vy"], st["vz"]], 1), 1e-10)
    # after sync the f fields hold accelerations (the grid after force_to_accel)
    assert _close(d["f"], np.stack([st["ax"], st["ay"], st["az"]], 1), 1e-10)
    assert _close(d["ep"], st["ep"], 1e-10)
    assert d["counts"][0] == 3  # one full upload when the whole-step mode took over


def test_plugin_bridge_diagonal_xform_and_rescale(driver, oracle, tmp_path):
    """A domain with the diagonal xform diag(1.05, 0.97, 1.02): the grid holds
    grid coordinates (physical / scale) and the bridge hands the library the
    physical ones.  Half-way through the whole-step phase the xform becomes
    diag(1.07, 0.96, 1.01) (a deformation step): the device state goes back
    into the grid with the old scale and comes back with the new one, the
    atoms moving with the box.  Forces, energies and virials of phases A-C
    within 1e-12 of the oracle on the physical coordinates; the trajectory
    across the rescale within 1e-10 of the oracle's, which continues from
    the accelerations of before the rescale as the device does."""
    s = _system()
    s1 = np.array([1.05, 0.97, 1.02])
    s2 = np.array([1.07, 0.96, 1.01])
    glo, ghi = s.lo / s1, s.hi / s1
    gx, gy, gz = s.x / s1[0], s.y / s1[1], s.z / s1[2]
    eps, sig, rcut, skin, dt = 1.0, 1.0, 2.5, 0.3, 0.004
    inp, outp = str(tmp_path / "in.bin"), str(tmp_path / "out.bin")
    with open(inp, "wb") as fh:
        np.array([s.n, len(s.masses), NSTEPS, 3, 3, 3], np.int64).tofile(fh)
        np.concatenate([glo, ghi, [eps, sig, rcut, skin, dt]]).astype(np.float64).tofile(fh)
        np.asarray(s.masses, np.float64).tofile(fh)
        for a in (gx, gy, gz, s.vx, s.vy, s.vz):
            np.asarray(a, np.float64).tofile(fh)
        np.asarray(s.type, np.uint8).tofile(fh)
        np.asarray(s.id, np.uint64).tofile(fh)
    subprocess.run([driver, inp, outp] + ["%.17g" % v for v in np.concatenate([s1, s2])], check=True, timeout=300)
    ph = _read_phases(outp, s.n)
    order = np.argsort(s.id)
    types, ids = s.type[order], s.id[order]
    lo1, hi1 = glo * s1, ghi * s1
    lo2, hi2 = glo * s2, ghi * s2

    for k in range(3):
        r = ph[k]["r"] * s1            # the physical coordinates the library saw
        x, y, z = (np.ascontiguousarray(r[:, d]) for d in range(3))
        oracle.wrap(x, y, z, lo1, hi1)
        nl = oracle.build_neighbors(x, y, z, ids, lo1, hi1, rcut + skin)
        fx, fy, fz, ep, vir = oracle.lj_force(x, y, z, nl, hi1 - lo1, eps, sig, rcut)
        assert _close(ph[k]["f"], np.stack([fx, fy, fz], 1), 1e-12), k
        assert _close(ph[k]["ep"], ep, 1e-12), k
        assert _close(ph[k]["vir"], vir, 1e-12), k
    # D: the first half with diag(s1), the second with diag(s2)
    r = ph[2]["r"] * s1
    st = {"x": r[:, 0].copy(), "y": r[:, 1].copy(), "z": r[:, 2].copy(),
          "vx": ph[2]["v"][:, 0].copy(), "vy": ph[2]["v"][:, 1].copy(), "vz": ph[2]["v"][:, 2].copy(),
          "ax": np.zeros(s.n), "ay": np.zeros(s.n), "az": np.zeros(s.n), "ep": np.zeros(s.n),
          "type": np.ascontiguousarray(types), "id": np.ascontiguousarray(ids)}
    pot = oracle.LJParams(eps, sig, rcut)
    half = NSTEPS // 2
    oracle.run_nve(st, s.masses, lo1, hi1, oracle.POT_LJ, pot, skin, dt, half, -1, thermo=False)
    for d, k in enumerate(("x", "y", "z")):
        st[k] = (st[k] / s1[d]) * s2[d]
    oracle.run_nve(st, s.masses, lo2, hi2, oracle.POT_LJ, pot, skin, dt, NSTEPS - half, -1, thermo=False,
                   initial_forces=False)
    d = ph[3]
    got = [np.ascontiguousarray(d["r"][:, q] * s2[q]) for q in range(3)]
    oracle.wrap(*got, lo2, hi2)
    ref = [st["x"].copy(), st["y"].copy(), st["z"].copy()]
    oracle.wrap(*ref, lo2, hi2)
    dr = np.stack(got, 1) - np.stack(ref, 1)
    dr -= np.round(dr / (hi2 - lo2)) * (hi2 - lo2)
    assert np.abs(dr).max() < 1e-10
    assert _close(d["v"], np.stack([st["vx"], st["vy"], st["vz"]], 1), 1e-10)
    assert _close(d["f"], np.stack([st["ax"], st["ay"], st["az"]], 1), 1e-10)
    assert d["counts"][0] == 4  # whole-step mode, then again after the rescale
