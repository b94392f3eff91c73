#!/usr/bin/env python
"""Throughput of the GB300 MD hot path in atom-timesteps/s.

Default workload (one GPU): the copper-like eam_alloy FCC crystal of
100x100x100 unit cells (4,000,000 atoms, a = 3.615 A, 5,000-point splines,
rcut 5.0 A, skin 0.3 A, 300 K, dt = 1 fs), NVE velocity Verlet with a
neighbour rebuild every 10 steps, mixed precision (FP32 pair arithmetic,
FP64 state).  One step = first half push + (rebuild) + density/embedding +
force + second half push, for all atoms.

Reported (one JSON line on rank 0):
  value      device-resident throughput (state in HBM, K steps timed with
             CUDA events on the library's stream, CUDA graph of 2 rebuild
             intervals, thermo every 20 steps)
  e2e        the same step through the C ABI with the grid state on the
             host: gbmd_run_nve_host per step (r,v,a copied in from pinned
             memory, one verlet_nve step, r copied out while the force pass
             runs, then v,a)
  roofline   the final pair kernel (force + fused Verlet halves), algorithmic
             bytes per launch / its CUDA-event duration, against the measured
             HBM copy bandwidth
  fp64       the same steps through the plain-FP64 kernels, and the
             mixed-vs-FP64 force error and energy drift
  cpu_baseline  the FP64 OpenMP oracle on a bounded sample, all host threads

--impl reference times the reference's CPU path of this workload on the
host cores: the reference cannot be built here (it needs onika, exaNBody,
yaml-cpp and MPI), so it is the project's FP64 OpenMP restatement of the
reference operators (oracle/), on a sample sized to finish in minutes.
Multi-GPU (torchrun): independent replicas, one per rank, weak scaling.
"""
from __future__ import annotations

import argparse
import atexit
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
# minimiser that precedes the mixture's NVE run (reduced units): step 0.02
# and acceleration clip 100, so an atom moves at most 100*0.02^2/2 = 0.02
# sigma per component per step (the NVE step 0.002 would move overlapping
# atoms only 2e-4 sigma per step and leave forces that blow the NVE run up)
MIN_TOLF = 100.0
# measured DRAM traffic of the force kernel per atom (see roofline.traffic)
EAM_FORCE_DRAM_BYTES_PER_ATOM = (273.772288e6 + 51.000832e6) / 864000.0
# the same for k_lj_mixed on the 864,000-atom LJ mixture (lj_binary_16m --ncell 60)
LJ_MULTI_PAIR_DRAM_BYTES_PER_ATOM = (474.028544e6 + 51.887872e6) / 864000.0
MIN_DT = 0.02
sys.path.insert(0, ROOT)

WORKLOADS = {
    "eam_cu_4m": dict(kind="eam", ncell=100, a=3.615, T=300.0, seed=2, rcut=5.0, skin=0.3, dt=1e-3,
                      desc="eam_alloy Cu-like FCC 100^3 cells (4,000,000 atoms), 5000-point splines, "
                           "rcut 5.0 A, skin 0.3 A, 300 K, dt 1 fs, NVE, rebuild every 10"),
    "lj_fcc_32k": dict(kind="lj", ncell=20, T=1.0, seed=1, rcut=2.5, skin=0.3, dt=0.005,
                       desc="LJ FCC 20^3 cells (32,000 atoms), rho*=0.8442, rc 2.5, skin 0.3, T*=1, "
                            "dt 0.005, NVE, rebuild every 10"),
    "lj_binary_16m": dict(kind="lj_multi", n=16_777_216, seed=3, rcut=2.5, skin=0.3, dt=0.002, min_steps=200,
                          min_fp64_steps=20,
                          desc="LJ A:B 80:20 binary mixture, 16,777,216 atoms, rho 1.2, 64 voids of radius 8 sigma, "
                               "per-pair cutoff 2.5 sigma_ab, skin 0.3, 200 clipped minimiser steps (step 0.02, "
                               "clip 100; the first 20 in FP64, the rest mixed) then NVE dt 0.002, rebuild every 10"),
}


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=1000)
    p.add_argument("--warmup", type=int, default=20)
    p.add_argument("--impl", default="gbmd", choices=["gbmd", "reference"])
    p.add_argument("--workload", default="eam_cu_4m", choices=sorted(WORKLOADS))
    p.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    p.add_argument("--rebuild-every", type=int, default=10,
                   help="list rebuild interval in steps; -1 rebuilds on the skin/2 displacement trigger")
    p.add_argument("--list-buffer", type=float, default=-1.0,
                   help="two-level neighbour list: outer buffer beyond rcut + skin (0, the default: off)")
    p.add_argument("--no-two-level", action="store_true",
                   help="skip the 200-step comparison of the one- and two-level lists (EAM workload)")
    p.add_argument("--e2e-steps", type=int, default=20)
    p.add_argument("--fp64-steps", type=int, default=40)
    p.add_argument("--no-cpu", action="store_true")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-fp64", action="store_true")
    p.add_argument("--no-batch", action="store_true", help="skip the batched-replica and adjoint sections")
    p.add_argument("--lanes", type=int, default=0, help="lanes per atom (0: autotune)")
    p.add_argument("--block", type=int, default=0)
    p.add_argument("--vec", type=int, default=1, help="list entries per lane per load with --lanes (1 or 4)")
    p.add_argument("--staging", action="store_true",
                   help="with --lanes 1 --vec 4: stage neighbour positions in shared memory")
    p.add_argument("--newton3", action="store_true",
                   help="LJ workloads with --lanes 1 --vec 4: half list + scattered reaction forces")
    p.add_argument("--ref-seconds", type=float, default=150.0,
                   help="--impl reference: CPU seconds the warm-up + timed steps of the sample should take")
    p.add_argument("--thermalise", type=int, default=100,
                   help="untimed NVE steps from the lattice before the launch shape is tuned (lattice workloads)")
    p.add_argument("--ncell", type=int, default=0,
                   help="override the unit cells per edge (small profiling cases of the same workload)")
    p.add_argument("--no-mixture", action="store_true",
                   help="skip the 16.7 M-atom LJ mixture section of the default run")
    p.add_argument("--no-lj-crystal", action="store_true",
                   help="skip the 32,000-atom LJ crystal section of the default run")
    p.add_argument("--no-drift", action="store_true",
                   help="skip the 1,000-step mixed / 200-step FP64 NVE drift section")
    p.add_argument("--no-oracle-check", action="store_true",
                   help="skip the force error against the FP64 oracle at the benchmarked state")
    a = p.parse_args()
    if a.list_buffer >= 0.0:
        WORKLOADS[a.workload] = dict(WORKLOADS[a.workload], list_buffer=a.list_buffer)
    if a.ncell:
        extra = {"n": 4 * a.ncell ** 3} if WORKLOADS[a.workload]["kind"] == "lj_multi" else {}
        WORKLOADS[a.workload] = dict(WORKLOADS[a.workload], ncell=a.ncell, **extra)
    return a


# ---------------------------------------------------------------------------
def make_system(w):
    """The workload's atoms, stored as the reference's grid holds them (cell
    by cell, z slowest): the caller order of the e2e host arrays."""
    from exastamp_gb300 import systems as S
    if w["kind"] == "eam":
        s = S.eam_cu_fcc(ncell=w["ncell"], a=w["a"], T=w["T"], seed=w["seed"])
    elif w["kind"] == "lj_multi":
        s = S.lj_binary_voids(n=w["n"], seed=w["seed"], nvoids=max(1, round(64 * w["n"] / 16_777_216)))
    else:
        s = S.lj_fcc(ncell=w["ncell"], T=w["T"], seed=w["seed"])
    return S.grid_order(s, w["rcut"] + w["skin"])


def bind_potential(ctx, w):
    from exastamp_gb300 import setfl, systems as S
    if w["kind"] == "eam":
        sf = setfl.tabulate(setfl.load_cu_params())
        ctx.set_eam_alloy(sf, w["rcut"], S.EV, S.EV)
    elif w["kind"] == "lj_multi":
        eps, sig, rc = S.kob_andersen_tables()
        ctx.set_lj_multi(eps, sig, rc, 0.0)
    else:
        ctx.set_lj(1.0, 1.0, w["rcut"])
    ctx.set_skin(w["skin"])
    ctx.set_list_buffer(w.get("list_buffer", 0.0))


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.path = None

    def __enter__(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
            # the sampler never outlives the bench, also when it fails
            atexit.register(self.__exit__)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc and self.proc.poll() is None:
            self.proc.terminate()
            try:
                self.proc.wait(5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.path or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        rows = []
        for ln in open(self.path):
            f = [x.strip() for x in ln.split(",")]
            if len(f) >= 9:
                rows.append(f)
        os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "samples": len(rows), "reasons": reasons}


def measured_clock_mhz():
    """Maximum SM clock recorded with the measured peaks, if any."""
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            return float(json.load(fh).get("sm_max_mhz") or 0.0) or None
    except (OSError, ValueError):
        return None


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def dist_setup(args):
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch
        import torch.distributed as dist
        if torch.cuda.is_available():
            torch.cuda.set_device(local)
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    return ws, rank, local


def dist_max(x, ws):
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device="cuda" if torch.cuda.is_available() else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


# ---------------------------------------------------------------------------
def oracle_sample(w, O, nc):
    """A CPU-sized sample of workload `w` (nc FCC cells per edge, or 4 nc^3
    atoms for the mixture, which is first put through the same clipped
    minimiser as the GPU run) with the oracle's potential parameters."""
    from exastamp_gb300 import setfl, systems as S
    if w["kind"] == "eam":
        tab = O.EamOracleTables.from_setfl(setfl.tabulate(setfl.load_cu_params()), S.EV, S.EV, rcut=w["rcut"])
        s = S.eam_cu_fcc(ncell=nc, a=w["a"], T=w["T"], seed=w["seed"])
        return s, s.state(), O.POT_EAM, tab
    if w["kind"] == "lj_multi":
        eps, sig, rc = S.kob_andersen_tables()
        pot = O.multi_params(eps, sig, rc, float(rc.max()))
        n = 4 * nc ** 3
        s = S.lj_binary_voids(n=n, seed=w["seed"], nvoids=max(1, round(64 * n / w["n"])))
        st = s.state()
        O.run_minimize(st, s.masses, s.lo, s.hi, O.POT_LJ_MULTI, pot, w["skin"], MIN_DT, MIN_TOLF,
                       w["min_steps"], 10)
        return s, st, O.POT_LJ_MULTI, pot
    s = S.lj_fcc(ncell=nc, T=w["T"], seed=w["seed"])
    return s, s.state(), O.POT_LJ, O.LJParams(1.0, 1.0, w["rcut"])


def _oracle():
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    O.build()
    return O


def cpu_oracle_rate(w, target_s=15.0, ncell=None):
    """FP64 OpenMP oracle NVE throughput on a sample of the workload."""
    O = _oracle()
    nc = ncell or min(w.get("ncell", 20), 24 if w["kind"] == "eam" else 20)
    s, st0, pot_kind, pot = oracle_sample(w, O, nc)
    st = {k: v.copy() for k, v in st0.items()}
    t0 = time.perf_counter()
    O.run_nve(st, s.masses, s.lo, s.hi, pot_kind, pot, w["skin"], w["dt"], 2, 10, thermo=False)
    t_cal = (time.perf_counter() - t0) / 3.0
    steps = int(max(3, min(5000, target_s / max(t_cal, 1e-6))))
    st = {k: v.copy() for k, v in st0.items()}
    t0 = time.perf_counter()
    O.run_nve(st, s.masses, s.lo, s.hi, pot_kind, pot, w["skin"], w["dt"], steps, 10, thermo=False)
    dt = time.perf_counter() - t0
    return s.n * steps / dt, {"atoms": s.n, "steps": steps, "seconds": dt, "threads": O.num_threads(),
                              "ncell": nc}


def run_reference(args, w, ws, rank):
    """--impl reference: the FP64 OpenMP restatement of the reference
    operators (the reference itself does not build here), all host threads,
    each step one NVE step of a sample sized so W+K steps fit in minutes."""
    if rank != 0:
        return
    O = _oracle()
    # size the sample: --ref-seconds (150 s) for warmup + steps at the calibrated rate
    rate, _ = cpu_oracle_rate(w, target_s=min(3.0, args.ref_seconds), ncell=8 if w["kind"] == "eam" else 10)
    budget = args.ref_seconds
    atoms = rate * budget / max(1, args.steps + args.warmup)
    per = 4
    nc = int(max(4, min(w.get("ncell", 64), round((atoms / per) ** (1.0 / 3.0)))))
    s, st, pot_kind, pot = oracle_sample(w, O, nc)
    O.run_nve(st, s.masses, s.lo, s.hi, pot_kind, pot, w["skin"], w["dt"], args.warmup, args.rebuild_every,
              thermo=False)
    t0 = time.perf_counter()
    O.run_nve(st, s.masses, s.lo, s.hi, pot_kind, pot, w["skin"], w["dt"], args.steps, args.rebuild_every,
              thermo=False)
    sec = time.perf_counter() - t0
    value = s.n * args.steps / sec
    sample = "%d-atom sample of the workload, %d NVE steps, rebuild every %d" % (
        s.n, args.steps, args.rebuild_every)
    line = {"impl": "reference", "metric": "atom-timesteps/s", "value": value, "unit": "atom-timesteps/s",
            "n_gpus": ws, "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * sec / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded FCC lattice, Maxwell-Boltzmann velocities)",
            "config": {"workload": args.workload, "description": w["desc"], "atoms": s.n},
            "cpu_baseline": {"value": value, "unit": "atom-timesteps/s", "cores": O.num_threads(),
                             "kind": "port", "sample": sample,
                             "note": "reference unbuildable here (needs onika, exaNBody, yaml-cpp, MPI); "
                                     "FP64 OpenMP restatement of its operators"},
            "e2e": {"value": value, "unit": "atom-timesteps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def _time_batch(b, torch, stream, reps, **kw):
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    b.run(**kw)
    b.synchronize()
    torch.cuda.synchronize()
    ev0.record(stream)
    for _ in range(reps):
        b.run(**kw)
    ev1.record(stream)
    b.synchronize()
    torch.cuda.synchronize()
    return ev0.elapsed_time(ev1) / reps


def bench_batched(stream, torch):
    """4,096 independent periodic copper-like replicas (32-2,048 atoms,
    log-uniform, FCC/BCC, strain <= 3%, 300-1,200 K displacements): forward
    + parameter adjoint in one persistent launch (CUDA graph), against one
    launch per replica."""
    from exastamp_gb300 import _capi, autotune, setfl, systems as S
    cfg = setfl.load_cu_params()
    sf = setfl.tabulate(cfg)
    reps = S.replica_set(nrep=4096, seed=6)
    n = sum(s.n for s in reps)
    J_F, J_f, J_z = setfl.table_param_jacobian(cfg)
    with _capi.Batch(0, stream.cuda_stream) as b:
        b.set_eam_alloy(sf, 5.0)
        b.set_param_derivatives(J_F, J_f, J_z)
        b.upload(reps)
        b.run()
        d = b.download()
        b.set_targets(d["F"] * 1.01, d["ep"] * 1.01, 1.0 / n, 0.1 / n)
        block, stencil, small_block, tun = autotune.tune_batch(b, "replicas4096", adjoint=True)
        ms_graph = _time_batch(b, torch, stream, 5, adjoint=True, use_graph=True)
        ms_fwd = _time_batch(b, torch, stream, 5, adjoint=False, use_graph=True)
        ms_each = _time_batch(b, torch, stream, 1, adjoint=True, per_replica=True)
    return {"replicas": len(reps), "atoms": n, "block": block, "stencil": stencil,
            "small_replica_block": small_block,
            "replicas_over_512_atoms": sum(1 for s in reps if s.n > 512),
            "ms_forward_adjoint_persistent_graph": ms_graph, "ms_forward_persistent_graph": ms_fwd,
            "ms_forward_adjoint_one_launch_per_replica": ms_each,
            "replicas_per_s": len(reps) / (ms_graph * 1e-3), "atom_evaluations_per_s": n / (ms_graph * 1e-3),
            "speedup_vs_one_launch_per_replica": ms_each / ms_graph, "autotune_ms": tun}


def bench_adjoint(stream, torch):
    """256 copper-like training configurations (4^3 FCC, 5% vacancies, a in
    [3.5, 3.75] A, Gaussian displacements 0.05-0.15 A), loss = mean |dF|^2 +
    0.1 mean dE^2 against targets from parameters scaled by U(0.9, 1.1):
    one forward + adjoint evaluation of the 9 parameter gradients."""
    from exastamp_gb300 import _capi, setfl, systems as S
    cfg = setfl.load_cu_params()
    confs = S.adjoint_training_set(nconf=256, ncell=4, seed=4)
    rng = np.random.default_rng(5)
    pert = {k: v * rng.uniform(0.9, 1.1) for k, v in cfg["params"].items()}
    n = sum(c.n for c in confs)
    with _capi.Batch(0, stream.cuda_stream) as b:
        b.set_eam_alloy(setfl.tabulate(cfg, pert), 5.0)
        b.upload(confs)
        b.run()
        t = b.download()
        b.set_eam_alloy(setfl.tabulate(cfg), 5.0)
        b.set_param_derivatives(*setfl.table_param_jacobian(cfg))
        b.set_targets(t["F"], t["ep"], 1.0 / n, 0.1 / n)
        ms = _time_batch(b, torch, stream, 10, adjoint=True, use_graph=True)
        g = b.download()
    return {"configurations": len(confs), "atoms": n, "ms_per_loss_and_gradient": ms, "loss": g["loss"],
            "grad": dict(zip(setfl.PARAM_NAMES, g["grad"].tolist()))}




# ---------------------------------------------------------------------------
KEYS9 = ("x", "y", "z", "vx", "vy", "vz", "ax", "ay", "az")


def _etot(th):
    """Total energy (kinetic + potential) of each thermo row."""
    return th[:, 21:24].sum(1) + th[:, 24]


def _drift(th, every, n):
    """Energy drift per atom per 1,000 steps: end minus start, and the slope
    of a least-squares line through the thermo rows (every `every` steps)."""
    e = _etot(th)
    t = np.arange(len(e)) * float(every)
    slope = float(np.polyfit(t, e, 1)[0]) if len(e) > 2 else float("nan")
    steps = t[-1] if len(t) > 1 else 1.0
    return {"end_minus_start": float(e[-1] - e[0]) / n / steps * 1000.0, "fit": slope / n * 1000.0,
            "steps": int(steps), "thermo_every": every}


def _rel_rms(a, b):
    return float(np.sqrt(((a - b) ** 2).sum() / max((b ** 2).sum(), 1e-300)))


def oracle_force_check(ctx, s, w, sample):
    """Relative RMS error of the GPU's mixed and FP64 forces against the FP64
    oracle at the context's current state.  EAM: every atom (the density
    pass needs all of them).  Pair potentials: the first `sample` atoms of
    a seeded permutation (their lists built among all atoms)."""
    O = _oracle()
    d = ctx.download(("x", "y", "z"))
    ctx.set_precision(True)
    ctx.compute_forces(energy=False)
    am = ctx.download(("ax", "ay", "az"))
    ctx.set_precision(False)
    ctx.compute_forces(energy=False)
    a64 = ctx.download(("ax", "ay", "az"))
    ctx.set_precision(True)
    x, y, z = d["x"].copy(), d["y"].copy(), d["z"].copy()
    O.wrap(x, y, z, s.lo, s.hi)
    t0 = time.perf_counter()
    if w["kind"] == "eam":
        from exastamp_gb300 import setfl, systems as S
        tab = O.EamOracleTables.from_setfl(setfl.tabulate(setfl.load_cu_params()), S.EV, S.EV, rcut=w["rcut"])
        nl = O.build_neighbors(x, y, z, s.id, s.lo, s.hi, w["rcut"] + w["skin"])
        fx, fy, fz, _, _, _, _ = O.eam_forces(x, y, z, s.type, nl, s.L, tab, w["rcut"], virial=False)
        sel = np.arange(s.n)
        F = np.stack([fx, fy, fz], 1) / s.masses[s.type][:, None]
        how = "all %d atoms" % s.n
    elif w["kind"] == "lj":
        nl = O.build_neighbors(x, y, z, s.id, s.lo, s.hi, w["rcut"] + w["skin"])
        fx, fy, fz, _, _ = O.lj_force(x, y, z, nl, s.L, 1.0, 1.0, w["rcut"], virial=False)
        sel = np.arange(s.n)
        F = np.stack([fx, fy, fz], 1) / s.masses[s.type][:, None]
        how = "all %d atoms" % s.n
    else:
        from exastamp_gb300 import systems as S
        perm = np.random.default_rng(7).permutation(s.n)
        m = min(sample, s.n)
        sel = perm[:m]
        xp, yp, zp = x[perm], y[perm], z[perm]
        ids, types = s.id[perm], np.ascontiguousarray(s.type[perm])
        eps, sig, rc = S.kob_andersen_tables()
        rcmax = float(rc.max())
        nl = O.build_neighbors_first(xp, yp, zp, ids, s.lo, s.hi, rcmax + w["skin"], m)
        fx, fy, fz, _, _ = O.lj_multi_force(xp, yp, zp, types, nl, s.L, eps, sig, rc, rcmax, virial=False)
        F = np.stack([fx, fy, fz], 1) / s.masses[types[:m]][:, None]
        how = "%d atoms of %d (seeded sample; their lists built among all atoms)" % (m, s.n)
    t_orc = time.perf_counter() - t0
    M = np.stack([am[k][sel] for k in ("ax", "ay", "az")], 1)
    G = np.stack([a64[k][sel] for k in ("ax", "ay", "az")], 1)
    return {"force_rel_rms_error_mixed_vs_oracle": _rel_rms(M, F),
            "force_rel_rms_error_fp64_vs_oracle": _rel_rms(G, F),
            "oracle_atoms": how, "oracle_seconds": t_orc, "oracle_threads": O.num_threads()}


def nve_drift(ctx, s, w, R, mixed_steps, fp64_steps):
    """From one saved state: mixed_steps NVE steps in mixed precision, then
    fp64_steps from the same state through the plain-FP64 kernels (thermo
    every 20 steps); drifts per atom per 1,000 steps in internal units and
    in eV (EAM) or epsilon (LJ)."""
    from exastamp_gb300 import systems as S
    st = ctx.download(KEYS9)
    unit = S.EV if w["kind"] == "eam" else 1.0
    out = {"unit": "eV per atom per 1000 steps" if w["kind"] == "eam" else "epsilon per atom per 1000 steps"}
    for name, mixed, nsteps in (("mixed", True, mixed_steps), ("fp64", False, fp64_steps)):
        ctx.upload_state(*(st[k] for k in KEYS9))
        ctx.set_precision(mixed)
        t0 = time.perf_counter()
        th = ctx.run_nve(nsteps, w["dt"], R, 20, use_graph=True)
        ctx.synchronize()
        dd = _drift(th, 20, s.n)
        out[name] = {"steps": nsteps, "seconds": time.perf_counter() - t0,
                     "drift_end_minus_start": dd["end_minus_start"] / unit, "drift_fit": dd["fit"] / unit}
        if mixed and nsteps >= fp64_steps:
            dd2 = _drift(th[: fp64_steps // 20 + 1], 20, s.n)
            out["mixed_first_%d_steps" % fp64_steps] = {"drift_end_minus_start": dd2["end_minus_start"] / unit,
                                                         "drift_fit": dd2["fit"] / unit}
    ctx.upload_state(*(st[k] for k in KEYS9))
    ctx.set_precision(True)
    return out


def two_level_section(ctx, s, w, R, torch, stream, steps=200, buffer=1.0):
    """From one saved state: `steps` NVE steps (rebuild every R, CUDA graphs)
    with the one-level list, then the same steps with the two-level list
    (gbmd_set_list_buffer(buffer)), each after a fresh full build.  An outer
    build comes every ~100 steps in this state, so a window of this length
    holds its amortised cost (a 20-step window holds one or none)."""
    st = ctx.download(KEYS9)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    out = {"steps": steps, "list_buffer": buffer, "rebuild_every": R}
    for name, b in (("one_level", 0.0), ("two_level", buffer)):
        ctx.upload_state(*(st[k] for k in KEYS9))
        ctx.set_list_buffer(b)
        ctx.build_neighbors()
        ctx.run_nve(2 * R, w["dt"], R, 0, use_graph=True)  # graph capture
        ctx.upload_state(*(st[k] for k in KEYS9))
        ctx.build_neighbors()
        b0, o0 = ctx.list_builds(), ctx.list_buffer()[1]
        torch.cuda.synchronize()
        ev0.record(stream)
        ctx.run_nve(steps, w["dt"], R, 0, use_graph=True)
        ev1.record(stream)
        torch.cuda.synchronize()
        out[name] = {"ms_per_step": ev0.elapsed_time(ev1) / steps, "list_builds": ctx.list_builds() - b0,
                     "outer_builds": ctx.list_buffer()[1] - o0}
    out["one_level_over_two_level"] = out["one_level"]["ms_per_step"] / out["two_level"]["ms_per_step"]
    ctx.set_list_buffer(w.get("list_buffer", 0.0))
    ctx.upload_state(*(st[k] for k in KEYS9))
    ctx.build_neighbors()
    return out


def e2e_section(ctx, s, w, R, steps, ws, torch, stream):
    """The same step through the C ABI with the grid state in pinned host
    arrays: gbmd_run_nve_host per step, copies inside the timed region."""
    n = s.n
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    pin = lambda: torch.empty(n, dtype=torch.float64, pin_memory=True).numpy()  # noqa: E731
    host = {k: pin() for k in KEYS9}
    d = ctx.download(KEYS9)
    for k in host:
        host[k][:] = d[k]
    L = ctx._L
    ptr = lambda k: host[k].ctypes.data  # noqa: E731
    start = {k: host[k].copy() for k in KEYS9}
    dt = w["dt"]
    # untimed: the first host-step call allocates its position staging buffer
    ctx._chk(L.gbmd_run_nve_host(ctx.h, 1, dt, R, *[ptr(k) for k in KEYS9]))

    def loop(host_call):
        """K steps from the same state, list freshly built: (CUDA-event ms,
        wall ms, list builds)."""
        for k in KEYS9:
            host[k][:] = start[k]
        ctx.upload_state(*(host[k] for k in KEYS9))
        ctx.build_neighbors()
        b0 = ctx.list_builds()
        torch.cuda.synchronize()
        ev0.record(stream)
        t0 = time.perf_counter()
        for _ in range(steps):
            if host_call:
                ctx._chk(L.gbmd_run_nve_host(ctx.h, 1, dt, R, *[ptr(k) for k in KEYS9]))
            else:
                ctx._chk(L.gbmd_upload_state(ctx.h, *[ptr(k) for k in KEYS9]))
                ctx._chk(L.gbmd_run_nve(ctx.h, 1, dt, R, 0, None, 0))
                ctx._chk(L.gbmd_download(ctx.h, *[ptr(k) for k in KEYS9], None, None))
        ev1.record(stream)
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
        return ev0.elapsed_time(ev1), wall * 1e3, ctx.list_builds() - b0

    sep_ms, sep_wall, _ = loop(False)   # the same step as three calls, for comparison
    ctx.set_host_pipeline(0)
    unpiped_ms, unpiped_wall, _ = loop(True)   # one call per step, host link not overlapped
    ctx.set_host_pipeline(-1)
    slabs, piped0, redone0 = ctx.host_pipeline()
    mse, wall_ms, builds = loop(True)
    piped = ctx.host_pipeline()[1] - piped0
    redone = ctx.host_pipeline()[2] - redone0
    timeline = None
    if slabs:
        # one more (untimed) step with the pipeline's timeline recorded
        ctx.set_host_pipeline_trace(True)
        for k in KEYS9:
            host[k][:] = start[k]
        ctx.upload_state(*(host[k] for k in KEYS9))
        ctx.build_neighbors()
        ctx._chk(L.gbmd_run_nve_host(ctx.h, 1, dt, R, *[ptr(k) for k in KEYS9]))
        ctx._chk(L.gbmd_run_nve_host(ctx.h, 1, dt, R, *[ptr(k) for k in KEYS9]))
        marks = ctx.host_pipeline_trace()
        ctx.set_host_pipeline_trace(False)
        last = lambda kind: max((m[0] for m in marks if m[1] == kind), default=None)  # noqa: E731
        timeline = {"ms_last_chunk_in": last("in"), "ms_last_density": last("density"),
                    "ms_last_force": last("force"), "ms_last_chunk_out": last("out"), "ms_end": last("end"),
                    "marks": [[round(m[0], 4), m[1], m[2]] for m in marks]}
    mse = dist_max(max(mse, wall_ms), ws)
    sep_ms = max(sep_ms, sep_wall)
    t0 = time.perf_counter()
    for _ in range(3):
        ctx._chk(L.gbmd_upload_state(ctx.h, *[ptr(k) for k in KEYS9]))
    up_ms = (time.perf_counter() - t0) * 1e3 / 3
    t0 = time.perf_counter()
    for _ in range(3):
        ctx._chk(L.gbmd_download(ctx.h, *[ptr(k) for k in KEYS9], None, None))
    down_ms = (time.perf_counter() - t0) * 1e3 / 3
    return {"value": n * steps * ws / (mse * 1e-3), "unit": "atom-timesteps/s",
            "upload_ms": up_ms, "download_ms": down_ms,
            "h2d_bytes_per_step": 72 * n, "d2h_bytes_per_step": 72 * n, "steps": steps,
            "ms_per_step": mse / steps, "ms_per_step_as_three_calls": sep_ms / steps,
            "ms_per_step_unpipelined": max(unpiped_ms, unpiped_wall) / steps,
            "list_builds": builds, "slabs": slabs, "pipelined_steps": piped,
            "pipelined_steps_discarded_for_a_rebuild": redone, "pipeline_timeline": timeline,
            "host_order": "grid cells, z slowest (as the reference's grid stores atoms)",
            "path": "gbmd_run_nve_host(1 step, pinned r,v,a): chunks of the caller order read over the host link "
                    "with the first half and skin/2 test applied, pair passes slab by slab as their chunks "
                    "arrive, v,a written back chunk by chunk; a step that needs a rebuild finishes unpipelined"
            if slabs else "gbmd_run_nve_host(1 step; pinned r,v,a read with the first half applied, skin/2 "
                          "displacement test, r copied back during the force pass, then v,a)"}


def measure(args, w, ws, dev, stream, torch, *, steps, fp64_steps, e2e_steps, drift_steps, oracle_sample,
            name):
    """One workload on one GPU: the device-resident timed region (value), the
    roofline of its final pair kernel, and the optional sections (FP64
    comparison, oracle force check, NVE drift, e2e).  Returns the fields of
    the JSON line."""
    from exastamp_gb300 import _capi
    s = make_system(w)
    ctx = _capi.Context(dev, stream.cuda_stream)
    ctx.upload_system(s)
    bind_potential(ctx, w)
    t_min = None
    tuned = None
    # clocks are sampled every 200 ms from here (thermalisation or minimiser,
    # tuning, warm-up: the GPU under the same kernels) to the end of the
    # timed region, which alone is too short for more than a sample or two
    clk = ClockSampler(dev).__enter__()
    if w.get("min_steps"):
        # random positions overlap: the first steps of the clipped minimiser
        # in FP64 (separations far below sigma), the rest in mixed precision
        t0 = time.perf_counter()
        ctx.set_precision(False)
        ctx.run_minimize(w["min_fp64_steps"], MIN_DT, tolF=MIN_TOLF, rebuild_every=args.rebuild_every)
        ctx.set_precision(True)
        ctx.run_minimize(w["min_steps"] - w["min_fp64_steps"], MIN_DT, tolF=MIN_TOLF,
                         rebuild_every=args.rebuild_every)
        ctx.synchronize()
        t_min = time.perf_counter() - t0
    ctx.set_precision(args.precision == "mixed")
    t_therm = None
    if not w.get("min_steps") and args.thermalise > 0:
        # a perfect lattice gathers far fewer distinct spline knots and list
        # layouts than the thermal state the timed steps see: tune on the latter
        t0 = time.perf_counter()
        ctx.run_nve(args.thermalise, w["dt"], args.rebuild_every, 0, use_graph=True)
        ctx.synchronize()
        t_therm = time.perf_counter() - t0
    if args.lanes:
        ctx.set_launch(args.lanes, args.block or 128, args.vec)
        ctx.set_neighbor_staging(args.staging)
        ctx.set_newton3(args.newton3)
    else:
        from exastamp_gb300 import autotune
        lanes, vec, block, tuned = autotune.tune(ctx, key="%s-%s" % (name, args.precision))
    R, dt = args.rebuild_every, w["dt"]
    # fixed interval: thermo at the end of each 2R-step graph chunk; with the
    # displacement trigger (R = -1) every 20 steps
    thermo_every = 2 * R if R > 0 else (20 if R < 0 else 0)
    # warm-up: at least W steps in a whole number of thermo intervals, then
    # two runs of min(K, 2 chunks) steps.  The runner replays CUDA graphs of
    # 20-step chunks (one for a chunk followed by more steps, one for the
    # chunk that ends a run), kept per parity of its double buffers; a run
    # flips that parity, so the two short runs capture both graphs at both
    # parities here rather than inside the timed region.  When that run
    # length is a whole number of thermo intervals the timed run starts from
    # a state whose energies are current (its step-0 thermo row needs only
    # the reduction).
    warm = max(args.warmup, 3)
    if thermo_every:
        warm = -(-warm // thermo_every) * thermo_every
    ctx.run_nve(warm, dt, R, thermo_every, use_graph=True)
    short = min(steps, 2 * thermo_every) if thermo_every else steps
    for _ in range(2):
        ctx.run_nve(short, dt, R, thermo_every, use_graph=True)
    warm += 2 * short
    energies_reused = bool(thermo_every) and short % thermo_every == 0
    npairs, maxnb, nc = ctx.neighbor_stats()

    # ---- timed region: K steps, device resident --------------------------
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    try:
        barrier(ws)
        torch.cuda.synchronize()
        builds0 = ctx.list_builds()
        outer0 = ctx.list_buffer()[1]
        ev0.record(stream)
        ctx.run_nve(steps, dt, R, thermo_every, use_graph=True)
        ev1.record(stream)
        torch.cuda.synchronize()
        barrier(ws)
        rebuilds = ctx.list_builds() - builds0
        outer_builds = ctx.list_buffer()[1] - outer0
    finally:
        clk.__exit__()
    ms = ev0.elapsed_time(ev1)
    ms = dist_max(ms, ws)
    clocks = clk.summary()
    clocks["window"] = "sampled every 200 ms from the thermalisation/minimiser through the timed region"
    value = s.n * steps * ws / (ms * 1e-3)
    # EAM: density + force; Newton-3 LJ: half-list pair pass + epilogue
    kernels_per_step = 2 if w["kind"] == "eam" or args.newton3 else 1
    # Launches of the timed gbmd_run_nve call: the pair kernel(s) once per
    # step; the thermo reduction (2)
    # at step 0 and every thermo_every steps; the standalone first half at
    # the start and after every thermo step but the last; the rebuild chain
    # (wrap/bin, 3 scan kernels, scatter, rank, gather, posf, list build) per
    # rebuild.  With the trigger the kernels that move the atoms test them, and
    # a graph step launches the conditional's setter, plus the 13-kernel
    # rebuild body (2 fills, the chain, copy-back, reference positions) when
    # the gate opens; the steps after the last whole graph chunk run the 13
    # gated launches every step.
    n_thermo = steps // thermo_every if thermo_every else 0
    last_is_thermo = bool(thermo_every) and steps % thermo_every == 0
    # step 0's forces and energies are recomputed unless the warm-up ended on
    # a thermo step
    gpu_launches = kernels_per_step * (steps if energies_reused else steps + 1)
    gpu_launches += 2 * (n_thermo + (1 if thermo_every else 0))
    gpu_launches += 1 + n_thermo - (1 if last_is_thermo else 0)
    # With a list buffer a rebuild is the outer test, the conditional's
    # setter and the filter (3), plus 13 for an outer build (2 fills, the
    # chain, copy-back, outer positions); with the trigger all 16 are gated
    # launches inside its body.
    two_level = w.get("list_buffer", 0.0) > 0.0
    if R < 0:
        n_graph = (steps // thermo_every) * thermo_every
        per = 16 if two_level else 13
        gpu_launches += n_graph + per * rebuilds + per * (steps - n_graph)
    elif two_level:
        gpu_launches += 3 * rebuilds + 13 * outer_builds
    else:
        gpu_launches += 9 * rebuilds

    out = {"metric": "atom-timesteps/s", "value": value, "unit": "atom-timesteps/s", "n_gpus": ws,
           "steps": steps, "warmup": args.warmup, "ms_per_step": ms / steps,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
           "dtype": "f32-pair/f64-state" if args.precision == "mixed" else "f64",
           "data": "synthetic (seeded random positions with voids, Maxwell-Boltzmann velocities)"
           if w["kind"] == "lj_multi" else "synthetic (seeded FCC lattice, Maxwell-Boltzmann velocities)",
           "config": {"workload": name, "description": w["desc"], "atoms": s.n,
                      "precision": args.precision, "thermo_every": thermo_every,
                      "rebuild_every": R if R >= 0 else "on displacement > skin/2",
                      "list_builds_in_timed_region": rebuilds,
                      "list_buffer": w.get("list_buffer", 0.0),
                      "outer_list_builds_in_timed_region": outer_builds,
                      "warmup_steps_run": warm,
                      "neighbours_per_atom": npairs / s.n, "cells": nc.tolist(),
                      "lanes_per_atom": ctx.get_launch_ex()[0], "list_entries_per_load": ctx.get_launch_ex()[1],
                      "block": ctx.get_launch_ex()[2], "density_block": ctx.get_density_block(),
                      "staged_neighbour_positions": ctx.get_neighbor_staging(),
                      "newton3_half_list": ctx.get_newton3(),
                      "parallelism": "replicas" if ws > 1 else "single-gpu",
                      "l2": "inputs larger than L2 (neighbour list %.2f GB)" % (npairs * 4 / 1e9)
                      if npairs * 4 > 129e6 else "inputs resident in L2 (not flushed)",
                      "cuda_graph": True},
           "gpu_launches": gpu_launches, "clocks": clocks}
    if tuned:
        out["autotune_density_plus_pair_ms"] = tuned
    if t_therm is not None:
        out["thermalisation"] = {"steps": args.thermalise, "seconds": t_therm,
                                 "note": "untimed NVE steps from the lattice before tuning and warm-up"}
    if t_min is not None:
        out["minimiser"] = {"steps": w["min_steps"], "step": MIN_DT, "clip": MIN_TOLF,
                            "precision": "fp64 for the first %d steps, then mixed" % w["min_fp64_steps"],
                            "seconds": t_min}

    # ---- per-kernel timing for the roofline -------------------------------
    prof = ctx.profile_step(reps=10)
    peak, peak_kind = measured_peaks()
    nbar = npairs / s.n
    if w["kind"] == "eam":
        # list 4 B/entry, own posf 16 B + F' 4 B, state r 24+24, v 24+24, a 24, posf 16, posd 32 written
        per_atom = 4.0 * nbar + 16 + 4 + 48 + 48 + 24 + 16 + 32
    else:
        per_atom = 4.0 * nbar + 16 + 48 + 48 + 24 + 16 + 32
    alg_bytes = per_atom * s.n
    t_pair = prof["pair"] * 1e-3
    achieved = alg_bytes / t_pair / 1e9
    traffic, traffic_src = None, None
    if w["kind"] == "eam" and args.precision == "mixed":
        # DRAM bytes per atom of k_eam_force_mixed from one ncu capture of the
        # same kernel on the 864,000-atom case (60^3 cells), scaled by atoms
        traffic = EAM_FORCE_DRAM_BYTES_PER_ATOM * s.n
        traffic_src = ("ncu dram__bytes_read.sum + dram__bytes_write.sum of k_eam_force_mixed<1,4> on the "
                       "864,000-atom case (273.8 + 51.0 MB), scaled to %d atoms" % s.n)
    elif w["kind"] == "lj_multi" and args.precision == "mixed":
        traffic = LJ_MULTI_PAIR_DRAM_BYTES_PER_ATOM * s.n
        traffic_src = ("ncu dram__bytes_read.sum + dram__bytes_write.sum of k_lj_mixed<1,4,multi> on the "
                       "864,000-atom mixture (474.0 + 51.9 MB), scaled to %d atoms" % s.n)
    # the resource that binds the pair kernels (ncu on the 864,000-atom cases)
    binding = ({"resource": "L1/tex LSU data-pipe wavefronts (neighbour and spline-knot gathers)", "frac": 0.796,
                "source": "ncu l1tex__data_pipe_lsu_wavefronts.avg.pct_of_peak_sustained_elapsed of "
                          "k_eam_force_mixed<1,4> (density kernel: 0.858)"}
               if w["kind"] == "eam" else
               {"resource": "issue slots + L1/tex (neighbour gathers)", "frac": 0.78,
                "source": "ncu smsp__issue_active of k_lj_mixed<1,4,multi> (L1/tex throughput 0.75)"}
               if w["kind"] == "lj_multi" else None)
    out["roofline"] = {"kernel": "k_eam_force (mixed, fused Verlet halves)" if w["kind"] == "eam" else "k_lj",
                       "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                       "frac": achieved / peak, "peak_source": peak_kind,
                       "algorithmic_bytes_per_launch": alg_bytes, "bytes_per_atom": per_atom,
                       "traffic": traffic, "traffic_source": traffic_src, "binding": binding, "kernel_ms": prof}
    if w["kind"] == "eam" and args.precision == "mixed":
        # the FP-pipe side of the same kernels: useful flops per unordered
        # pair within rc (density 20, force 54, embedding 14 per atom), the
        # FCC Cu lattice's 42 neighbours within rc=5.0 A (21 unordered pairs
        # per atom), against the nominal FP32 rate (no measured FP32 peak)
        pairs = 21.0 * s.n
        fp32_peak = 152 * 128 * 2 * (measured_clock_mhz() or 2070.0) * 1e6 / 1e12
        dens_tf = (20.0 * pairs + 14.0 * s.n) / (prof["density"] * 1e-3) / 1e12
        force_tf = 54.0 * pairs / (prof["pair"] * 1e-3) / 1e12
        out["roofline"]["fp32"] = {
            "useful_flop_per_launch": {"density": 20.0 * pairs + 14.0 * s.n, "force": 54.0 * pairs},
            "achieved_tflops": {"density": dens_tf, "force": force_tf}, "nominal_peak_tflops": fp32_peak,
            "frac": {"density": dens_tf / fp32_peak, "force": force_tf / fp32_peak},
            "peak_source": "nominal: 152 SMs x 128 FP32 lanes x 2 flop x max SM clock (not measured)",
            "pairs_source": "42 lattice neighbours within rc per atom, counted once per unordered pair"}

    single = ws == 1
    # ---- accuracy against the FP64 oracle at the benchmarked state ----------
    if single and not args.no_oracle_check and args.precision == "mixed":
        out["accuracy"] = oracle_force_check(ctx, s, w, oracle_sample)

    # ---- FP64 comparison ----------------------------------------------------
    if single and not args.no_fp64:
        st = ctx.download(KEYS9)
        ctx.set_precision(args.precision == "mixed")
        ctx.compute_forces(energy=False)
        d_mixed = ctx.download(("ax", "ay", "az"))
        ctx.set_precision(False)
        ctx.compute_forces(energy=False)
        d64 = ctx.download(("ax", "ay", "az"))
        A = np.stack([d_mixed[k] for k in ("ax", "ay", "az")], 1)
        B = np.stack([d64[k] for k in ("ax", "ay", "az")], 1)
        ferr = _rel_rms(A, B)
        ctx.run_nve(3, dt, R, 0, use_graph=False)
        torch.cuda.synchronize()
        ev0.record(stream)
        ctx.run_nve(fp64_steps, dt, R, 0, use_graph=True)
        ev1.record(stream)
        torch.cuda.synchronize()
        ms64 = ev0.elapsed_time(ev1)
        v64 = s.n * fp64_steps / (ms64 * 1e-3)
        out["fp64"] = {"value": v64, "ms_per_step": ms64 / fp64_steps, "steps": fp64_steps,
                       "mixed_over_fp64": value / v64, "force_rel_rms_error_mixed_vs_fp64": ferr}
        ctx.upload_state(*(st[k] for k in KEYS9))
        ctx.set_precision(args.precision == "mixed")

    # ---- NVE energy drift, mixed vs FP64 from one state -----------------------
    if single and not args.no_drift and drift_steps:
        out["nve_drift"] = nve_drift(ctx, s, w, R, *drift_steps)

    # ---- one- and two-level neighbour lists over 200 steps ----------------------
    if single and not args.no_two_level and w["kind"] == "eam" and R > 0:
        out["two_level_list"] = two_level_section(ctx, s, w, R, torch, stream)

    # ---- end-to-end through the C ABI with host buffers -----------------------
    if not args.no_e2e:
        out["e2e"] = e2e_section(ctx, s, w, R, e2e_steps, ws, torch, stream)
    ctx.close()
    return out


def main():
    args = parse()
    w = WORKLOADS[args.workload]
    ws, rank, local = dist_setup(args)
    if args.impl == "reference":
        run_reference(args, w, ws, rank)
        return
    import torch
    assert torch.cuda.is_available(), "bench.py needs a GPU (no CPU fallback)"
    dev = local if ws > 1 else 0
    torch.cuda.set_device(dev)
    stream = torch.cuda.Stream(device=dev)
    eam = w["kind"] == "eam"
    out = measure(args, w, ws, dev, stream, torch, steps=args.steps, fp64_steps=args.fp64_steps,
                  e2e_steps=args.e2e_steps, drift_steps=(1000, 200) if eam else (500, 50),
                  oracle_sample=65536, name=args.workload)

    # ---- batched replicas (4,096 EAM systems) and the parameter adjoint --------
    if not args.no_batch and ws == 1:
        out["batched_replicas"] = bench_batched(stream, torch)
        out["parameter_adjoint"] = bench_adjoint(stream, torch)

    # ---- CPU baseline (rank 0, N=1) -------------------------------------------
    if not args.no_cpu and ws == 1 and rank == 0:
        rate, info = cpu_oracle_rate(w)
        out["cpu_baseline"] = {"value": rate, "unit": "atom-timesteps/s", "cores": info["threads"],
                               "kind": "port",
                               "sample": "%d-atom sample of the workload, %d FP64 NVE steps on the OpenMP "
                                         "oracle (%.1f s)" % (info["atoms"], info["steps"], info["seconds"])}

    # ---- the 16.7 M-atom LJ binary mixture, in the same line -------------------
    if eam and not args.no_mixture and not args.ncell and ws == 1:
        wm = WORKLOADS["lj_binary_16m"]
        mix = measure(args, wm, ws, dev, stream, torch, steps=args.steps, fp64_steps=10, e2e_steps=10,
                      drift_steps=(500, 50), oracle_sample=65536, name="lj_binary_16m")
        if not args.no_cpu and rank == 0:
            rate, info = cpu_oracle_rate(wm, target_s=8.0)
            mix["cpu_baseline"] = {"value": rate, "unit": "atom-timesteps/s", "cores": info["threads"],
                                   "kind": "port",
                                   "sample": "%d-atom sample of the workload (minimised first), %d FP64 NVE "
                                             "steps on the OpenMP oracle (%.1f s)"
                                             % (info["atoms"], info["steps"], info["seconds"])}
        for k in ("metric", "unit", "n_gpus", "steps", "warmup", "higher_is_better", "scaling", "vs_baseline"):
            mix.pop(k, None)
        out["lj_mixture"] = mix
    # ---- the 32,000-atom LJ crystal (the CPU-runnable case), in the same line --
    if eam and not args.no_lj_crystal and not args.ncell and ws == 1:
        wc = WORKLOADS["lj_fcc_32k"]
        c1 = measure(args, wc, ws, dev, stream, torch, steps=args.steps, fp64_steps=40, e2e_steps=20,
                     drift_steps=(100, 100), oracle_sample=0, name="lj_fcc_32k")
        if not args.no_cpu and rank == 0:
            rate, info = cpu_oracle_rate(wc, target_s=5.0)
            c1["cpu_baseline"] = {"value": rate, "unit": "atom-timesteps/s", "cores": info["threads"],
                                  "kind": "port",
                                  "sample": "the whole %d-atom workload, %d FP64 NVE steps on the OpenMP oracle "
                                            "(%.1f s)" % (info["atoms"], info["steps"], info["seconds"])}
        for k in ("metric", "unit", "n_gpus", "steps", "warmup", "higher_is_better", "scaling", "vs_baseline"):
            c1.pop(k, None)
        out["lj_fcc_32k"] = c1
    if rank == 0:
        print(json.dumps(out), flush=True)
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
