"""Autotuner for the pair kernels' launch shape.

The knobs are the lanes that share one atom's neighbour list (1-16; more
lanes give more parallelism for small systems, fewer lanes avoid the
per-atom shuffle reduction for large ones), the list entries each lane reads
per load (1, or 4 in one 16-byte load with at most 4 lanes), whether
neighbour positions come from shared-memory staging (1 lane x 4 entries) and
the threads per block.  tune() leaves the staging choice set on the context.  Each
candidate is timed with gbmd_profile_step (CUDA events on the context's
stream, density + final pair kernel) and the fastest is kept.  Results are
cached in a JSON file keyed by GPU name, workload key and atom count
($GBMD_AUTOTUNE_CACHE, default ~/.cache/exastamp_gb300/autotune.json).
"""
from __future__ import annotations

import json
import os

LANES = (1, 2, 4, 8, 16)
VECS = (1, 4)
BLOCKS = (64, 128, 256)


def _cache_path():
    return os.environ.get("GBMD_AUTOTUNE_CACHE",
                          os.path.join(os.path.expanduser("~"), ".cache", "exastamp_gb300", "autotune.json"))


def _gpu_name():
    try:
        import torch
        return torch.cuda.get_device_name(0)
    except Exception:
        return "unknown"


def _load():
    try:
        with open(_cache_path()) as fh:
            return json.load(fh)
    except Exception:
        return {}


def _store(d):
    p = _cache_path()
    try:
        os.makedirs(os.path.dirname(p), exist_ok=True)
        tmp = "%s.%d.tmp" % (p, os.getpid())  # one per process: ranks may store at once
        with open(tmp, "w") as fh:
            json.dump(d, fh, indent=1)
        os.replace(tmp, p)
    except OSError:
        pass


def tune_batch(batch, key: str, blocks=(128, 256, 512), stencils=(1, 2), small_blocks=(64, 128, 256),
               adjoint=False, reps: int = 3, use_cache: bool = True):
    """Pick (block, stencil radius, small-replica block) for a gbmd_batch:
    each candidate runs the persistent launch `reps` times, timed on the host
    around a synchronize; the small-replica kernel's block is tried last, with
    the best (block, stencil).  Leaves the choice set on the batch and returns
    (block, stencil, small_block, timings)."""
    import time

    def timed():
        batch.run(adjoint=adjoint)
        batch.synchronize()
        t0 = time.perf_counter()
        for _ in range(reps):
            batch.run(adjoint=adjoint)
        batch.synchronize()
        return (time.perf_counter() - t0) * 1e3 / reps

    ck = "%s|batch2|%s|%d|%d|%d" % (_gpu_name(), key, batch.nrep, batch.n, int(adjoint))
    cache = _load() if use_cache else {}
    if ck in cache:
        e = cache[ck]
        batch.set_launch(int(e["block"]), int(e["stencil"]))
        batch.set_small_block(int(e["small_block"]))
        return int(e["block"]), int(e["stencil"]), int(e["small_block"]), e.get("timings", {})
    timings, best = {}, None
    batch.set_small_block(128)
    for s in stencils:
        for b in blocks:
            batch.set_launch(b, s)
            ms = timed()
            timings["%dx%d" % (b, s)] = ms
            if best is None or ms < best[0]:
                best = (ms, b, s)
    _, b, s = best
    batch.set_launch(b, s)
    best_small = None
    for sb in small_blocks:
        batch.set_small_block(sb)
        ms = timed()
        timings["%dx%d small %d" % (b, s, sb)] = ms
        if best_small is None or ms < best_small[0]:
            best_small = (ms, sb)
    batch.set_small_block(best_small[1])
    cache[ck] = {"block": b, "stencil": s, "small_block": best_small[1], "timings": timings}
    if use_cache:
        _store(cache)
    return b, s, best_small[1], timings


def tune(ctx, key: str, lanes=LANES, blocks=BLOCKS, vecs=VECS, reps: int = 3, use_cache: bool = True):
    """Return (lanes, entries per load, block, timings) for this context's
    system and potential and leave the chosen shape set on the context: the
    pair-kernel block, the density-kernel block (chosen separately, the two
    kernels being independent) and the staging switch."""
    n = ctx.n
    ck = "%s|%s|%d|vsd" % (_gpu_name(), key, n)
    cache = _load() if use_cache else {}
    if ck in cache:
        e = cache[ck]
        ctx.set_launch(int(e["lanes"]), int(e["block"]), int(e["vec"]))
        ctx.set_neighbor_staging(bool(e.get("staged", False)))
        ctx.set_density_block(int(e.get("density_block", 0)))
        return int(e["lanes"]), int(e["vec"]), int(e["block"]), e.get("timings", {})
    timings = {}
    best = None
    for t in lanes:
        for v in vecs:
            if v > 1 and t > 4:
                continue
            # shared-memory staging of neighbour positions exists for 1 lane x 4 entries
            for staged in ((False, True) if (t == 1 and v == 4) else (False,)):
                dens, pair = {}, {}
                for b in blocks:
                    if b % t:
                        continue
                    ctx.set_launch(t, b, v)
                    ctx.set_density_block(0)
                    ctx.set_neighbor_staging(staged)
                    prof = ctx.profile_step(reps=reps)
                    dens[b], pair[b] = prof["density"], prof["pair"]
                    timings["%dx%dx%d%s" % (t, v, b, "s" if staged else "")] = [prof["density"], prof["pair"]]
                bd = min(dens, key=dens.get)
                bp = min(pair, key=pair.get)
                ms = dens[bd] + pair[bp]
                if best is None or ms < best[0]:
                    best = (ms, t, v, bp, staged, bd)
    _, t, v, bp, staged, bd = best
    cache[ck] = {"lanes": t, "vec": v, "block": bp, "staged": staged, "density_block": bd, "timings": timings}
    if use_cache:
        _store(cache)
    ctx.set_launch(t, bp, v)
    ctx.set_neighbor_staging(staged)
    ctx.set_density_block(bd)
    return t, v, bp, timings
