"""Autotuner for the fused kernels' launch variants.

Two knobs, each a compile-time variant of one fused kernel (every variant
computes the same result, bit for bit):

* ``fp_batch`` -- Siddon steps walked per gather round in the forward
  projection (2, 4, 8): more steps keep more volume gathers in flight but use
  more registers (fewer resident warps); 2 and 4 are also tried with the
  volume staged slab by slab in shared memory by TMA (``fp_stage``), where
  the geometry allows it;
* ``upd_planes`` -- z planes walked per block by the fused update (8, 16, 32):
  deeper slabs amortise the halo planes, shallower ones give more blocks;
  tried with each update tile (``upd_tile``: one voxel per thread; two side
  by side in x, with fewer instructions per voxel but fewer resident blocks,
  when the subsets hold one view each; or one voxel per thread with the
  planes streamed by TMA through a ring filled by a producer warp, where the
  volume's rows allow TMA); a tile other than the default one voxel per
  thread must win by ``TILE_MARGIN``.

The tuner times each variant on the plan's own geometry (CUDA events on the
launching stream, best of a few repetitions over all subsets) and keeps the
fastest of each knob.  Results are cached in a JSON file keyed by GPU name,
geometry and the parameters that change the work, at
``$NR_TUNE_CACHE`` or ``~/.cache/newrecon_gb300/tune.json``.
"""
from __future__ import annotations

import json
import os
from typing import Dict, Optional, Tuple

import torch

FP_BATCHES = (2, 4, 8)
# (fp_batch, fp_stage) variants of the projection: direct gathers for every
# batch, TMA-staged slabs for 2 and 4
FP_VARIANTS = ((2, 0), (4, 0), (8, 0), (2, 1), (4, 1))
UPD_PLANES = (8, 16, 32)
UPD_TILES = (0, 1, 2)  # NR_TILE_1, NR_TILE_2, NR_TILE_TMA
TILE_NAMES = {0: "", 1: "-x2", 2: "-tma"}
# A tile other than the default one-voxel tile is kept only when it beats the
# best one-voxel variant by this fraction: near a tie the choice would
# otherwise follow the timing noise from run to run.
TILE_MARGIN = 0.02


def cache_path() -> str:
    return os.environ.get("NR_TUNE_CACHE") or os.path.join(
        os.path.expanduser("~"), ".cache", "newrecon_gb300", "tune.json")


def signature(plan) -> str:
    g = plan.geom
    p = plan.params
    dev = torch.cuda.get_device_name(plan.ws.device)
    return (f"{dev}|{g.nx}x{g.ny}x{g.nz}|{g.nbx}x{g.nby}|A{g.n_angles}|M{p.subset_num}"
            f"|pot{p.potential}|scat{p.has_scatter}|v4")


def _load() -> Dict[str, dict]:
    try:
        with open(cache_path()) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _store(key: str, val: dict) -> None:
    path = cache_path()
    try:
        os.makedirs(os.path.dirname(path), exist_ok=True)
        data = _load()
        data[key] = val
        tmp = path + f".{os.getpid()}.tmp"
        with open(tmp, "w") as f:
            json.dump(data, f, indent=1, sort_keys=True)
        os.replace(tmp, path)
    except OSError:
        pass  # a read-only home: tune again next time


def _time(fn, reps: int) -> float:
    stream = torch.cuda.current_stream()
    best = float("inf")
    for _ in range(reps):
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        fn()
        b.record(stream)
        b.synchronize()
        best = min(best, a.elapsed_time(b))
    return best


def choose_update(up_ms: Dict[Tuple[int, int], float]) -> Tuple[int, int]:
    """(upd_tile, upd_planes) from the timings of the update variants: the
    fastest, except that a tile other than the one-voxel tile (0) must beat
    the fastest one-voxel variant by TILE_MARGIN."""
    best_t, best_z = min(up_ms, key=up_ms.get)
    if best_t != 0:
        z1 = min((z for t, z in up_ms if t == 0), key=lambda z: up_ms[(0, z)])
        if up_ms[(0, z1)] <= up_ms[(best_t, best_z)] * (1.0 + TILE_MARGIN):
            best_t, best_z = 0, z1
    return best_t, best_z


def apply_cached(plan) -> Optional[dict]:
    """Applies the cached choice for the plan's GPU, geometry and parameters;
    None (and the plan unchanged) when the cache holds none."""
    hit = _load().get(signature(plan))
    if not (hit and hit.get("fp_batch") in FP_BATCHES and hit.get("upd_planes") in UPD_PLANES
            and hit.get("fp_stage", 0) in (0, 1) and hit.get("upd_tile", 0) in UPD_TILES):
        return None
    plan.params.fp_batch = int(hit["fp_batch"])
    plan.params.upd_planes = int(hit["upd_planes"])
    plan.params.fp_stage = int(hit.get("fp_stage", 0))
    plan.params.upd_tile = int(hit.get("upd_tile", 0))
    return hit


def tune(plan, x: Optional[torch.Tensor] = None, reps: int = 3,
         use_cache: bool = True) -> Tuple[int, int, dict]:
    """Picks (fp_batch, upd_planes) -- with fp_stage and upd_tile -- for a set-up
    plan and applies them."""
    key = signature(plan)
    if use_cache:
        hit = apply_cached(plan)
        if hit is not None:
            return plan.params.fp_batch, plan.params.upd_planes, hit
    if x is None:
        x = torch.zeros(plan.geom.n_voxels, dtype=torch.float32, device=plan.ws.device)
    xo = torch.empty_like(x)
    M = plan.params.subset_num
    saved = (plan.params.fp_batch, plan.params.upd_planes, plan.params.fp_stage)
    one_view = plan.geom.n_angles == M  # the two-voxel tile serves one-view subsets
    fp_ms, up_ms = {}, {}
    for k, st in FP_VARIANTS:
        plan.params.fp_batch = k
        plan.params.fp_stage = st
        plan.project(x, 0)  # warm-up
        fp_ms[(k, st)] = _time(lambda: [plan.project(x, a) for a in range(M)], reps)
    plan.params.fp_batch, plan.params.fp_stage = saved[0], saved[2]
    plan.project(x, 0)  # h of subset 0 for the update timings
    for t in (UPD_TILES if one_view else (0, 2)):
        for z in UPD_PLANES:
            plan.params.upd_tile = t
            plan.params.upd_planes = z
            plan.update(x, xo, 0)
            up_ms[(t, z)] = _time(lambda: [plan.update(x, xo, 0) for _ in range(M)], reps)
    best_k, best_st = min(fp_ms, key=fp_ms.get)
    best_t, best_z = choose_update(up_ms)
    plan.params.fp_batch = best_k
    plan.params.fp_stage = best_st
    plan.params.upd_planes = best_z
    plan.params.upd_tile = best_t
    rec = {"fp_batch": best_k, "fp_stage": best_st, "upd_planes": best_z, "upd_tile": best_t,
           "fp_ms": {f"{k}{'-tma' if st else ''}": v for (k, st), v in fp_ms.items()},
           "update_ms": {f"{z}{TILE_NAMES[t]}": v for (t, z), v in up_ms.items()}}
    if use_cache:
        _store(key, rec)
    return best_k, best_z, rec
