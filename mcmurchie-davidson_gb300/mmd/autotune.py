"""Autotuner of the Fock-build launch schedule.

Tunables (C ABI ``mmdg_set_tuning`` / ``mmdg_set_streams``):

* per angular class, the persistent grid of its evaluation kernel: one full wave at
  the kernel's occupancy (0), or k blocks per SM for k in {1, 2, 4} -- small grids
  pack the tail of small classes, full waves hide latency in large ones;
* the number of concurrent streams the 21 classes (screening and evaluation) are
  spread over (1, 2, 4, 8): one class at a time leaves the GPU idle in the small
  classes and in every kernel's tail;
* with several streams, one grid size for all classes, timed as whole builds;
* per angular class, the tile of its evaluation kernel (``mmdg_set_tile``): threads
  per block {64, 128, 256} of the one-thread-per-quartet kernels (classes whose
  Hermite tables live in shared memory keep 128), quartets per warp work item
  {1, 2, 4, 8} of the warp-cooperative high-L kernels (whose Boys functions are
  evaluated together).

Each candidate is timed with CUDA events on a representative density difference
(``mmdg_fock_timed`` per class for the per-class grids, whole builds otherwise).
Results are cached as JSON under ``_build/tuning.json`` keyed by the GPU name, the
basis signature (molecules, functions, shells) and the FP32 threshold.
"""
from __future__ import annotations

import json
import os
import time

import numpy as np

from . import _native

CACHE = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "_build", "tuning.json")


BLOCKS = (64, 128, 256)   # threads per block, one-thread-per-quartet kernels
ITEMS = (1, 2, 4, 8)      # quartets per warp work item, warp-cooperative kernels


class Tuning:
    """A launch schedule: per-class persistent grid (0 = one full wave), per-class tile
    (threads per block or quartets per warp item; 0 = default) and the number of
    concurrent class streams."""

    def __init__(self, grids=None, streams=1, measured=None, tiles=None):
        self.grids = list(grids) if grids is not None else [0] * _native.NCLASS
        self.tiles = list(tiles) if tiles is not None else [0] * _native.NCLASS
        self.streams = int(streams)
        self.measured = measured or {}

    def apply(self, ctx):
        from .flop_model import CLASSES, fock_kernel
        for c, g in enumerate(self.grids):
            _native.check(_native.lib().mmdg_set_tuning(ctx._h, c, int(g)), "mmdg_set_tuning")
            warp = fock_kernel(CLASSES[c]) == "warp"
            t = int(self.tiles[c])
            _native.check(_native.lib().mmdg_set_tile(ctx._h, c, 0 if warp else t, t if warp else 0),
                          "mmdg_set_tile")
        _native.check(_native.lib().mmdg_set_streams(ctx._h, self.streams), "mmdg_set_streams")

    def to_json(self):
        return {"grids": self.grids, "tiles": self.tiles, "streams": self.streams, "measured": self.measured}


def _key(ctx, fp32_below=0.0):
    torch = ctx.torch
    name = torch.cuda.get_device_name(ctx.device)
    return f"{name}|nmol={ctx.nmol}|nfunc={int(np.sum(ctx.nfunc))}|nshell={ctx.nshell}|fp32_below={float(fp32_below):g}"


def _load_cache():
    try:
        with open(CACHE) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _store_cache(key, tun):
    """Adds one entry; the file is replaced atomically (concurrent tuners may lose an
    entry, never corrupt the file)."""
    os.makedirs(os.path.dirname(CACHE), exist_ok=True)
    cache = _load_cache()
    cache[key] = tun.to_json()
    tmp = f"{CACHE}.{os.getpid()}.tmp"
    with open(tmp, "w") as f:
        json.dump(cache, f, indent=1)
    os.replace(tmp, CACHE)


def _time_build(ctx, dP, tol, split, reps):
    torch = ctx.torch
    G = torch.empty_like(dP)
    ctx.fock(dP, G, tol=tol, fp32_below=split)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(reps):
        ctx.fock(dP, G, tol=tol, fp32_below=split)
    torch.cuda.synchronize()
    return (time.perf_counter() - t0) / reps


def autotune(ctx, dP, tol=1e-12, fp32_below=0.0, reps=3, use_cache=True) -> Tuning:
    """Times the candidate schedules on the density difference ``dP`` and applies the
    fastest to ``ctx`` (cached per GPU, basis signature and FP32 threshold)."""
    key = _key(ctx, fp32_below)
    if use_cache:
        t = _load_cache().get(key)
        if t is not None:
            tun = Tuning(t["grids"], t["streams"], t.get("measured"), t.get("tiles"))
            tun.apply(ctx)
            return tun
    torch = ctx.torch
    sms = torch.cuda.get_device_properties(ctx.device).multi_processor_count
    candidates = [0, sms, 2 * sms, 4 * sms]
    best = np.full(_native.NCLASS, np.inf)
    grids = [0] * _native.NCLASS
    per = {}
    for g in candidates:
        Tuning([g] * _native.NCLASS, 1).apply(ctx)
        ctx.fock_timed(dP, tol=tol, fp32_below=fp32_below)  # warm
        acc = np.zeros(_native.NCLASS)
        for _ in range(reps):
            _, ms, _ = ctx.fock_timed(dP, tol=tol, fp32_below=fp32_below)
            acc += ms
        acc /= reps
        per[str(g)] = acc.tolist()
        for c in range(_native.NCLASS):
            if acc[c] < best[c] * 0.98:  # prefer the default unless clearly better
                best[c] = acc[c]
                grids[c] = g
    # tiles, one class at a time on one stream (with the grids chosen above)
    from .flop_model import CLASSES, fock_kernel
    warp = np.array([fock_kernel(c) == "warp" for c in CLASSES])
    tiles = [0] * _native.NCLASS
    best_tile = best.copy()
    tile_ms = {}
    for k in range(len(ITEMS)):
        cand = [ITEMS[k] if w else (BLOCKS[k] if k < len(BLOCKS) else 0) for w in warp]
        Tuning(grids, 1, tiles=cand).apply(ctx)
        ctx.fock_timed(dP, tol=tol, fp32_below=fp32_below)  # warm
        acc = np.zeros(_native.NCLASS)
        for _ in range(reps):
            _, ms, _ = ctx.fock_timed(dP, tol=tol, fp32_below=fp32_below)
            acc += ms
        acc /= reps
        tile_ms[str(k)] = {"tiles": cand, "class_ms": acc.tolist()}
        for c in range(_native.NCLASS):
            if cand[c] and acc[c] < best_tile[c] * 0.98:
                best_tile[c] = acc[c]
                tiles[c] = cand[c]
    stream_ms = {}
    best_s, best_t = 1, np.inf
    for s in (1, 2, 4, 8):
        Tuning(grids, s, tiles=tiles).apply(ctx)
        t = _time_build(ctx, dP, tol, fp32_below, reps)
        stream_ms[str(s)] = t * 1e3
        if t < best_t * 0.98:
            best_s, best_t = s, t
    # with several streams the classes share the GPU: one grid size for every class,
    # timed as whole builds, may beat the per-class choice made one class at a time
    grid_ms = {}
    if best_s > 1:
        for g in candidates:
            Tuning([g] * _native.NCLASS, best_s, tiles=tiles).apply(ctx)
            t = _time_build(ctx, dP, tol, fp32_below, reps)
            grid_ms[str(g)] = t * 1e3
            if t < best_t * 0.98:
                grids, best_t = [g] * _native.NCLASS, t
    tun = Tuning(grids, best_s, {"class_ms_by_grid": per, "class_ms_by_tile": tile_ms,
                                 "build_ms_by_streams": stream_ms,
                                 "build_ms_by_grid_with_streams": grid_ms}, tiles=tiles)
    tun.apply(ctx)
    if use_cache:
        _store_cache(key, tun)
    return tun
