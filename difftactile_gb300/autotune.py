"""Launch-shape autotuner for a World.

The substep's particle-role launches can be shaped three ways, and which is fastest depends on the
scene (particle count and density, how many environments share the launch):
  scatter   how P2G and the G2P adjoint accumulate into the grid (dt_world.scatter_mode): a warp
            segmented reduction before one RED per run and node ("warp"), whole-run sums added into a
            shared-memory tile of the CTA's nodes flushed with one RED per node ("smem"), one RED per
            particle and node ("global"), or a shared-memory gather tile per CTA ("tile", 128 threads
            only);
  p_block   threads per CTA of the particle / tet / vertex launches (dt_world.p_block): 64, 128, 256;
  depth     with the warp scatter, the shuffle steps of the segmented reduction before the REDs
            (dt_world.scatter_depth): 0 sums whole runs (fewest REDs, longest shuffle chain), 1 or 2
            sum windows of 2 or 4 lanes (more REDs, fewer shuffles: faster when the launch is
            throughput-bound, slower when it is latency-bound);
  lanes     lanes per active grid node in the contact search (dt_world.contact_lanes): 8 shortens
            each node's dependent chain (latency-bound launches), 4 issues fewer instructions per node
            (throughput-bound launches);
  ppt       particles per thread of the particle-role launches (dt_world.p_per_thread): each CTA
            takes 1 or 2 consecutive chunks of p_block particles (fewer, longer-lived CTAs; the second
            chunk finds the first one's grid neighbourhood in L1);
  adj_depth with the warp scatter, the G2P adjoint's own depth (dt_world.scatter_depth_adj; absent:
            the P2G's): tried after the search, on the fastest shape, with the other depths;
  pdl       programmatic dependent launch of the substep kernels (dt_set_pdl, library-wide).

``tune_substep`` times every candidate on one forward + backward substep of the world at a chosen
frame (CUDA events on the launching stream, median of ``reps`` after ``warmup``), then the fastest
one's variants with another adjoint depth, and applies the fastest; ``tune`` does the same for any callable (e.g. a whole rollout).  Results are kept per
device and world shape, in memory and optionally in a JSON file, so a second world of the same
shape skips the measurement.  Recorded CUDA graphs hold the launch shape they were recorded with:
re-record them (Trajectory.reset_graphs) after tuning.
"""
from __future__ import annotations

import json
import os
import statistics

import torch

SCATTERS = {"tile": 0, "global": 1, "warp": 2, "smem": 3}
DEFAULT = {"scatter": "warp", "p_block": 128, "depth": 0, "lanes": 8, "pdl": 1, "ppt": 1}

_cache: dict[str, dict] = {}


def candidates(scatters=("warp", "smem", "global", "tile"), p_blocks=(64, 128, 256), depths=(0, 1, 2), lanes=(8, 4),
               pdl=(1, 0), ppts=(1, 2)):
    out = []
    for s in scatters:
        for b in (p_blocks if s != "tile" else (128,)):
            for d in (depths if s == "warp" else (0,)):
                for ln in lanes:
                    for p in pdl:
                        for k in ppts:
                            out.append({"scatter": s, "p_block": int(b), "depth": int(d), "lanes": int(ln),
                                        "pdl": int(p), "ppt": int(k)})
    return out


# dt_world.scatter_depth_adj of an adjoint depth (0: whole runs) and back; 0 in the field: the P2G's depth
_ADJ_CODE = {0: 3, 1: 1, 2: 2}
_ADJ_DEPTH = {v: k for k, v in _ADJ_CODE.items()}


def apply(world, cfg: dict):
    """Set ``cfg`` (scatter, p_block, depth, lanes, ppt, adj_depth, pdl) on ``world`` (and the
    library's PDL switch)."""
    world.w.scatter_mode = SCATTERS[cfg["scatter"]]
    world.w.p_block = int(cfg["p_block"])
    world.w.scatter_depth = int(cfg.get("depth", 0))
    world.w.contact_lanes = int(cfg.get("lanes", 8))
    world.w.p_per_thread = int(cfg.get("ppt", 1))
    adj = cfg.get("adj_depth")
    world.w.scatter_depth_adj = _ADJ_CODE[int(adj)] if adj is not None else 0
    world.lib.dt_set_pdl(int(cfg["pdl"]))  # returns the previous setting


def current(world) -> dict:
    inv = {v: k for k, v in SCATTERS.items()}
    out = {"scatter": inv.get(int(world.w.scatter_mode), "warp"), "p_block": int(world.w.p_block) or 128,
           "depth": int(world.w.scatter_depth), "lanes": 4 if int(world.w.contact_lanes) == 4 else 8,
           "pdl": int(world.lib.dt_get_pdl()), "ppt": max(1, int(world.w.p_per_thread))}
    adj = _ADJ_DEPTH.get(int(getattr(world.w, "scatter_depth_adj", 0)))
    if adj is not None:
        out["adj_depth"] = adj
    return out


def adjoint_depths(best: dict) -> list[dict]:
    """The variants of a warp-scatter shape whose G2P adjoint takes each other depth."""
    if best["scatter"] != "warp":
        return []
    return [dict(best, adj_depth=d) for d in (0, 1, 2) if d != int(best.get("depth", 0))]


def signature(world, tag: str = "") -> str:
    name = torch.cuda.get_device_name(world.device) if torch.cuda.is_available() else "no-device"
    return "|".join(str(x) for x in (name, tag, world.n_envs, world.n_particles, world.n_verts, world.n_tets,
                                     world.n_tris, world.n_blocks, world.n_rope_particles))


def _load(path):
    if path and os.path.exists(path):
        with open(path) as fh:
            return json.load(fh)
    return {}


def _store(path, key, entry):
    if not path:
        return
    data = _load(path)
    data[key] = entry
    tmp = path + ".tmp"
    with open(tmp, "w") as fh:
        json.dump(data, fh, indent=1, sort_keys=True)
    os.replace(tmp, path)


def _time(run, reps, warmup):
    for _ in range(warmup):
        run()
    ts = []
    for _ in range(reps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        run()
        e1.record()
        e1.synchronize()
        ts.append(e0.elapsed_time(e1))
    return statistics.median(ts)


def tune(world, run, cands=None, reps: int = 5, warmup: int = 1, tag: str = "", cache_path: str | None = None,
         use_cache: bool = True, prepare=None, margin: float = 0.02, timer=None, refine=None) -> dict:
    """Time ``run()`` under every candidate launch shape (``prepare()``, untimed, before each
    candidate's runs), then under ``refine(fastest)`` (variants of the fastest shape), apply the
    fastest and return {"best": cfg, "ms": {label: median ms}, "cached": bool}.
    The library default (``DEFAULT``) is kept unless a candidate beats it by more than ``margin``
    (relative), so that timing noise between near-equal shapes does not flip the choice.  ``timer``
    replaces the CUDA-event timing (called as timer(run, reps, warmup) -> ms)."""
    key = signature(world, tag)
    if use_cache:
        hit = _cache.get(key) or _load(cache_path).get(key)
        if hit is not None:
            apply(world, hit["best"])
            _cache[key] = hit
            return dict(hit, cached=True)
    cands = cands or candidates()
    times = {}
    best, best_ms = None, float("inf")

    def measure(c):
        apply(world, c)
        if prepare is not None:
            prepare()
        ms = (timer or _time)(run, reps, warmup)
        if world.error_word():
            raise RuntimeError(f"device error word {world.error_word()} while tuning {c}")
        times[label(c)] = ms
        return ms

    for c in cands:
        ms = measure(c)
        if ms < best_ms:
            best, best_ms = c, ms
    for c in (refine(best) if refine is not None else []):
        ms = measure(c)
        if ms < best_ms:
            best, best_ms = c, ms
    d_ms = times.get(label(DEFAULT))
    if d_ms is not None and best_ms > (1.0 - margin) * d_ms:
        best = dict(DEFAULT)
    apply(world, best)
    entry = {"best": best, "ms": times}
    _cache[key] = entry
    _store(cache_path, key, entry)
    return dict(entry, cached=False)


def tune_substep(world, frame: int = 0, **kw) -> dict:
    """Tune on one forward substep ``frame`` -> ``frame`` + 1 and its adjoint.  The frame's state
    must be valid (e.g. after a rollout); frame + 1, the grid tape of ``frame``, the tape counters
    of every frame and the adjoint buffers are overwritten."""
    if not 0 <= frame < world.n_frames - 1:
        raise ValueError(f"frame {frame} outside [0, {world.n_frames - 1})")

    def run():  # the adjoint buffers are cleared once per candidate; repeated sweeps only accumulate
        world.step_begin()
        world.substep(frame)
        world.substeps_bwd(frame + 1, frame)

    kw.setdefault("prepare", world.adj_clear)
    kw.setdefault("refine", adjoint_depths)
    kw.setdefault("tag", "substep")
    kw.setdefault("reps", 15)
    kw.setdefault("warmup", 2)
    return tune(world, run, **kw)


def label(c: dict) -> str:
    depth = f"/d{c.get('depth', 0)}" if c["scatter"] == "warp" else ""
    ppt = f"/ppt{c['ppt']}" if c.get("ppt", 1) != 1 else ""
    adj = f"/a{c['adj_depth']}" if c["scatter"] == "warp" and c.get("adj_depth") is not None else ""
    return f"{c['scatter']}/{c['p_block']}{depth}/l{c.get('lanes', 8)}/{'pdl' if c['pdl'] else 'nopdl'}{ppt}{adj}"
