"""Launch-shape autotuner: the candidate set, the cache, and (GPU) a tuning pass that measures every
candidate on a real substep, applies the fastest, and is served from the cache (in memory and from
its JSON file) for a second world of the same shape."""
import json

import pytest
import torch

from difftactile_gb300 import autotune as AT


def test_candidates_cover_the_shapes():
    c = AT.candidates()
    assert len(c) == 2 * 2 * (3 * 3 * 2 + 2 * 3 * 2 + 2)
    assert {x["lanes"] for x in c} == {8, 4}
    assert {x["ppt"] for x in c} == {1, 2}
    assert {x["p_block"] for x in c if x["scatter"] == "tile"} == {128}
    assert {(x["scatter"], x["p_block"]) for x in c if x["scatter"] != "tile"} == \
        {(s, b) for s in ("warp", "smem", "global") for b in (64, 128, 256)}
    assert {x["depth"] for x in c if x["scatter"] == "warp"} == {0, 1, 2}
    assert {x["depth"] for x in c if x["scatter"] != "warp"} == {0}
    assert len({AT.label(x) for x in c}) == len(c)
    assert AT.label(AT.DEFAULT) in {AT.label(x) for x in c}


def test_cache_file_round_trip(tmp_path):
    path = str(tmp_path / "tune.json")
    entry = {"best": {"scatter": "warp", "p_block": 64, "pdl": 1}, "ms": {"warp/64/pdl": 0.1}}
    AT._store(path, "k1", entry)
    AT._store(path, "k2", dict(entry, best={"scatter": "tile", "p_block": 128, "pdl": 0}))
    data = json.load(open(path))
    assert data["k1"] == entry and data["k2"]["best"]["scatter"] == "tile"
    assert AT._load(str(tmp_path / "missing.json")) == {}


@pytest.mark.gpu
def test_tune_substep_applies_and_caches(cuda_lib, tmp_path):
    from difftactile_gb300.world import World
    from tests import small_scenes as SS

    env = SS.pad_over_box()
    path = str(tmp_path / "tune.json")
    pdl0 = cuda_lib.dt_get_pdl()
    try:
        w = World([env], n_frames=3, dt=1e-4)
        w.step_begin()
        w.substep(0)
        w.substep(1)
        AT._cache.clear()
        r = AT.tune_substep(w, frame=1, reps=3, warmup=1, cache_path=path)
        n = len(AT.candidates())
        assert not r["cached"] and len(r["ms"]) in (n, n + 2)  # + the warp winner's two other adjoint depths
        assert all(0.0 < v < 1e3 for v in r["ms"].values())
        fastest = min(r["ms"], key=r["ms"].get)
        # the default is kept unless the fastest beats it by more than the 2% margin
        assert AT.label(r["best"]) == fastest or (AT.label(r["best"]) == AT.label(AT.DEFAULT) and
                                                  r["ms"][fastest] > 0.98 * r["ms"][AT.label(AT.DEFAULT)])
        assert AT.current(w) == r["best"]
        torch.cuda.synchronize()
        assert w.error_word() == 0

        w2 = World([env], n_frames=3, dt=1e-4)
        r2 = AT.tune_substep(w2, frame=1, cache_path=path)
        assert r2["cached"] and AT.current(w2) == r["best"]
        AT._cache.clear()  # the JSON file serves it too
        r3 = AT.tune_substep(w2, frame=1, cache_path=path)
        assert r3["cached"] and r3["best"] == r["best"]
    finally:
        cuda_lib.dt_set_pdl(pdl0)
        AT._cache.clear()


class _FakeLib:
    def __init__(self):
        self.pdl = 1

    def dt_set_pdl(self, on):
        old, self.pdl = self.pdl, int(on)
        return old

    def dt_get_pdl(self):
        return self.pdl


class _FakeWorld:
    """The fields the tuner sets, without a device: the 'time' of a shape is a fixed function of it."""
    def __init__(self, n_particles=1000):
        import types
        self.w = types.SimpleNamespace(scatter_mode=2, p_block=128, scatter_depth=0, contact_lanes=8, p_per_thread=1,
                                       scatter_depth_adj=0)
        self.lib = _FakeLib()
        self.device = "cpu"
        self.n_envs, self.n_particles, self.n_verts, self.n_tets, self.n_tris = 1, n_particles, 10, 10, 10
        self.n_blocks, self.n_rope_particles = 100, 0

    def error_word(self):
        return 0


def _timer_for(costs):
    def timer(run, reps, warmup):
        run()
        return costs(run.world)
    return timer


def test_tuner_picks_the_fastest_shape_and_keeps_the_default_within_the_margin():
    AT._cache.clear()
    world = _FakeWorld()

    def run():
        pass
    run.world = world
    cur = lambda w: AT.current(w)  # noqa: E731
    # a shape 10% faster than the default wins
    fast = {"scatter": "warp", "p_block": 256, "depth": 1, "lanes": 4, "pdl": 1, "ppt": 2}
    cost = lambda w: 0.9 if cur(w) == fast else 1.0  # noqa: E731
    r = AT.tune(world, run, timer=_timer_for(cost), use_cache=False)
    assert r["best"] == fast and AT.current(world) == fast and not r["cached"]
    # a shape only 1% faster does not displace the default
    cost2 = lambda w: 0.99 if cur(w) == fast else 1.0  # noqa: E731
    r2 = AT.tune(world, run, timer=_timer_for(cost2), use_cache=False)
    assert r2["best"] == AT.DEFAULT and AT.current(world) == AT.DEFAULT
    # the result is cached per world shape; a different shape is tuned afresh
    r3 = AT.tune(world, run, timer=_timer_for(cost), tag="t")
    r4 = AT.tune(world, run, timer=lambda *a: 1 / 0, tag="t")  # served from the cache, no timing
    assert r4["cached"] and r4["best"] == r3["best"] == fast
    other = _FakeWorld(n_particles=2000)
    run.world = other
    r5 = AT.tune(other, run, timer=_timer_for(cost2), tag="t")
    assert not r5["cached"]
    AT._cache.clear()


def test_tuner_refines_the_adjoint_depth_of_the_fastest_shape():
    """After the search, the fastest warp shape is timed with the G2P adjoint at each other depth; a
    faster variant wins and is applied (dt_world.scatter_depth_adj 3 for whole runs, else the depth),
    and the field reads back through current()."""
    AT._cache.clear()
    world = _FakeWorld()

    def run():
        pass
    run.world = world
    fast = {"scatter": "warp", "p_block": 64, "depth": 1, "lanes": 4, "pdl": 0, "ppt": 2}
    for adj, code in ((2, 2), (0, 3)):
        def cost(w, adj=adj):
            c = AT.current(w)
            base = {k: v for k, v in c.items() if k != "adj_depth"}
            if base != fast:
                return 1.0
            return 0.8 if c.get("adj_depth") == adj else 0.9
        r = AT.tune(world, run, timer=_timer_for(cost), use_cache=False, refine=AT.adjoint_depths)
        assert r["best"] == dict(fast, adj_depth=adj) and world.w.scatter_depth_adj == code
        assert AT.current(world) == r["best"]
        assert len(r["ms"]) == len(AT.candidates()) + 2
    # a variant no faster leaves the adjoint on the P2G's depth
    cost = lambda w: 0.9 if {k: v for k, v in AT.current(w).items() if k != "adj_depth"} == fast else 1.0  # noqa: E731
    r = AT.tune(world, run, timer=_timer_for(cost), use_cache=False, refine=AT.adjoint_depths)
    assert r["best"] == fast and world.w.scatter_depth_adj == 0 and "adj_depth" not in AT.current(world)
    assert AT.adjoint_depths(dict(fast, scatter="global")) == []
    AT._cache.clear()
