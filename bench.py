"""Benchmark: forward+backward particle-substeps/s of the differentiable DiffTactile substep on one
GB300, batched against the plain one-scene-per-launch path (replicas on N GPUs under torchrun).

Default workload: the batched population (64 independent environments of 8k-128k particles on
48^3-128^3 grids, one 20x20x5 FEM pad each, 200 control steps x 20 substeps, checkpoint at every step
start and recompute of each step's substep tape in the backward sweep).  One bench step = one training
iteration of all environments at once: the forward rollout, the marker loss, the backward sweep down
to the action gradients.  The unit counts each particle advanced one substep forward and
back-propagated once: n_particles x 200 x 20 per bench step.

Before timing, the autotuner picks the launch shape on a mid-rollout substep and the rollout is
recorded as CUDA graphs (the timed iterations replay them).  The line carries:
  plain / batched_over_plain  a sample of the environments, each in a World of its own, launched
                              one after the other (tuned and graphed the same way);
  roofline                    the dominant kernel's algorithmic bytes over its CUDA-event duration
                              (events around every 25th of its launches inside the timed region);
  e2e                         the same metric through the public API with host buffers;
  grad_check                  one adjoint substep of environment 0 at mid-rollout, seeded by the
                              real loss's adjoint, against the float64 oracle (on the branch of the
                              von Mises return map the forward took, and free);
  cpu_baseline                the oracle on the host cores (1 thread and all threads) from the same
                              mid-rollout state;
  sensor_press                configuration 2 (64,000 particles, 100 x 20, full tape), nested.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--config NAME]
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

FALLBACK_HBM_GBS = 6800.0
PROBE_EVERY = 25  # substeps between the timed region's event-timed launches of the dominant kernel
METRIC, UNIT = "fwd+bwd particle-substeps/s", "particle-substeps/s"  # both arms report these


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", default="batched_population", choices=["batched_population", "sensor_press",
                                                                        "rope_pads"])
    ap.add_argument("--horizon", type=int, default=None, help="control steps (default: the config's)")
    ap.add_argument("--envs", type=int, default=None, help="batched_population: the first N environments only")
    ap.add_argument("--plain", type=int, default=8,
                    help="batched_population: time K environments (evenly spaced over the population) one "
                    "World each, one after the other, and report the batched / plain ratio (0: skip)")
    ap.add_argument("--scatter", default=None, choices=["tile", "global", "warp", "smem"],
                    help="27-node scatter strategy (default: the library's)")
    ap.add_argument("--no-pdl", action="store_true", help="launch the substep kernels without programmatic "
                    "dependent launch")
    ap.add_argument("--p-block", type=int, default=None, choices=[64, 128, 256],
                    help="threads per CTA of the particle launches")
    ap.add_argument("--depth", type=int, default=None, choices=[0, 1, 2, 3, 4, 5],
                    help="shuffle steps of the warp scatter's segmented reduction (0: whole runs)")
    ap.add_argument("--adj-depth", type=int, default=None, choices=[0, 1, 2],
                    help="shuffle steps of the G2P adjoint's warp scatter (0: whole runs; default: the P2G's)")
    ap.add_argument("--ppt", type=int, default=None, choices=[1, 2],
                    help="particles per thread of the particle-role launches (default: the tuner's choice)")
    ap.add_argument("--lanes", type=int, default=None, choices=[4, 8],
                    help="lanes per active grid node in the contact search")
    ap.add_argument("--no-tune", action="store_true", help="keep the library's default launch shape instead of "
                    "the autotuner's choice (also implied by --scatter, --no-pdl, --p-block, --depth, --adj-depth, "
                    "--ppt or --lanes)")
    ap.add_argument("--no-svd-tape", action="store_true", help="the adjoint recomputes the SVD instead of "
                    "reading the forward's from the tape")
    ap.add_argument("--no-graph", action="store_true", help="launch every substep from the host instead of "
                    "replaying the rollout's recorded CUDA graphs")
    ap.add_argument("--rebin", type=int, default=1,
                    help="checkpointed rollouts: sort the particles by cell again at every N-th checkpoint (0: never)")
    ap.add_argument("--readouts", action="store_true",
                    help="run every readout / action / deform-loss entry point once (for a profiler) and exit")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline and the gradient check")
    ap.add_argument("--no-nested", action="store_true", help="skip the nested sensor-press measurement")
    return ap.parse_args()


def make_config(name, horizon, envs=None):
    from difftactile_gb300 import configs
    if name == "sensor_press":
        return configs.sensor_press(n_steps=horizon or 100)
    if name == "rope_pads":
        return configs.rope_pads(n_steps=horizon or 500, n_envs=envs or 16)
    return configs.batched_population(n_steps=horizon or 200, n_envs=envs or 64)


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


class Clocks:
    """nvidia-smi sampling during the timed region (clocks, throttle reasons)."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--id={gpu_index}", f"--query-gpu={self.Q}",
                                       "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                                      stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None

    def stop(self):
        if self.p is None:
            return None
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except Exception:
            self.p.kill()
        self.f.seek(0)
        rows = [r.split(",") for r in self.f.read().strip().splitlines() if r.strip()]
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].strip().replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].strip().replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({n for r in rows for n, v in zip(names, r[5:9]) if v.strip().lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


# algorithmic bytes per unit of each fused launch (compulsory reads and writes of the launch's state;
# the SVD tape the forward writes for the adjoint, 96 B per particle, is this design's choice and is not
# counted)
BYTES = {
    ("fwd", 0): {"particle": 96 + 36, "node": 16, "tet": 148, "tri": 68},
    ("fwd", 1): {"node": 96},
    ("fwd", 2): {"particle": 16 + 60, "node": 16, "vert": 176},
    ("bwd", 0): {"node": 32},
    ("bwd", 1): {"particle": 16 + 64 + 16, "node": 32, "vert": 128},
    ("bwd", 2): {"node": 80},
    ("bwd", 3): {"particle": 96 + 48 + 96, "node": 16, "tet": 196, "vert": 32},
}
NAMES = {("fwd", 0): "k_fwd_p2g_fem", ("fwd", 1): "k_fwd_grid", ("fwd", 2): "k_fwd_g2p_fem",
         ("bwd", 0): "k_bwd_restore", ("bwd", 1): "k_bwd_g2p_fem", ("bwd", 2): "k_bwd_grid",
         ("bwd", 3): "k_bwd_p2g_fem"}

# DRAM traffic (dram__bytes_read.sum + dram__bytes_write.sum) per launch, from one ncu capture of the
# 16-environment population (the first 16 environments, 843,880 particles; ncu --set full, the sixth
# launch of each kernel, --clock-control none; the forward P2G's is a launch of the first, untaped
# forward pass) scaled to the full population by its particle count (3,221,208 / 843,880): a static
# capture, not a live measurement, valid for the kernel build it was taken of
NCU_TRAFFIC = {"captured_at": "the build of commit aa5e952 (re-binning, two particles per thread, tet SVD tape, four-block grid "
                              "steps, per-axis stencil node indices); the G2P adjoint's with 4-lane scatter windows, "
                              "ABI 8",
               "per_launch_bytes": {k: b * 3.817 for k, b in (
                   ("k_fwd_p2g_fem", 130.55e6), ("k_fwd_grid", 4.65e6), ("k_fwd_g2p_fem", 31.89e6),
                   ("k_bwd_restore", 3.92e6), ("k_bwd_g2p_fem", 85.5e6), ("k_bwd_grid", 12.11e6),
                   ("k_bwd_p2g_fem", 335.46e6))}}


def algo_bytes(key, units):
    return sum(b * units.get(u, 0) for u, b in BYTES[key].items())


# ------------------------------------------------------------------------------------------------
# the GPU arm
# ------------------------------------------------------------------------------------------------
def build(cfg, dev, args, **extra):
    kw = dict(extra)
    if args.scatter is not None:
        kw["scatter_mode"] = {"tile": 0, "global": 1, "warp": 2, "smem": 3}[args.scatter]
    if args.no_svd_tape:
        kw["svd_tape"] = False
    if args.p_block is not None:
        kw["p_block"] = args.p_block
    if args.depth is not None:
        kw["scatter_depth"] = args.depth
    if args.lanes is not None:
        kw["contact_lanes"] = args.lanes
    if args.ppt is not None:
        kw["p_per_thread"] = args.ppt
    if args.adj_depth is not None:
        kw["scatter_depth_adj"] = 3 if args.adj_depth == 0 else args.adj_depth
    if args.rebin and cfg.ckpt_every > 0:
        kw["rebin_every"] = args.rebin
    return cfg.build(dev, **kw)


def tune_launch(args):
    return not (args.no_tune or args.scatter or args.no_pdl or args.p_block or args.depth is not None
                or args.lanes is not None or args.ppt is not None or args.adj_depth is not None)


def mid_frame(traj):
    return traj.f_end // 2 if traj.full else traj.S // 2


def measure(cfg, w, traj, args, dev, flush, steps, warmup, barrier, tuned_ok=True):
    """Tune, break the substep down per launch, warm up (recording the graphs), then time ``steps``
    iterations with the dominant launch probed.  Returns (result dict, acts)."""
    import torch

    from difftactile_gb300 import autotune

    w.lib.dt_set_pdl(0 if args.no_pdl else 1)
    acts = torch.as_tensor(cfg.actions, dtype=torch.float64, device=dev)

    def iteration():
        traj.forward(acts)
        return traj.backward()

    iteration()  # untimed: a valid mid-rollout frame for the tuner and the breakdown
    torch.cuda.synchronize()
    f_mid = mid_frame(traj)
    tuned = None
    if tuned_ok and tune_launch(args):
        tuned = autotune.tune_substep(w, frame=f_mid)
        tuned["frame"] = f_mid
        iteration()  # the tuner overwrote frame f_mid + 1 and the adjoint buffers
        torch.cuda.synchronize()
    # per-launch breakdown on a replay of the mid-rollout substep; a checkpointed rollout runs each
    # forward launch twice per substep (forward, then the recompute of the backward sweep)
    bd = w.stage_breakdown(f_mid)
    fwd_runs = 1 if traj.full else 2
    share_w = {k: v * (fwd_runs if k[0] == "fwd" else 1) for k, v in bd.items()}
    tot = sum(share_w.values())
    dom = max(share_w, key=share_w.get)

    w.set_probe(*dom, every=PROBE_EVERY)
    traj.graph = not args.no_graph
    traj.reset_graphs()
    for _ in range(max(warmup, 0)):
        iteration()
    torch.cuda.synchronize()
    if w.error_word():
        raise RuntimeError(f"device error word {w.error_word()} during warm-up")
    clocks = Clocks(dev.index or 0)
    traj.launches = 0
    times, dom_acc = [], []
    w.probe_events.clear()  # host-recorded pairs of the warm-up; graph-recorded pairs are re-recorded
    for _ in range(steps):
        flush.zero_()  # L2 flush between timed iterations (256 MiB > 129 MB L2)
        torch.cuda.synchronize()
        barrier()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        g = iteration()
        e1.record()
        torch.cuda.synchronize()
        barrier()
        times.append(e0.elapsed_time(e1))
        dom_acc.append(w.probe_ms())  # this iteration's launches of the dominant kernel
        if not traj.graph:
            w.probe_events.clear()
    clk = clocks.stop()
    if w.error_word():
        raise RuntimeError(f"device error word {w.error_word()} in the timed region")
    dom_n = sum(n for _, n in dom_acc)
    dom_ms = sum(m * n for m, n in dom_acc) / max(dom_n, 1)
    w.set_probe(None)
    traj.reset_graphs()
    ms = sum(times) / len(times)
    # roofline of the dominant launch: algorithmic bytes of one launch over its event-timed duration
    used = w.t["tape_bcount"][: traj.f_end]
    cnt = used.clamp(max=w.tape_blocks).double().mean().item()
    units = {"particle": w.n_particles, "node": 64 * cnt, "tet": w.n_tets, "tri": w.n_tris, "vert": w.n_verts}
    ab = algo_bytes(dom, units)
    achieved = ab / (dom_ms / 1e3) / 1e9
    peak, peak_kind = peaks()
    res = {"ms": ms, "times_ms": times, "loss": float(traj.loss.item()), "grad_norm": float(g.norm().item()),
           "launches_per_iter": traj.launches // max(steps, 1) + 2, "clocks": clk, "tuned": tuned,
           "active_blocks_mean": cnt, "active_blocks_max": int(used.max().item()),
           "breakdown": {NAMES[k]: {"ms_per_launch": v, "launches_per_substep": fwd_runs if k[0] == "fwd" else 1,
                                    "share": share_w[k] / tot, "algorithmic_GBps": algo_bytes(k, units) / v / 1e6}
                         for k, v in bd.items()},
           "roofline": {"kernel": NAMES[dom], "bound": "hbm", "achieved": achieved, "peak": peak,
                        "peak_kind": peak_kind, "unit": "GB/s", "frac": achieved / peak,
                        "algorithmic_bytes_per_launch": ab, "launch_ms": dom_ms, "launches_timed": dom_n,
                        "timed_every_nth_launch": PROBE_EVERY}}
    return res, acts


def end_to_end(cfg, w, traj, dev, flush, n, barrier):
    """The same iteration through the public API with host buffers: actions and initial particles copied
    in, the loss and the action gradients copied out, every iteration."""
    import numpy as np
    import torch

    h_act = torch.as_tensor(cfg.actions, dtype=torch.float32).pin_memory()
    xs = np.concatenate([e.x for e in cfg.envs], 0)
    h_x = torch.as_tensor(xs, dtype=torch.float32).pin_memory()
    h_v = torch.zeros_like(h_x).pin_memory()
    traj.graph = True
    out = []
    for i in range(n + 1):  # the first iteration records the graphs
        flush.zero_()
        torch.cuda.synchronize()
        barrier()
        t0 = time.perf_counter()
        d_act = h_act.to(dev, non_blocking=True)
        d_x = h_x.to(dev, non_blocking=True)
        d_v = h_v.to(dev, non_blocking=True)
        w.set_particles(0, x=d_x, v=d_v)
        loss = traj.forward(d_act.double())
        g = traj.backward()
        res = torch.cat([loss.double(), g.reshape(-1)]).cpu()
        t1 = time.perf_counter()
        if i > 0:
            out.append(t1 - t0)
    traj.reset_graphs()
    return {"ms": 1e3 * sum(out) / len(out), "iterations": len(out),
            "h2d_bytes_per_step": int(h_act.numel() * 4 + h_x.numel() * 4 + h_v.numel() * 4),
            "d2h_bytes_per_step": int(res.numel() * 8)}


def time_plain(cfg, args, dev, flush):
    """A sample of the environments, each in a World of its own (the one-scene-per-launch path), stepped
    one after the other with the same actions, tuned and graphed like the batched World; aggregate
    particle-substeps/s of the sample."""
    import numpy as np
    import torch

    from difftactile_gb300 import autotune
    from difftactile_gb300.configs import Config

    k = min(args.plain, len(cfg.envs))
    pick = sorted({int(round(i)) for i in np.linspace(0, len(cfg.envs) - 1, k)})
    total_ms, units, per = 0.0, 0, []
    for e in pick:
        sub = Config(cfg.name, [cfg.envs[e]], cfg.dt, cfg.substeps, cfg.n_steps, cfg.actions[:, e:e + 1],
                     tuple((0, lay, tg) for s, lay, tg in cfg.loss_terms if s == e), cfg.ckpt_every,
                     max(1024, 2 * cfg.envs[e].n_particles // 64))
        w, traj = build(sub, dev, args)
        acts = torch.as_tensor(sub.actions, dtype=torch.float64, device=dev)
        traj.forward(acts)
        traj.backward()
        if tune_launch(args):  # each single-environment World gets its own launch shape
            autotune.tune_substep(w, frame=mid_frame(traj))
        traj.graph = not args.no_graph
        for _ in range(2):
            traj.forward(acts)
            traj.backward()
        flush.zero_()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        traj.forward(acts)
        traj.backward()
        e1.record()
        torch.cuda.synchronize()
        if w.error_word():
            raise RuntimeError(f"device error word {w.error_word()} in the plain run of environment {e}")
        ms = e0.elapsed_time(e1)
        u = cfg.envs[e].n_particles * cfg.n_steps * cfg.substeps
        per.append({"env": e, "particles": cfg.envs[e].n_particles, "ms": ms, "value": u / (ms / 1e3)})
        total_ms += ms
        units += u
        del w, traj
        torch.cuda.empty_cache()
    return {"value": units / (total_ms / 1e3), "unit": UNIT, "envs": pick, "ms": total_ms,
            "sample_particles": sum(p["particles"] for p in per), "per_env": per,
            "path": "one World per environment (tuned, CUDA graphs), launched one after the other"}


# ------------------------------------------------------------------------------------------------
# mid-rollout state, gradient check and CPU baseline (oracle: test infrastructure, used as the checker)
# ------------------------------------------------------------------------------------------------
def mid_rollout(cfg, w, traj, acts):
    """Environment 0 at a mid-rollout substep, from one forward and the backward sweep of its real loss
    down to that substep: state of frame f (float64 of the float32 device values), the adjoint of frame
    f + 1, the frames' control velocities, the forward's yield branch per particle, and the CUDA
    adjoint of the substep."""
    import numpy as np
    import torch

    traj.graph = False
    traj.forward(acts)
    t_mid, f_loc = traj.T // 2, traj.S // 2
    f = traj.adjoint_at(t_mid, f_loc)
    torch.cuda.synchronize()
    n0 = cfg.envs[0].n_particles
    P = w.particles(f)
    st = {k: P[k][:n0].double().cpu().numpy() for k in ("x", "v", "C", "F")}
    sl = w.vslice(w.env_rows[0].s_begin)
    fem = lambda name, fr: w.t[name][fr, sl, :3].double().cpu().numpy()  # noqa: E731
    st["pos"], st["vel"], st["vpos"] = [fem("v_pos", f)], [fem("v_vel", f)], [fem("v_vpos", f)]
    A1 = w.particle_adjoint(f + 1)
    nb = (f + 1) & 1
    adj1 = {k: A1[k][:n0].double().cpu().numpy() for k in ("x", "v", "C", "F")}
    for key, name in (("pos", "v_adj_pos"), ("vel", "v_adj_vel"), ("vpos", "v_adj_vpos")):
        adj1[key] = [w.t[name][nb, sl, :3].double().cpu().numpy()]
    yb = w.yield_flags(f)[:n0].cpu().numpy() if w.t["p_svd"] is not None else None
    w.substep_bwd(f)
    torch.cuda.synchronize()
    A0 = w.particle_adjoint(f)
    g = {k: A0[k][:n0].double().cpu().numpy() for k in ("x", "v", "C", "F")}
    g["pos"] = w.t["v_adj_pos"][f & 1, sl, :3].double().cpu().numpy()
    return {"t": t_mid, "f": f_loc, "frame": f, "st": st, "adj1": adj1, "cv": [fem("v_cv", f)],
            "cv1": [fem("v_cv", f + 1)], "yield": yb, "g": g}


def grad_check(cfg, w, mid, threads):
    """The CUDA adjoint of one mid-rollout substep (environment 0, seeded by the real loss's adjoint)
    against the oracle's adjoint of the same substep from the same float32 state: in float64 on the
    branch of the von Mises return map that the CUDA forward took for each particle (both then
    differentiate the same piecewise-smooth function), in float64 with every branch decided by its
    own yield test, and in float32."""
    import numpy as np

    from oracle import oracle as O

    env = cfg.envs[0]
    n0 = env.n_particles
    rel = lambda a, b: float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))  # noqa: E731
    g = mid["g"]
    out = {"env": 0, "step": mid["t"], "substep": mid["f"], "particles": n0,
           "adjoint_seed": "the real loss's adjoint of frame f + 1 (backward sweep from the final marker loss)"}
    runs = {}
    yb = mid["yield"]
    variants = [("f64_branch_pinned", np.float64, yb), ("f64", np.float64, None), ("f32", np.float32, None)]
    for key, dtype, branch in variants:
        if key.endswith("pinned") and branch is None:
            continue
        o = O.Oracle(env, cfg.dt, dtype, n_threads=threads, grad_clip=float(w.w.grad_clip),
                     yield_branch=None if branch is None else branch.astype(np.int8))
        st = {k: (v.copy() if not isinstance(v, list) else [a.copy() for a in v]) for k, v in mid["st"].items()}
        ref = runs[key] = o.substep_bwd(st, mid["adj1"], cv=mid["cv"], cv1=mid["cv1"])
        errs = {k: rel(g[k], ref[k]) for k in ("x", "v", "C", "F")}
        errs["sensor_pos"] = rel(g["pos"], ref["pos"][0])
        out[key] = {"rel_err": errs, "max_rel_err": max(errs.values())}
    if yb is not None:
        m = env.materials[0]
        Fn = (np.eye(3)[None] + cfg.dt * mid["st"]["C"]) @ mid["st"]["F"]
        eps = np.log(np.maximum(np.linalg.svd(Fn, compute_uv=False), 0.05))
        dg = np.sqrt(((eps - eps.mean(1, keepdims=True)) ** 2).sum(1) + 1e-8) - m.yield_stress / (2.0 * m.mu_lam[0])
        out["yielding"] = int(yb.sum())
        out["branch_differs_from_f64_test"] = int(((dg > 0) != yb).sum())
    out["max_rel_err"] = out.get("f64_branch_pinned", out["f64"])["max_rel_err"]
    out["against"] = "the oracle (CPU restatement of the reference substep) run on the same state and adjoint"
    return out


def cpu_sample(env, dt, st, adj1, cv, cv1, threads, target_s, max_sub):
    """The oracle's work per substep of the reference's training iteration (the forward substep, then in
    the backward sweep its recompute and adjoint: memory_from_cache, forward, .grad) from ``st``,
    repeated on the control velocities of the mid-rollout frames until ``target_s`` elapses; returns
    (substeps, seconds)."""
    import numpy as np

    from oracle import oracle as O

    o = O.Oracle(env, dt, np.float32, n_threads=threads)
    done, t0 = 0, time.perf_counter()
    s = st
    while (time.perf_counter() - t0 < target_s or done == 0) and done < max_sub:
        s1, _ = o.substep(s, cv=cv, cv1=cv1)
        o.substep_bwd(s, adj1, cv=cv, cv1=cv1)
        s = s1
        done += 1
    return done, time.perf_counter() - t0


def cpu_baseline(cfg, st, adj1, cv, cv1, where, target_s=10.0):
    env = cfg.envs[0]
    threads = os.cpu_count() or 1
    n1, s1 = cpu_sample(env, cfg.dt, st, adj1, cv, cv1, 1, target_s / 2, cfg.substeps)
    nN, sN = cpu_sample(env, cfg.dt, st, adj1, cv, cv1, threads, target_s, cfg.substeps)
    return {"value": env.n_particles * nN / sN, "unit": UNIT, "cores": threads, "kind": "port",
            "value_1thread": env.n_particles * n1 / s1,
            "sample": f"{nN} substeps ({n1} with 1 thread) of environment 0 of {cfg.name} ({env.n_particles} "
                      f"particles) from {where}, each the forward substep plus the backward sweep's recompute and "
                      f"adjoint, float32; {threads} OpenMP threads (and 1)"}


def run_ours(args):
    import torch
    import torch.distributed as dist

    from difftactile_gb300 import replicas

    rank, world_size, local = replicas.rank_info()
    if world_size > 1:
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    barrier = replicas.barrier
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)

    cfg = make_config(args.config, args.horizon, args.envs)
    w, traj = build(cfg, dev, args)
    res, acts = measure(cfg, w, traj, args, dev, flush, args.steps, args.warmup, barrier)
    ms = replicas.slowest(res["ms"], dev)  # the step of the whole job lasts as long as its slowest rank
    units = cfg.n_particles * cfg.n_steps * cfg.substeps
    value = replicas.total(units, dev) / (ms / 1e3)
    out = {"metric": METRIC, "value": value, "unit": UNIT,
           "n_gpus": world_size, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
           "data": "synthetic (seeded scene generators)",
           "config": {"workload": cfg.name, "envs": len(cfg.envs), "particles": cfg.n_particles,
                      "control_steps": cfg.n_steps, "substeps": cfg.substeps,
                      "grids": sorted({e.n_grid[0] for e in cfg.envs}), "fem_tets": w.n_tets, "fem_nodes": w.n_verts,
                      "surface_tris": w.n_tris, "checkpoint_every": cfg.ckpt_every, "tape_blocks": w.tape_blocks,
                      "rebin_every": int(getattr(traj, "rebin_every", 0)),
                      "scatter": ["tile", "global", "warp", "smem"][w.w.scatter_mode], "p_block": int(w.w.p_block),
                      "scatter_depth": int(w.w.scatter_depth),
                      "scatter_depth_adjoint": {1: 1, 2: 2, 3: 0}.get(int(w.w.scatter_depth_adj), int(w.w.scatter_depth)),
                      "contact_lanes": 4 if int(w.w.contact_lanes) == 4 else 8,
                      "particles_per_thread": max(1, int(w.w.p_per_thread)),
                      "programmatic_dependent_launch": bool(w.lib.dt_get_pdl()),
                      "launch_shape": "autotuned" if res["tuned"] else "fixed", "cuda_graph": not args.no_graph,
                      "svd_tape": w.t["p_svd"] is not None, "active_blocks_mean": res["active_blocks_mean"],
                      "active_blocks_max": res["active_blocks_max"],
                      "l2": "flushed between timed iterations (256 MiB write); inputs exceed L2",
                      "parallelism": f"replicas x{world_size}"},
           "gpu_launches": res["launches_per_iter"] * args.steps,
           "roofline": dict(res["roofline"], traffic=None, traffic_static_capture={
               "bytes_per_launch": NCU_TRAFFIC["per_launch_bytes"].get(res["roofline"]["kernel"]),
               "captured_at": NCU_TRAFFIC["captured_at"]} if cfg.name == "batched_population" else None),
           "kernel_breakdown": res["breakdown"], "loss": res["loss"], "grad_norm": res["grad_norm"],
           "times_ms": res["times_ms"]}
    if res["clocks"]:
        out["clocks"] = res["clocks"]
    if res["tuned"]:
        out["autotune"] = {"frame": res["tuned"]["frame"], "best": res["tuned"]["best"],
                           "substep_ms": {k: round(v, 4) for k, v in res["tuned"]["ms"].items()}}
    if not args.no_e2e:
        e = end_to_end(cfg, w, traj, dev, flush, min(args.steps, 3), barrier)
        e_ms = replicas.slowest(e["ms"], dev)
        out["e2e"] = {"value": replicas.total(units, dev) / (e_ms / 1e3), "unit": UNIT, "ms_per_step": e_ms,
                      "iterations": e["iterations"], "h2d_bytes_per_step": e["h2d_bytes_per_step"],
                      "d2h_bytes_per_step": e["d2h_bytes_per_step"]}
    if rank == 0 and not args.no_cpu:
        try:
            mid = mid_rollout(cfg, w, traj, acts)
            out["grad_check"] = grad_check(cfg, w, mid, os.cpu_count() or 1)
            where = (f"the GPU rollout's state at step {mid['t']}, substep {mid['f']} (the pad in contact; that "
                     f"frame's control velocities; the real loss's adjoint)")
            out["cpu_baseline"] = cpu_baseline(cfg, mid["st"], mid["adj1"], mid["cv"], mid["cv1"], where)
        except Exception as exc:  # reported in the line, not fatal to the measurement
            out.setdefault("grad_check", {"error": repr(exc)})
    del w, traj
    torch.cuda.empty_cache()
    if cfg.name == "batched_population" and args.plain > 0:
        out["plain"] = time_plain(cfg, args, dev, flush)
        out["batched_over_plain"] = value / out["plain"]["value"]
    if cfg.name == "batched_population" and not args.no_nested:
        sp = make_config("sensor_press", None)
        w2, traj2 = build(sp, dev, args)
        r2, _ = measure(sp, w2, traj2, args, dev, flush, 3, 3, barrier)
        u2 = sp.n_particles * sp.n_steps * sp.substeps
        out["sensor_press"] = {"value": u2 / (r2["ms"] / 1e3), "unit": UNIT, "ms_per_step": r2["ms"], "steps": 3,
                               "warmup": 3, "particles": sp.n_particles, "control_steps": sp.n_steps,
                               "substeps": sp.substeps, "checkpoint_every": sp.ckpt_every,
                               "roofline": r2["roofline"],
                               "kernel_breakdown": {k: {"ms_per_launch": v["ms_per_launch"], "share": v["share"]}
                                                    for k, v in r2["breakdown"].items()}}
        del w2, traj2
    if rank == 0:
        print(json.dumps(out))
    if world_size > 1:
        dist.destroy_process_group()


# ------------------------------------------------------------------------------------------------
# the reference arm: the reference's CPU path on the host cores
# ------------------------------------------------------------------------------------------------
def reference_state(cfg, threads, steps):
    """Environment 0 rolled forward by the oracle from rest through ``steps`` control steps of the
    workload's press (the pad reaches the object after ~17 steps): the state, the next step's per-frame
    control velocities (fem_sensor.py:229-266 with the workload's actions) and a seeded adjoint."""
    import numpy as np
    import torch

    from difftactile_gb300.trajectory import eul2mat_zyx
    from oracle import oracle as O

    env = cfg.envs[0]
    sp = env.sensors[0]
    o = O.Oracle(env, cfg.dt, np.float32, n_threads=threads)
    st = o.initial_state()
    TW = np.eye(4) if sp.trans_world is None else np.asarray(sp.trans_world, np.float64)
    k = cfg.dt * cfg.substeps
    inv_T = 1.0 / k

    def cv_of(t, vp):
        a = torch.as_tensor(cfg.actions[t, 0], dtype=torch.float64)
        M = eul2mat_zyx(a[3:6] * k, a[0:3] * k).numpy()
        D = TW @ M @ np.linalg.inv(TW)
        return [(((vp.astype(np.float64) @ D[:3, :3].T) + D[:3, 3]) - vp.astype(np.float64)) * inv_T]

    for t in range(steps):
        cv = cv_of(t, st["vpos"][0])
        for _ in range(cfg.substeps):
            st, _ = o.substep(st, cv=cv, cv1=cv)
    cv = cv_of(steps, st["vpos"][0])
    rng = np.random.default_rng(8)
    N = env.n_particles
    adj1 = {"x": rng.standard_normal((N, 3)), "v": rng.standard_normal((N, 3)),
            "C": 1e-2 * rng.standard_normal((N, 3, 3)), "F": rng.standard_normal((N, 3, 3)),
            "pos": [rng.standard_normal(sp.verts.shape)], "vel": [rng.standard_normal(sp.verts.shape)],
            "vpos": [rng.standard_normal(sp.verts.shape)]}
    return st, adj1, cv


def run_reference(args):
    """The reference's CPU path.  Its Taichi CPU backend is not installable here, so the oracle (a C++
    restatement of the same kernels, all host threads) runs a bounded sample of the same workload:
    environment 0 rolled forward by the oracle into contact, then per bench step about 10 s of whole
    substeps of its training iteration (forward substep + the backward sweep's recompute and adjoint).
    ms_per_step extrapolates the sample's rate to one whole iteration of the workload."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    cfg = make_config(args.config, args.horizon, args.envs)
    threads = os.cpu_count() or 1
    pre = min(25 if cfg.name == "batched_population" else 40, cfg.n_steps // 2)
    st, adj1, cv = reference_state(cfg, threads, pre)
    env = cfg.envs[0]
    for _ in range(max(args.warmup, 0)):
        cpu_sample(env, cfg.dt, st, adj1, cv, cv, threads, 1.0, cfg.substeps)
    vals = []
    for _ in range(max(args.steps, 1)):
        n, s = cpu_sample(env, cfg.dt, st, adj1, cv, cv, threads, 10.0, 10 ** 9)
        vals.append(env.n_particles * n / s)
    n1, s1 = cpu_sample(env, cfg.dt, st, adj1, cv, cv, 1, 5.0, 10 ** 9)
    v = sum(vals) / len(vals)
    units = cfg.n_particles * cfg.n_steps * cfg.substeps
    where = f"the oracle's own rollout of environment 0 through {pre} control steps of the press (pad in contact)"
    out = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT,
           "n_gpus": 0, "steps": args.steps, "warmup": args.warmup, "ms_per_step": units / v * 1e3,
           "ms_per_step_note": "extrapolated from the sample rate to one whole training iteration of the workload",
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
           "data": "synthetic (seeded scene generators)",
           "config": {"workload": cfg.name, "envs": len(cfg.envs), "particles": cfg.n_particles,
                      "control_steps": cfg.n_steps, "substeps": cfg.substeps},
           "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                            "value_1thread": env.n_particles * n1 / s1,
                            "sample": f"~10 s per step of whole substeps of environment 0 ({env.n_particles} "
                                      f"particles) from {where}, each the forward substep plus the backward sweep's "
                                      f"recompute and adjoint (seeded adjoint), float32, {threads} OpenMP threads; "
                                      f"the one-thread rate from a 5 s sample"},
           "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out))


def exercise_readouts():
    """Every readout, action and deform-loss entry point once, forward and adjoint, at configuration 2's
    size (and the gripper's affine control velocities on a small grasp): the launches a profiler
    captures for them (no timing, no JSON line)."""
    import numpy as np
    import torch
    from difftactile_gb300 import _native as N
    from difftactile_gb300 import configs, deform, markers, rigid
    from difftactile_gb300.trajectory import GripperTrajectory, Trajectory
    from difftactile_gb300.world import World
    dev = torch.device("cuda", 0)
    cfg = configs.sensor_press(n_steps=1)
    w, tr = cfg.build(dev)
    tr.forward(torch.as_tensor(cfg.actions, dtype=torch.float64, device=dev))
    tr.backward()  # step begin, pose control, substeps, marker loss; their adjoints
    f = 1
    w.com(f)
    gb = torch.zeros((w.n_envs, 4), device=dev)
    gb[:, 1] = 1.0
    N.check(w.lib.dt_com_bwd(w.wp, f, gb.data_ptr(), w.stream), "dt_com_bwd")
    out = torch.zeros((1, 4), device=dev)
    N.check(w.lib.dt_contact_force(w.wp, 0, f, out.data_ptr(), w.stream), "dt_contact_force")
    ob = torch.ones((1, 4), device=dev)
    N.check(w.lib.dt_contact_force_bwd(w.wp, 0, ob.data_ptr(), w.stream), "dt_contact_force_bwd")
    mm = markers.MarkerModel(w, 0)
    pred, virt = mm.readout(f)
    mm.readout_bwd(f, torch.ones_like(pred), torch.ones_like(virt))
    dl = deform.DeformLoss(w, 0)
    n = dl.n
    tgt = np.zeros(tuple(n), np.float32)
    tgt[n[0] // 3:2 * n[0] // 3, 4:12, n[2] // 3:2 * n[2] // 3] = 1.0
    dl.initialize(tgt, passes=2)
    dl.grid_mass(f)
    dl.compute_loss(f)
    dl.compute_loss_grad(f)
    rm = rigid.RigidMatch(w, 0, 0)
    rm.H(f)
    rm.backward(f, torch.ones(9, device=dev), 0)
    cfg3, kin = configs.grasp_sphere(n_steps=2, substeps=5, n_grid=64, n_core=2_000, n_shell=18_000, ckpt_every=1)
    w3 = World(cfg3.envs, n_frames=Trajectory.frames_needed(2, 5, 1), dt=cfg3.dt)
    t3 = GripperTrajectory(w3, 2, kin, (0, 1), 1, ())
    t3.forward(torch.as_tensor(cfg3.actions, dtype=torch.float64, device=dev))
    t3.backward()
    torch.cuda.synchronize()
    if w.error_word() or w3.error_word():
        raise SystemExit(f"device error word {w.error_word()} / {w3.error_word()}")


def main():
    args = parse()
    if args.readouts:
        exercise_readouts()
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
