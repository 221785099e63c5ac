"""Benchmark: forward+backward particle-substeps/s of the differentiable DiffTactile substep on one
GB300 (replicas on N GPUs under torchrun).

One bench step = one training iteration of the sensor-press task: 100 control steps x 20 substeps
forward (every frame kept on the device), then the backward sweep (adjoint substeps straight down
the tape) down to the action gradients.  The batched-population workload keeps a device checkpoint
of every step start instead and recomputes each step's substep tape in the backward sweep.  The
unit counts each particle advanced one substep forward and back-propagated once: n_particles x 100
x 20 per bench step.

Before timing, the autotuner picks the launch shape on a mid-rollout substep and the rollout is
recorded as CUDA graphs (the timed iterations replay them).  The line carries the dominant kernel's
roofline (CUDA events around every 25th of its launches), the end-to-end rate through the public API
with host buffers, the oracle on the host cores as the CPU baseline, and a full-size gradient check
against the oracle's adjoint of one mid-rollout substep.

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
    ap.add_argument("--config", default="sensor_press", choices=["sensor_press", "batched_population"])
    ap.add_argument("--horizon", type=int, default=None, help="control steps (default: the config's)")
    ap.add_argument("--envs", type=int, default=None, help="batched_population: the first N environments only")
    ap.add_argument("--scatter", default=None, choices=["tile", "global", "warp"],
                    help="27-node scatter strategy (default: the library's)")
    ap.add_argument("--no-pdl", action="store_true", help="launch the substep kernels without programmatic "
                    "dependent launch")
    ap.add_argument("--p-block", type=int, default=None, choices=[64, 128, 256],
                    help="threads per CTA of the particle launches")
    ap.add_argument("--depth", type=int, default=None, choices=[0, 1, 2, 3, 4, 5],
                    help="shuffle steps of the warp scatter's segmented reduction (0: whole runs)")
    ap.add_argument("--no-tune", action="store_true", help="keep the library's default launch shape instead of "
                    "the autotuner's choice (also implied by --scatter, --no-pdl, --p-block or --depth)")
    ap.add_argument("--plain", type=int, default=0,
                    help="also time the first K environments one World each (one scene per launch "
                    "sequence) and report the batched / plain ratio")
    ap.add_argument("--no-svd-tape", action="store_true", help="the adjoint recomputes the SVD instead of "
                    "reading the forward's from the tape")
    ap.add_argument("--no-graph", action="store_true", help="launch every substep from the host instead of "
                    "replaying the rollout's recorded CUDA graphs")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    return ap.parse_args()


def make_config(name, horizon, envs=None):
    from difftactile_gb300 import configs
    if name == "sensor_press":
        return configs.sensor_press(n_steps=horizon or 100)
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


# algorithmic bytes per unit of each fused launch
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


# DRAM bytes (read + write) per launch from one ncu capture of the sensor-press workload
# (profiles/kernels_sensor_press.md); per-launch sizes equal the full workload's
NCU_TRAFFIC = {"sensor_press": {"k_fwd_p2g_fem": 7.875e6, "k_fwd_grid": 0.387e6, "k_bwd_p2g_fem": 18.662e6,
                                "k_bwd_g2p_fem": 6.152e6}}


def algo_bytes(key, units):
    return sum(b * units.get(u, 0) for u, b in BYTES[key].items())


def run_ours(args):
    import numpy as np
    import torch
    import torch.distributed as dist

    from difftactile_gb300 import replicas

    rank, world_size, local = replicas.rank_info()
    if world_size > 1:
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)

    barrier = replicas.barrier

    cfg = make_config(args.config, args.horizon, args.envs)
    kw = {} if args.scatter is None else {"scatter_mode": {"tile": 0, "global": 1, "warp": 2}[args.scatter]}
    if args.no_svd_tape:
        kw["svd_tape"] = False
    if args.p_block is not None:
        kw["p_block"] = args.p_block
    if args.depth is not None:
        kw["scatter_depth"] = args.depth
    w, traj = cfg.build(dev, **kw)
    w.lib.dt_set_pdl(0 if args.no_pdl else 1)
    tune_launch = not (args.no_tune or args.scatter or args.no_pdl or args.p_block or args.depth is not None)
    acts = torch.as_tensor(cfg.actions, dtype=torch.float64, device=dev)
    t = w.t
    init = [t["p_state"][0].clone(), t["v_pos"][0].clone(), t["v_vel"][0].clone(), t["v_vpos"][0].clone()]

    def reset():
        t["p_state"][0].copy_(init[0])
        t["v_pos"][0].copy_(init[1])
        t["v_vel"][0].copy_(init[2])
        t["v_vpos"][0].copy_(init[3])

    def iteration():
        reset()
        loss = traj.forward(acts)
        g = traj.backward()
        return loss, g

    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)

    # ---- launch shape (untimed): the autotuner times every candidate on one mid-rollout substep ----
    iteration()
    torch.cuda.synchronize()
    tuned = None
    if tune_launch:
        from difftactile_gb300 import autotune
        f_mid = traj.f_end // 2 if traj.full else traj.S // 2
        tuned = autotune.tune_substep(w, frame=f_mid)
        tuned["frame"] = f_mid
        iteration()
        torch.cuda.synchronize()

    # ---- per-kernel breakdown (untimed, launched from the host): probe each launch over one iteration ----
    breakdown = {}
    for key in NAMES:
        w.set_probe(*key)
        iteration()
        ms, n = w.probe_ms()
        breakdown[key] = (ms, n)
    w.set_probe(None)
    tot = sum(ms * n for ms, n in breakdown.values())
    dom = max(breakdown, key=lambda k: breakdown[k][0] * breakdown[k][1])

    # the timed iterations carry CUDA-event pairs around every PROBE_EVERY-th launch of the dominant
    # kernel; with graphs the first warm-up iteration records the rollout (events included) and the
    # rest replay it
    w.set_probe(*dom, every=PROBE_EVERY)
    traj.graph = not args.no_graph
    traj.reset_graphs()
    for _ in range(max(args.warmup, 0)):
        iteration()
    torch.cuda.synchronize()
    if w.error_word():
        raise RuntimeError(f"device error word {w.error_word()} during warm-up")

    # ---- timed region ----
    clocks = Clocks(local)
    traj.launches = 0
    times, dom_acc = [], []
    w.probe_events.clear()  # host-recorded pairs of the warm-up; graph-recorded pairs are re-recorded
    for _ in range(args.steps):
        flush.zero_()  # L2 flush between timed iterations (256 MiB > 129 MB L2)
        torch.cuda.synchronize()
        barrier()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        loss, g = iteration()
        e1.record()
        torch.cuda.synchronize()
        barrier()
        times.append(e0.elapsed_time(e1))
        dom_acc.append(w.probe_ms())  # this iteration's launches of the dominant kernel
        if not traj.graph:
            w.probe_events.clear()
    dom_n = sum(n for _, n in dom_acc)
    dom_ms = sum(m * n for m, n in dom_acc) / max(dom_n, 1)
    clk = clocks.stop()
    w.set_probe(None)
    traj.reset_graphs()  # the end-to-end iterations record their own graphs, without the event pairs
    launches_per_iter = traj.launches // max(args.steps, 1) + 2  # + loss readout/adjoint seeds
    ms = sum(times) / len(times)
    ms = replicas.slowest(ms, dev)  # the step of the whole job lasts as long as its slowest rank
    units = cfg.n_particles * cfg.n_steps * cfg.substeps
    value = replicas.total(units, dev) / (ms / 1e3)

    # ---- roofline of the dominant kernel ----
    used = t["tape_bcount"][: traj.f_end]
    cnt = used.clamp(max=w.tape_blocks).double().mean().item()
    cnt_max = int(used.max().item())
    unit_counts = {"particle": w.n_particles, "node": 64 * cnt, "tet": w.n_tets, "tri": w.n_tris,
                   "vert": w.n_verts}
    peak, peak_kind = peaks()
    ab = algo_bytes(dom, unit_counts)
    achieved = ab / (dom_ms / 1e3) / 1e9

    out = {"metric": METRIC, "value": value, "unit": UNIT,
           "n_gpus": world_size, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
           "data": "synthetic (seeded scene generators)",
           "config": {"workload": cfg.name, "particles": cfg.n_particles, "control_steps": cfg.n_steps,
                      "substeps": cfg.substeps, "grid": list(cfg.envs[0].n_grid), "envs": len(cfg.envs),
                      "fem_tets": w.n_tets, "fem_nodes": w.n_verts, "surface_tris": w.n_tris,
                      "checkpoint_every": cfg.ckpt_every, "tape_blocks": w.tape_blocks,
                      "scatter": ["tile", "global", "warp"][w.w.scatter_mode],
                      "p_block": int(w.w.p_block), "scatter_depth": int(w.w.scatter_depth),
                      "contact_lanes": 4 if int(w.w.contact_lanes) == 4 else 8,
                      "programmatic_dependent_launch": bool(w.lib.dt_get_pdl()),
                      "launch_shape": "autotuned" if tuned else "fixed",
                      "cuda_graph": traj.graph,
                      "svd_tape": w.w.p_svd is not None,
                      "active_blocks_mean": cnt, "active_blocks_max": cnt_max, "l2": "flushed between timed iterations (256 MiB write)",
                      "parallelism": f"replicas x{world_size}"},
           "gpu_launches": launches_per_iter * args.steps,
           "roofline": {"kernel": NAMES[dom], "bound": "hbm", "achieved": achieved, "peak": peak,
                        "peak_kind": peak_kind, "unit": "GB/s", "frac": achieved / peak,
                        "traffic": NCU_TRAFFIC.get(cfg.name, {}).get(NAMES[dom]),
                        "algorithmic_bytes_per_launch": ab, "launch_ms": dom_ms, "launches_timed": dom_n,
                        "timed_every_nth_launch": PROBE_EVERY},
           "kernel_breakdown": {NAMES[k]: {"ms_per_launch": v[0], "launches": v[1],
                                           "share": v[0] * v[1] / tot} for k, v in breakdown.items()},
           "loss": float(loss.item()), "grad_norm": float(g.norm().item())}
    if clk:
        out["clocks"] = clk
    if tuned:
        out["autotune"] = {"frame": tuned["frame"], "best": tuned["best"],
                           "substep_ms": {k: round(v, 4) for k, v in tuned["ms"].items()}}

    # ---- end to end through the public API with host buffers ----
    if not args.no_e2e:
        h_act = torch.as_tensor(cfg.actions, dtype=torch.float32).pin_memory()
        xs = np.concatenate([e.x for e in cfg.envs], 0)
        h_x = torch.as_tensor(xs, dtype=torch.float32).pin_memory()
        h_v = torch.zeros_like(h_x).pin_memory()
        e2e = []
        for i in range(args.steps + 1):
            flush.zero_()
            torch.cuda.synchronize()
            barrier()
            t0 = time.perf_counter()
            d_act = h_act.to(dev, non_blocking=True)
            d_x = h_x.to(dev, non_blocking=True)
            d_v = h_v.to(dev, non_blocking=True)
            reset()
            w.set_particles(0, x=d_x, v=d_v)
            loss = traj.forward(d_act.double())
            g = traj.backward()
            res = torch.cat([loss.double(), g.reshape(-1)]).cpu()
            t1 = time.perf_counter()
            if i > 0:
                e2e.append(t1 - t0)
        e_ms = 1e3 * sum(e2e) / len(e2e)
        e_ms = replicas.slowest(e_ms, dev)
        out["e2e"] = {"value": replicas.total(units, dev) / (e_ms / 1e3), "unit": UNIT,
                      "ms_per_step": e_ms,
                      "h2d_bytes_per_step": int(h_act.numel() * 4 + h_x.numel() * 4 + h_v.numel() * 4),
                      "d2h_bytes_per_step": int(res.numel() * 8)}
    if args.plain > 0:
        out["plain"] = time_plain(cfg, args, dev, flush, tune_launch)
        out["batched_over_plain"] = value / out["plain"]["value"]
    if rank == 0 and not args.no_cpu:
        out["cpu_baseline"] = cpu_baseline(cfg, threads=os.cpu_count() or 1)
        try:
            out["grad_check"] = grad_check(cfg, w, traj, threads=os.cpu_count() or 1)
        except Exception as exc:  # reported in the line, not fatal to the measurement
            out["grad_check"] = {"error": repr(exc)}
    if rank == 0:
        print(json.dumps(out))
    if world_size > 1:
        dist.destroy_process_group()


def time_plain(cfg, args, dev, flush, tune_launch):
    """Each of the first K environments in a World of its own, stepped one after the other with the
    same actions (the one-scene-per-launch path); aggregate particle-substeps/s of the sample."""
    import torch

    from difftactile_gb300.configs import Config

    k = min(args.plain, len(cfg.envs))
    total_ms, units = 0.0, 0
    for e in range(k):
        sub = Config(cfg.name, [cfg.envs[e]], cfg.dt, cfg.substeps, cfg.n_steps, cfg.actions[:, e:e + 1],
                     tuple((0, lay, tg) for s, lay, tg in cfg.loss_terms if s == e), cfg.ckpt_every, cfg.tape_blocks)
        w, traj = sub.build(dev)
        acts = torch.as_tensor(sub.actions, dtype=torch.float64, device=dev)
        traj.forward(acts)
        traj.backward()
        if tune_launch:  # each single-environment World gets its own launch shape
            from difftactile_gb300 import autotune
            autotune.tune_substep(w, frame=traj.f_end // 2 if traj.full else traj.S // 2)
        traj.graph = not args.no_graph
        for _ in range(max(args.warmup, 1)):
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
        total_ms += e0.elapsed_time(e1)
        units += cfg.envs[e].n_particles * cfg.n_steps * cfg.substeps
        del w, traj
    return {"value": units / (total_ms / 1e3), "unit": UNIT, "envs": k, "ms": total_ms,
            "path": "one World per environment, launched one after the other"}


def cpu_baseline(cfg, threads, target_s=15.0):
    """The oracle (CPU restatement of the reference step) on the host cores: a bounded sample of
    whole substeps of the same scene, forward + backward."""
    import numpy as np

    from oracle import oracle as O

    env = cfg.envs[0]
    o = O.Oracle(env, cfg.dt, np.float32, n_threads=threads)
    st = o.initial_state()
    cv = [np.zeros((len(s.verts), 3), np.float32) for s in env.sensors]
    adj = {k: np.ones_like(st[k]) for k in ("x", "v", "C", "F")}
    done, t0 = 0, time.perf_counter()
    # the reference's work per substep: forward, then (in the backward sweep) recompute + adjoint
    while time.perf_counter() - t0 < target_s and done < cfg.substeps:
        st1, _ = o.substep(st, cv=cv, cv1=cv)
        o.substep_bwd(st, adj, cv=cv, cv1=cv)
        st = st1
        done += 1
    dt_ = time.perf_counter() - t0
    return {"value": env.n_particles * done / dt_, "unit": UNIT, "cores": threads,
            "kind": "port",
            "sample": f"{done} substeps of env 0 of {cfg.name} ({env.n_particles} particles), forward + "
                      f"recompute + adjoint per substep, float32, {threads} OpenMP threads"}


def grad_check(cfg, w, traj, threads):
    """Gradient parity on the benchmark's own state: one adjoint substep of the CUDA path at a
    mid-rollout frame, against the float64 oracle's adjoint of the same substep from the same
    (float32) state of environment 0, the oracle serving as the reference.  Returns norm-wise
    relative errors of the frame-f adjoints of x, v, C, F and of the sensor positions."""
    import numpy as np
    import torch

    from oracle import oracle as O

    f = traj.f_end // 2 if traj.full else traj.S // 2
    env = cfg.envs[0]
    n0 = env.n_particles
    P = w.particles(f)
    st = {k: P[k][:n0].double().cpu().numpy() for k in ("x", "v", "C", "F")}
    sl = w.vslice(w.env_rows[0].s_begin)
    fem = lambda name, fr: w.t[name][fr, sl, :3].double().cpu().numpy()  # noqa: E731
    st["pos"], st["vel"], st["vpos"] = [fem("v_pos", f)], [fem("v_vel", f)], [fem("v_vpos", f)]
    cv, cv1 = [fem("v_cv", f)], [fem("v_cv", f + 1)]
    rng = np.random.default_rng(8)
    Np = w.n_particles
    W = {"x": 1e-2 * rng.standard_normal((Np, 3)), "v": 1e-2 * rng.standard_normal((Np, 3)),
         "C": 1e-4 * rng.standard_normal((Np, 3, 3)), "F": 1e-2 * rng.standard_normal((Np, 3, 3))}
    for k in W:
        W[k][n0:] = 0.0
        W[k] = W[k].astype(np.float32)
    w.adj_clear()
    w.set_particle_adjoint(f + 1, **W)
    w.substep_bwd(f)
    torch.cuda.synchronize()
    g = {k: v[:n0].double().cpu().numpy() for k, v in w.particle_adjoint(f).items()}
    gpos = w.t["v_adj_pos"][f & 1, sl, :3].double().cpu().numpy()
    rel = lambda a, b: float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))  # noqa: E731
    # particles on the von Mises yield surface (|delta gamma| < 1e-6, a few float32 ulps of the
    # log-strain norm; mpm_plastic.py:151-166): the return map's branch there flips under any rounding
    # of the forward recompute, so their F adjoint is not a precision-stable quantity (the oracle in
    # float32 and in float64 disagree there alike)
    m = env.materials[0]
    keep = np.ones(n0, bool)
    if len(env.materials) == 1 and m.model == 1 and m.yield_stress > 0:
        Fn = (np.eye(3)[None] + cfg.dt * st["C"]) @ st["F"]
        eps = np.log(np.maximum(np.linalg.svd(Fn, compute_uv=False), 0.05))
        dgam = np.linalg.norm(eps - eps.mean(1, keepdims=True), axis=1) - m.yield_stress / (2.0 * m.mu_lam[0])
        keep = np.abs(dgam) >= 1e-6
    out = {"frame": f, "env": 0, "particles": n0, "on_yield_surface": int(n0 - keep.sum())}
    refs = {}
    for dtype, key in ((np.float64, "f64"), (np.float32, "f32")):
        o = O.Oracle(env, cfg.dt, dtype, n_threads=threads, grad_clip=float(w.w.grad_clip))
        ref = refs[key] = o.substep_bwd(st, {k: W[k][:n0].astype(np.float64) for k in W}, cv=cv, cv1=cv1)
        errs = {k: rel(g[k], ref[k]) for k in ("x", "v", "C", "F")}
        errs["sensor_pos"] = rel(gpos, ref["pos"][0])
        off = {k: rel(g[k][keep], ref[k][keep]) for k in ("x", "v", "C", "F")}
        out[key] = {"rel_err": errs, "max_rel_err": max(errs.values()), "rel_err_off_yield_surface": off,
                    "max_rel_err_off_yield_surface": max(off.values())}
    out["oracle_f32_vs_f64"] = {k: rel(refs["f32"][k], refs["f64"][k]) for k in ("x", "v", "C", "F")}
    out["against"] = ("the oracle's adjoint of the same substep from the same state, in float64 and in "
                      "float32 (the CUDA path's precision)")
    return out


def run_reference(args):
    """The reference's CPU path (its Taichi CPU backend is not installable here; the oracle, a C++
    restatement of the same kernels, runs on all host cores instead)."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    cfg = make_config(args.config, args.horizon, args.envs)
    threads = os.cpu_count() or 1
    for _ in range(max(args.warmup, 0)):
        cpu_baseline(cfg, threads, target_s=2.0)
    vals = [cpu_baseline(cfg, threads, target_s=10.0) for _ in range(max(args.steps, 1))]
    v = sum(x["value"] for x in vals) / len(vals)
    units = cfg.n_particles * cfg.n_steps * cfg.substeps
    out = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT,
           "n_gpus": 0, "steps": args.steps, "warmup": args.warmup, "ms_per_step": units / v * 1e3,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
           "data": "synthetic (seeded scene generators)",
           "config": {"workload": cfg.name, "particles": cfg.n_particles, "control_steps": cfg.n_steps,
                      "substeps": cfg.substeps},
           "cpu_baseline": dict(vals[-1], value=v),
           "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out))


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
