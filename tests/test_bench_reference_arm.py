"""The benchmark's reference arm on the host (no GPU): `bench.py --impl reference` rolls environment 0
forward with the oracle, times bounded samples of whole substeps of the training iteration on the host
cores (all threads per step, then one thread) and prints one JSON line with our arm's metric, unit and
direction, the CPU-baseline description and an end-to-end entry without device copies; under torchrun
only rank 0 prints."""
import json
import types

import bench


def _args(**kw):
    a = dict(config="sensor_press", horizon=1, envs=None, steps=2, warmup=1)
    a.update(kw)
    return types.SimpleNamespace(**a)


def _short(monkeypatch):
    real = bench.cpu_sample
    calls = []

    def short(env, dt, st, adj1, cv, cv1, threads, target_s, max_sub):
        calls.append((threads, target_s))
        return real(env, dt, st, adj1, cv, cv1, min(threads, 4), 0.01, 1)

    monkeypatch.setattr(bench, "cpu_sample", short)
    return calls


def test_reference_arm_prints_one_line(monkeypatch, capsys):
    calls = _short(monkeypatch)
    monkeypatch.delenv("RANK", raising=False)
    bench.run_reference(_args())
    lines = capsys.readouterr().out.strip().splitlines()
    assert len(lines) == 1
    out = json.loads(lines[0])
    assert out["impl"] == "reference"
    assert (out["metric"], out["unit"], out["higher_is_better"]) == (bench.METRIC, bench.UNIT, True)
    assert out["value"] > 0 and out["steps"] == 2 and out["warmup"] == 1
    assert out["config"]["workload"] == "sensor_press" and out["config"]["particles"] == 64_000
    cb = out["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and "substeps" in cb["sample"] and cb["value"] == out["value"]
    assert cb["value_1thread"] > 0
    assert out["e2e"] == {"value": out["value"], "unit": bench.UNIT, "h2d_bytes_per_step": 0,
                          "d2h_bytes_per_step": 0}
    # units of one bench step / the measured rate
    assert abs(out["ms_per_step"] - 64_000 * 1 * 20 / out["value"] * 1e3) <= 1e-6 * out["ms_per_step"]
    n = cb["cores"]
    # one short warm-up sample, one bounded sample per step on all threads, then one on a single thread
    assert calls == [(n, 1.0), (n, 10.0), (n, 10.0), (1, 5.0)]


def test_reference_arm_is_silent_off_rank_0(monkeypatch, capsys):
    calls = _short(monkeypatch)
    monkeypatch.setenv("RANK", "1")
    bench.run_reference(_args())
    assert capsys.readouterr().out == "" and calls == []
