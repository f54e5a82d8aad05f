"""bench.py's output line carries the keys of the measurement contract.

The GPU work is replaced by stand-ins returning values of the right shape,
so the line's assembly (the part that must not break at the end of a run)
is checked on the CPU, for the library's arm and for the reference arm."""
import io
import json
import sys
from contextlib import redirect_stdout

import pytest

import bench
from cafproject_gb300 import params as P

BASE_KEYS = {"metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
             "vs_baseline", "dtype", "data", "config"}


def _run(monkeypatch, argv):
    monkeypatch.setattr(sys, "argv", ["bench.py"] + argv)
    monkeypatch.setattr(bench, "dist_init", lambda: (1, 0, 0))
    p = P.WORKLOADS["cdm512"]()
    monkeypatch.setattr(bench, "run_gb300", lambda args, ws, rank, lrank: dict(
        value=1.7e9, ms=76.0, clocks={"sm_mhz": 2070.0, "sm_max_mhz": 2070.0, "reasons": []},
        phases={"pp_force": {"ms_per_launch": 11.4}},
        roofline={"bound": "hbm", "achieved": 223.0, "peak": 6793.0, "unit": "GB/s", "frac": 0.033,
                  "traffic": 1.8e9},
        e2e={"value": 1.6e9, "unit": bench.UNIT, "h2d_bytes_per_step": 2, "d2h_bytes_per_step": 2},
        cpu={"value": 4.8e6, "unit": bench.UNIT, "cores": 16, "kind": "port", "sample": "one tile"},
        n=p.npglobal, p=p, t_ic=1.0, gpu_launches=bench.gpu_launches(p, 5)))
    monkeypatch.setattr(bench, "run_adjoint", lambda args, lrank: {"ratio": 2.3})
    monkeypatch.setattr(bench, "run_batched", lambda args, lrank: {"speedup": 2.3})
    monkeypatch.setattr(bench, "run_two_species", lambda args, lrank: {"value": 3.3e9})
    monkeypatch.setattr(bench, "run_redshifts", lambda args, lrank, zs: {"5": {"ms_per_step": 84.0, "value": 1.6e9},
                                                                         "1": {"ms_per_step": 102.0, "value": 1.3e9}})
    monkeypatch.setattr(bench, "run_reference", lambda args, ws, rank: dict(value=4.8e6, ms=27000.0, n=p.npglobal,
                                                                             p=p, steps=2, step_s=[27.0, 27.0]))
    buf = io.StringIO()
    with redirect_stdout(buf):
        bench.main()
    lines = [l for l in buf.getvalue().splitlines() if l.startswith("{")]
    assert len(lines) == 1
    return json.loads(lines[0])


def test_library_arm_line(monkeypatch):
    d = _run(monkeypatch, [])
    assert BASE_KEYS <= set(d)
    assert d["metric"] == bench.METRIC and d["n_gpus"] == 1 and d["steps"] == 5 and d["warmup"] == 3
    for k in ("clocks", "e2e", "roofline", "gpu_launches", "cpu_baseline"):
        assert k in d, k
    assert {"value", "unit", "h2d_bytes_per_step", "d2h_bytes_per_step"} <= set(d["e2e"])
    assert {"bound", "achieved", "peak", "unit", "frac", "traffic"} <= set(d["roofline"])
    assert {"value", "unit", "cores", "kind", "sample"} <= set(d["cpu_baseline"])
    assert d["gpu_launches"] == 37 * 5  # this library's launches per step, as the launch list shows
    assert "workload" in d["config"] and "model" not in d["config"]
    assert set(d["redshifts"]) == {"49", "5", "1"}
    for k in ("adjoint", "batched", "two_species"):
        assert k in d


def test_reference_arm_line(monkeypatch):
    d = _run(monkeypatch, ["--impl", "reference"])
    assert BASE_KEYS <= set(d) and d["impl"] == "reference"
    # the same workload description as the library's arm
    assert d["config"] == _run(monkeypatch, [])["config"]
    assert d["cpu_baseline"]["value"] == d["value"] and d["e2e"]["value"] == d["value"]
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["d2h_bytes_per_step"] == 0


@pytest.mark.parametrize("flag,key", [("--adjoint-only", "adjoint"), ("--batched-only", "batched"),
                                      ("--two-species-only", "two_species")])
def test_single_measurement_lines(monkeypatch, flag, key):
    d = _run(monkeypatch, [flag])
    assert list(d) == [key]
