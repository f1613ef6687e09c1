"""bench.py's default line summarises the mixed-size, serving and precision
runs, each run in a process of its own: the summary keeps the kept keys of a
run's JSON line, and a run that fails or runs out of time is reported as an
error entry instead of breaking the line (CPU; the processes are faked)."""

import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

import bench  # noqa: E402


def _fake_run(results):
    calls = []

    def run(cmd, **kw):
        calls.append(cmd)
        mode = next(a for a in cmd if a in ("--mixed", "--serve", "--precision"))
        r = results[mode]
        if isinstance(r, BaseException):
            raise r
        return subprocess.CompletedProcess(cmd, r[0], stdout=r[1], stderr=r[2])

    return run, calls


def test_modes_summarised_and_failures_reported(monkeypatch):
    mixed = {"metric": "m", "value": 5.0, "unit": "pairs/s", "form": "tensor_refined",
             "chosen": {"pairs_per_s": 5.0, "tuning": ["x"]}, "plain_form": {"pairs_per_s": 1.0},
             "chosen_over_plain": 5.0, "config": {}, "not_kept": 1}
    run, calls = _fake_run({
        "--mixed": (0, "log line\n" + json.dumps(mixed) + "\n", ""),
        "--serve": (1, "", "Traceback\nRuntimeError: no device\n"),
        "--precision": subprocess.TimeoutExpired(["python"], 900),
    })
    monkeypatch.setattr(bench.subprocess, "run", run)
    out = bench.other_modes()
    assert set(out) == {"mixed", "serve", "precision"}
    assert out["mixed"]["value"] == 5.0 and "not_kept" not in out["mixed"]
    assert "tuning" not in out["mixed"]["chosen"]
    assert "exit 1" in out["serve"]["error"] and "no device" in out["serve"]["error"]
    assert "did not finish" in out["precision"]["error"]
    assert len(calls) == 3 and all(c[1] == os.path.join(ROOT, "bench.py") for c in calls)


def test_no_modes_flag():
    sys_argv = sys.argv
    try:
        sys.argv = ["bench.py", "--no-modes"]
        assert bench.parse_args().no_modes
        sys.argv = ["bench.py"]
        assert not bench.parse_args().no_modes
    finally:
        sys.argv = sys_argv
