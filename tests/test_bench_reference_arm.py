"""The benchmark's reference arm on the host: `bench.py --impl reference` times real CheFSI
iterations of the CPU oracle (the FP64 restatement of chebyshevOrthogonalizedSubspaceIterationSolver
::solve, src/solvers/eigenSolvers/chebyshevOrthogonalizedSubspaceIterationSolver.cc:116-607) on a
bounded sample of the workload and prints one JSON line in the benchmark's format. Run here on
the 64,000-dof workload (a few seconds); no GPU is touched on this path."""
import json
import os
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def run_arm(extra_env=None):
    env = dict(os.environ)
    env.update(extra_env or {})
    p = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--workload", "small",
                        "--steps", "1", "--warmup", "3"], cwd=ROOT, env=env,
                       capture_output=True, text=True, timeout=600)
    assert p.returncode == 0, p.stderr[-2000:]
    return [l for l in p.stdout.splitlines() if l.strip()]


@pytest.fixture(scope="module")
def line():
    lines = run_arm()
    assert len(lines) == 1, lines
    return json.loads(lines[0])


def test_reference_arm_prints_one_contract_line(line):
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
                "higher_is_better", "scaling", "vs_baseline", "dtype", "data", "config"):
        assert key in line, key
    assert line["impl"] == "reference"
    assert line["unit"] == "s/iter" and line["higher_is_better"] is False
    assert line["dtype"] == "f64"
    assert line["steps"] == 1 and line["warmup"] >= 3
    assert line["steps_run"] == line["steps"] + line["warmup"]
    assert line["value"] > 0 and abs(line["ms_per_step"] - 1e3 * line["value"]) < 1e-6
    assert line["config"]["workload"] == "small"
    assert line["config"]["n_dofs"] == 64000 and line["config"]["n_wfc"] == 96


def test_reference_arm_reports_its_sample_and_no_copies(line):
    cb = line["cpu_baseline"]
    assert cb["kind"] == "port" and cb["value"] == line["value"] and cb["cores"] >= 1
    assert "8 of its 96 vectors" in cb["sample"]
    e2e = line["e2e"]
    assert e2e["value"] == line["value"] and e2e["unit"] == line["unit"]
    assert e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0
    # a scaled figure is labelled as such and kept out of `value`
    assert line["extrapolated_full_n"]["kind"] == "extrapolated"
    assert line["extrapolated_full_n"]["value"] > line["value"]


def test_reference_arm_other_ranks_exit_without_work():
    assert run_arm({"RANK": "1"}) == []
