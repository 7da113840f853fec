"""The benchmark's JSON contract, checked on the CPU arm (bench.py --impl
reference on a tiny 8^3 grid: the C restatement, no GPU): one JSON line with
the metric, value, units, step counts, config of the same workload as the
GPU arm, a cpu_baseline and an e2e object."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_prints_one_contract_line():
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--n", "8",
                        "--steps", "2", "--warmup", "1"], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr
    lines = [ln for ln in r.stdout.splitlines() if ln.strip().startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "data", "config", "impl", "cpu_baseline", "e2e"):
        assert key in d, key
    assert d["impl"] == "reference" and d["unit"] == "GB/s" and d["higher_is_better"] is True
    assert d["value"] > 0 and d["ms_per_step"] > 0 and d["steps"] == 2
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["kind"] == "port" and cb["cores"] >= 1 and cb["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    c = d["config"]
    assert c["N"] == 5 * 8 ** 3 and c["k"] == 10 and c["Nw"] == 32 and c["workload"].startswith("3D8:")


def _mock_runner(errs, per_q):
    """A solver stand-in for the time-to-gains search: the run at q returns
    a one-gain result whose relative error is errs[q] (0.5 elsewhere) and
    takes per_q[precision] * q seconds."""
    import numpy as np
    calls = []

    def runner(prec):
        def run(q, periods, tr, dtf):
            calls.append((prec, q))
            return per_q[prec] * q, np.array([[1.0 + errs.get(q, 0.5)]])
        return run
    return runner, calls


def test_time_to_gains_search_from_a_starting_q():
    """A plan with a starting q: the first form goes up from it until the
    tolerance is met and down while it still is; the further forms start
    one q below the first form's answer; each form's reported q is its own
    smallest one and the ratio is plain time over the fastest chosen form."""
    sys.path.insert(0, ROOT)
    import numpy as np
    import bench

    errs = {19: 2e-3, 20: 1.6e-3, 21: 1.3e-3, 22: 9.7e-4, 23: 7.4e-4}
    runner, calls = _mock_runner(errs, {"c64": 0.2, "c128": 3.0, "ref": 0.25})
    err = lambda S, j: float(np.abs(S[0, 0] - 1.0))  # noqa: E731
    forms = (("precision_c64", "c64"), ("plain_c128", "c128"), ("precision_c64_refine", "ref"))
    for start in (20, 22, 23):
        calls.clear()
        out = bench.ttg_forms(runner, err, [1.0, 1.0], [(3, 0, 0.7)], 24, "mock", forms=forms, budget_s=1e6,
                              q_start={(3, 0, 0.7): start})
        for name, _ in forms:
            assert out[name]["best"]["q"] == 22, (start, name, out[name]["trace"])
        assert [q for p, q in calls if p == "c128"][1:] == [21, 22]  # after the q = 0 warm-up
        assert out["chosen"] == "precision_c64"
        assert out["ratio_plain_over_chosen"] == 15.0
        assert out["q_start"] == {"3,0,0.7": start}
    # A tolerance never met: no best run and no ratio.
    runner, _ = _mock_runner({}, {"c64": 0.2, "c128": 3.0, "ref": 0.25})
    out = bench.ttg_forms(runner, err, [1.0, 1.0], [(3, 0, 0.7)], 24, "mock", forms=forms, budget_s=1e6,
                          q_start={(3, 0, 0.7): 22})
    assert out["precision_c64"]["best"] is None and out["ratio_plain_over_chosen"] is None
    summary = bench.summarize({"time_to_gains_1e-3": {"a": {"ratio_plain_over_chosen": 2.0, "chosen": "x"},
                                                      "b": {"ratio_plain_over_chosen": 15.0, "chosen": "y"}}})
    assert summary["ttg_best_ratio"] == 15.0 and summary["ttg_best_workload"] == "b"
