"""Host logic of bench.py, on the CPU: the served-ensemble request generator (seeded, with the
workload's distributions), the mapping of a request to the drop-in programs' flags, and the JSON
line of the reference arm (the CPU restatement timed on the host cores), whose keys the benchmark
contract fixes."""
import importlib.util
import json
import os
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def load_bench():
    spec = importlib.util.spec_from_file_location("bench_under_test", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


class FakeJ:
    FLAG_GRAPH = 4


def test_served_requests_are_seeded_and_follow_the_workload():
    B = load_bench()
    a = B.c5_requests(FakeJ, 2000, 50.0, 20261203)
    b = B.c5_requests(FakeJ, 2000, 50.0, 20261203)
    assert a == b                                             # same seed, same requests
    assert a != B.c5_requests(FakeJ, 2000, 50.0, 7)
    t = np.array([x[0] for x in a])
    assert np.all(np.diff(t) > 0)                             # arrival times increase
    assert abs(np.mean(np.diff(t)) - 1 / 50.0) < 0.1 / 50.0   # Poisson at 50 per second
    reqs = [x[1] for x in a]
    assert [r["rid"] for r in reqs] == list(range(2000))
    uni = [r for r in reqs if r["kind"] == "uniform"]
    amr = [r for r in reqs if r["kind"] == "amr"]
    assert abs(len(amr) / 2000 - 0.5) < 0.05
    assert {r["n"] for r in uni} == {32, 48, 64, 96, 128}
    assert {r["n"] for r in amr} == {16, 24, 32, 48}
    assert all(200.0 <= r["re"] <= 3200.0 for r in reqs)
    assert all(2.0 <= r["tstar"] <= 10.0 for r in reqs)
    assert abs(sum(r["storage"] == "fp16" for r in reqs) / 2000 - 0.5) < 0.05
    assert {r["storage"] for r in reqs} == {"fp16", "fp32"}
    for r in amr:                                             # sensor refinement, graph replay
        assert (r["l1_mode"], r["l2_mode"], r["frac1"], r["frac2"], r["adapt_every"]) == \
            ("sensor", "sensor", 0.3, 0.1, 20)
        assert r["flags"] & FakeJ.FLAG_GRAPH


def test_program_args_name_the_drop_in_flags():
    B = load_bench()
    u = dict(rid=0, kind="uniform", n=64, re=812.5, tstar=3.25, storage="fp16")
    a = B.program_args(FakeJ, u, 0)
    assert a[0].endswith(os.path.join("bin", "uniform"))
    assert a[1:] == ["--n", "64", "--re", "812.5", "--tstar", "3.25", "--prec", "fp16", "--device", "0"]
    m = dict(rid=1, kind="amr", n=24, re=400.0, tstar=2.0, storage="fp32", l1_mode="sensor", l2_mode="sensor",
             frac1=0.3, frac2=0.1, adapt_every=20, flags=FakeJ.FLAG_GRAPH)
    a = B.program_args(FakeJ, m, 0)
    assert a[0].endswith(os.path.join("bin", "amr"))
    for flag, value in (("--l1", "sensor"), ("--l2", "sensor"), ("--frac1", "0.3"), ("--frac2", "0.1"),
                        ("--adapt", "20"), ("--graph", "1"), ("--prec", "fp32")):
        assert a[a.index(flag) + 1] == value


def test_reference_arm_prints_the_contract_line():
    lib = os.path.join(ROOT, "oracle", "liboracle.so")
    if not os.path.exists(lib):
        pytest.skip("oracle not built (run __graft_entry__.build())")
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--n", "32",
                          "--steps", "1", "--warmup", "0"], capture_output=True, text=True, timeout=300, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    line = json.loads(out.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["metric"] == "GLUPS" and line["unit"] == "GLUPS"
    assert line["value"] > 0 and line["higher_is_better"] is True and line["n_gpus"] == 1
    assert line["warmup"] >= 3                                 # the contract's floor on warm-up steps
    cb = line["cpu_baseline"]
    assert cb["value"] == line["value"] and cb["kind"] in ("port", "reference") and cb["cores"] >= 1
    assert line["e2e"] == {"value": line["value"], "unit": "GLUPS", "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}
    assert line["config"]["n"] == 32
