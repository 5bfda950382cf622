"""GPU: the C++ drop-in programs (tests/cpp) against the reference goldens."""
import json
import os
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN, ROOT

pytestmark = pytest.mark.gpu
GOLD = json.load(open(os.path.join(GOLDEN, "reference_goldens.json")))
BUILD = os.path.join(ROOT, "tests", "_build")


def _run(name):
    exe = os.path.join(BUILD, name)
    if not os.path.exists(exe):
        import runpy
        runpy.run_path(os.path.join(ROOT, "tests", "cpp", "build.py"), run_name="__main__")
    r = subprocess.run([exe], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    return json.loads(r.stdout)


def _value(expr, case):
    """Maps a golden expression (front / size()/2 / back rows) to our rows."""
    row = {"front": 0, "mid": 1, "back": 2}
    if expr.startswith("test.output.times()"):
        key = "front" if ".front()" in expr else "back" if ".back()" in expr else "mid"
        return case["times"][row[key]]
    key = "front" if ".front()" in expr else "back" if ".back()" in expr else "mid"
    idx_expr = expr.rsplit("[", 1)[1].rstrip("]")
    n_var = len(case["rows"][0])
    idx = eval(idx_expr.replace("test.n_var", str(n_var)).replace("/", "//"))
    return case["rows"][row[key]][idx]


def _check(case, golden, rel):
    assert case["n_saved"] == golden["n_saved"]
    for chk in golden["checks"]:
        got = _value(chk["expr"], case)
        assert got == pytest.approx(chk["value"], rel=rel, abs=rel), chk["expr"]


def test_cpp_dropin_nvcc():
    out = _run("test_dropin")
    assert out.pop("state_executor_failures") == 0
    for name, case in out.items():
        g = GOLD["cases"][name]
        tol = 1e-6 if "Exponential" in name else 1e-10
        # N-body midpoint: CudaRKEmbeddedTest.cu:316-317 (1.657666 * tol * n / 2)
        _check(case, g, 2e-8 if "NBody" in name else 10 * tol)


def test_cpp_dropin_host_compiler():
    out = _run("test_dropin_host")
    g = GOLD["cases"]["RKF78NBodyConsistencyTest"]
    _check(out["RKF78NBodyConsistencyTest"], g, 2e-8)
    a, b = out["he21_tag"], out["he21_refstyle"]
    assert a == b  # a reference-layout tableau gives the same bits as the tag
