"""CPU checks of the C++ drop-in header: it compiles with the host compiler
alone (no CUDA headers), and the reference's own types plug into it."""
import os
import shutil
import subprocess

import pytest

import oracle
from conftest import ROOT

INC = os.path.join(ROOT, "include")
CPP = os.path.join(ROOT, "tests", "cpp")
REF = oracle.REF_ROOT


def _gxx(args):
    return subprocess.run(["g++", "-std=c++20", "-fsyntax-only", f"-I{INC}", f"-I{CPP}", *args],
                          capture_output=True, text=True)


@pytest.mark.skipif(shutil.which("g++") is None, reason="no g++")
def test_header_compiles_without_cuda():
    r = _gxx([os.path.join(CPP, "test_dropin_host.cpp")])
    assert r.returncode == 0, r.stderr


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "src")), reason="reference not present")
def test_reference_types_plug_in():
    inc = [f"-I{REF}/src/{d}" for d in ("integrator/RKEmbeddedParallel",
                                         "integrator/RKEmbeddedParallel/butcher_tableaus",
                                         "state", "par_exec", "ode", "output", "util")]
    r = _gxx(inc + [os.path.join(CPP, "reference_types_check.cpp")])
    assert r.returncode == 0, r.stderr
