"""Generates the golden fixtures under tests/golden/ (run in the container
that holds the reference sources; the outputs are committed and travel to
the GPU machine, which has no reference sources).

1. reference_goldens.json -- the golden values the reference's own tests
   assert, read as text from src/test/SingleThreadedRKEmbeddedTest.cpp
   (test name, saved-state count, first/middle/last times and state
   components), plus the fixtures' parameters restated from
   src/test/{VanDerPol,Exponential,NBody,SpinningCubeNBody}Test.hpp.
2. nbody_*.npz -- runs of the reference compiled in place (oracle/_ref,
   single-threaded executor) on seeded N-body inputs: the input state, saved
   times and the final state, and right-hand sides.

Usage: python tests/golden/make_goldens.py [--skip-long]
"""
from __future__ import annotations

import json
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle as O  # noqa: E402

REF = O.REF_ROOT
TEST_CPP = os.path.join(REF, "src/test/SingleThreadedRKEmbeddedTest.cpp")


def parse_reference_goldens() -> dict:
    """Extracts EXPECT_EQ / EXPECT_DOUBLE_EQ expectations per TEST_F."""
    src = open(TEST_CPP).read()
    out = {}
    for m in re.finditer(r"TEST_F\(\w+,\s*(\w+)\)\s*\{(.*?)\n\}", src, re.S):
        name, body = m.group(1), m.group(2)
        tab = re.search(r"RKEmbeddedParallel<(\w+)>", body).group(1)
        case = {"tableau": tab.replace("BT", ""), "checks": []}
        n = re.search(r"EXPECT_EQ\((\d+), test\.output\.times\(\)\.size\(\)\)", body)
        case["n_saved"] = int(n.group(1))
        for e in re.finditer(r"EXPECT_DOUBLE_EQ\(\s*([-0-9.eE+]+),\s*(.*?)\);", body, re.S):
            val = float(e.group(1))
            expr = re.sub(r"\s+", "", e.group(2))
            case["checks"].append({"expr": expr, "value": val, "literal": e.group(1)})
        if "VanDerPol" in name:
            case["problem"] = "vanderpol"
        elif "Exponential" in name:
            case["problem"] = "exponential"
        elif "SpinningCube" in name:
            case["problem"] = "spinning_cube"
        else:
            case["problem"] = "nbody5"
        out[name] = case
    return out


# Fixture parameters (src/test/*Test.hpp), restated.
PROBLEMS = {
    "vanderpol": {"x0": [2.0, 0.0], "t0": 0.0, "tf": 2.0, "tol": 1e-10},
    "exponential": {"x0": [float(i) for i in range(10)], "t0": 0.0, "tf": 10.0, "tol": 1e-6},
    "nbody5": {
        "x0": [1.657666, 0.0, 0.0, 0.439775, -0.169717, 0.0, -1.268608, -0.267651, 0.0,
               -1.268608, 0.267651, 0.0, 0.439775, 0.169717, 0.0, 0.0, -0.593786, 0.0,
               1.822785, 0.128248, 0.0, 1.271564, 0.168645, 0.0, -1.271564, 0.168645, 0.0,
               -1.822785, 0.128248, 0.0],
        "n_particles": 5, "softening": 0.0, "t0": 0.0, "tf": 6.3, "tol": 1e-10},
    "spinning_cube": {"n_particles": 1024, "L": 1.0, "seed": 0},
}


def lib_ic():
    """Initial conditions from the GB300 library's host generators (the same
    generator the benchmark uses), loaded without a GPU."""
    import ode_prototyping_gb300 as G
    return G


def nbody_case(tag, tab, n, x0, soft, mass, t0, tf, tol, rhs=False):
    print(f"  {tag}: {tab} N={n} ...", flush=True)
    r = O.ref_integrate_nbody(tab, n, soft, mass, x0, t0, tf, tol, tol)
    d = {"x0": x0, "times": r.times, "final": r.states[-1],
         "mid": r.states[len(r.times) // 2],
         "meta": np.array([n, soft, mass, t0, tf, tol])}
    if rhs:
        d["rhs"] = O.ref_rhs(n, soft, mass, x0)
    np.savez_compressed(os.path.join(HERE, f"nbody_{tag}.npz"), tableau=np.array(tab), **d)
    print(f"    {len(r.times)} saved states", flush=True)


def main():
    if not os.path.exists(TEST_CPP):
        sys.exit("reference sources not present")
    O.build(ref=True)
    goldens = parse_reference_goldens()
    json.dump({"source": "src/test/SingleThreadedRKEmbeddedTest.cpp", "cases": goldens,
               "problems": PROBLEMS}, open(os.path.join(HERE, "reference_goldens.json"), "w"),
              indent=1)
    print(f"wrote {len(goldens)} reference golden cases")
    G = lib_ic()
    # small seeded systems (live-oracle sizes) and config 1 (N=1024)
    x64 = G.ic_uniform_ball(64, 11, 0.1)
    nbody_case("ball64_dopri5", "DOPRI5", 64, x64, 0.05, 1 / 64, 0.0, 0.5, 1e-10, rhs=True)
    nbody_case("ball64_rkf78", "RKF78", 64, x64, 0.05, 1 / 64, 0.0, 0.5, 1e-10)
    x256 = G.ic_plummer(256, 7, 1.0)
    nbody_case("plummer256_rkf78", "RKF78", 256, x256, 0.02, 1 / 256, 0.0, 0.25, 1e-8, rhs=True)
    if "--skip-long" not in sys.argv:
        x1024 = G.ic_uniform_ball(1024, 1, 0.1)
        nbody_case("config1_ball1024_dopri5", "DOPRI5", 1024, x1024, 0.01, 1 / 1024, 0.0, 1.0,
                   1e-10, rhs=True)


if __name__ == "__main__":
    main()
