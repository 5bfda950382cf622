"""CPU tests: the oracle (C restatement of the reference) pinned against the
reference's own golden values and against the reference compiled in place."""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN

GOLD = json.load(open(os.path.join(GOLDEN, "reference_goldens.json")))


def _problem(orc, case):
    P = GOLD["problems"][case["problem"]]
    if case["problem"] == "vanderpol":
        return orc.small_ode(orc.ODE_VANDERPOL, 2), np.array(P["x0"]), P["t0"], P["tf"], P["tol"]
    if case["problem"] == "exponential":
        return (orc.small_ode(orc.ODE_EXPONENTIAL, 10), np.array(P["x0"]), P["t0"], P["tf"],
                P["tol"])
    if case["problem"] == "nbody5":
        ode, _ = orc.nbody_ode(5, 0.0)
        return ode, np.array(P["x0"]), P["t0"], P["tf"], P["tol"]
    n = P["n_particles"]
    x0 = orc.spinning_cube(n, P["L"], P["seed"])
    soft = 4.0 * P["L"] / np.sqrt(n)
    ode, _ = orc.nbody_ode(n, soft)
    return ode, x0, 0.0, np.sqrt(P["L"] ** 3 / n), soft


def eval_check(expr: str, times, states, n_var: int, n_particles: int = 1024) -> float:
    """Evaluates one golden expression of the reference test, e.g.
    test.output.states()[test.output.states().size()/2][test.n_var/2]."""
    e = expr.replace("test.output.times().size()", str(len(times)))
    e = e.replace("test.output.states().size()", str(len(states)))
    e = e.replace("test.output.times()", "times").replace("test.output.states()", "states")
    e = e.replace("test.n_var", str(n_var)).replace("n_particles", str(n_particles))
    e = e.replace(".front()", "[0]").replace(".back()", "[-1]")
    e = e.replace("/", "//")
    return float(eval(e, {"times": times, "states": states}))


@pytest.mark.parametrize("name", sorted(GOLD["cases"]))
def test_oracle_matches_reference_goldens(orc, name):
    case = GOLD["cases"][name]
    ode, x0, t0, tf, tol = _problem(orc, case)
    r = orc.integrate(case["tableau"], ode, x0, t0, tf, tol, tol, capacity=1 << 18)
    assert len(r.times) == case["n_saved"]
    for chk in case["checks"]:
        got = eval_check(chk["expr"], r.times, r.states, int(ode.n_var))
        # EXPECT_DOUBLE_EQ: within 4 ULP
        assert got == pytest.approx(chk["value"], rel=4 * np.finfo(float).eps, abs=0), chk["expr"]


def test_oracle_threadpool_same_step_count(orc):
    case = GOLD["cases"]["RKF78NBodyConsistencyTest"]
    ode, x0, t0, tf, tol = _problem(orc, case)
    r = orc.integrate("RKF78", ode, x0, t0, tf, tol, tol, n_threads=4)
    assert len(r.times) == 172
    # ThreadPoolRKEmbeddedTest.cpp:343-352 relaxes the final state to tol
    np.testing.assert_allclose(r.states[-1][[0, 3, 6, 9, 12]],
                               [1.6573213121279662, 0.46802604979077689, -1.2481480178176445,
                                -1.2883624086182086, 0.41116306451711232], atol=tol, rtol=0)


@pytest.mark.parametrize("tag", ["ball64_dopri5", "ball64_rkf78", "plummer256_rkf78",
                                 "config1_ball1024_dopri5"])
def test_oracle_matches_reference_runs(orc, tag):
    """Bit-for-bit agreement with the reference compiled in place (fixture)."""
    path = os.path.join(GOLDEN, f"nbody_{tag}.npz")
    if not os.path.exists(path):
        pytest.skip("fixture not generated")
    d = np.load(path)
    n, soft, mass, t0, tf, tol = d["meta"]
    n = int(n)
    if n > 256:
        pytest.skip("long oracle run; covered on the GPU machine by the parity tests")
    ode, _ = orc.nbody_ode(n, soft, mass)
    r = orc.integrate(str(d["tableau"]), ode, d["x0"], t0, tf, tol, tol)
    assert len(r.times) == len(d["times"])
    np.testing.assert_array_equal(r.times, d["times"])
    np.testing.assert_array_equal(r.states[-1], d["final"])
    if "rhs" in d:
        np.testing.assert_array_equal(orc.rhs(ode, d["x0"]), d["rhs"])


def test_oracle_rhs_config1_fixture(orc):
    path = os.path.join(GOLDEN, "nbody_config1_ball1024_dopri5.npz")
    if not os.path.exists(path):
        pytest.skip("fixture not generated")
    d = np.load(path)
    n, soft, mass = int(d["meta"][0]), d["meta"][1], d["meta"][2]
    ode, _ = orc.nbody_ode(n, soft, mass)
    np.testing.assert_array_equal(orc.rhs(ode, d["x0"]), d["rhs"])


def test_oracle_rows_equal_serial_pair_order(orc):
    """Owner-form row sums equal the reference's serial pair-order sums."""
    rng = np.random.default_rng(3)
    n = 97
    x = rng.standard_normal(6 * n)
    ode, _ = orc.nbody_ode(n, 0.03, 1.0 / n)
    full = orc.rhs(ode, x)[3 * n:].reshape(n, 3)
    rows = np.array([0, 1, 50, 96])
    np.testing.assert_array_equal(orc.acc_rows(ode, x, rows), full[rows])


def test_oracle_energy_two_body(orc):
    x = np.array([0.5, 0, 0, -0.5, 0, 0, 0, 0.1, 0, 0, -0.1, 0.0])
    ode, _ = orc.nbody_ode(2, 0.0, 0.5)
    e = orc.energy(ode, x)
    assert e["pe"] == pytest.approx(-0.25)
    assert e["ke"] == pytest.approx(0.5 * 0.5 * 0.01 * 2)
    np.testing.assert_allclose(e["p"], 0, atol=1e-15)
    assert e["l"][2] == pytest.approx(0.5 * (0.5 * 0.1) * 2)


def test_oracle_budget_guard(orc):
    """A bounded attempt budget stops the loop (the reference has none)."""
    ode = orc.small_ode(orc.ODE_VANDERPOL, 2)
    r = orc.integrate("HE21", ode, np.array([2.0, 0.0]), 0.0, 2.0, 1e-10, 1e-10, max_attempts=10)
    assert r.stats["status"] == 2 and r.stats["n_attempts"] == 10


def test_reference_build_agrees_when_present(orc):
    if not orc.ref_available():
        pytest.skip("reference not compiled here")
    x = orc.spinning_cube(16, 1.0, 0)
    ode, _ = orc.nbody_ode(16, 0.5, 1 / 16)
    np.testing.assert_array_equal(orc.rhs(ode, x), orc.ref_rhs(16, 0.5, 1 / 16, x))
    r1 = orc.integrate("DOPRI5", ode, x, 0.0, 0.1, 1e-9, 1e-9)
    r2 = orc.ref_integrate_nbody("DOPRI5", 16, 0.5, 1 / 16, x, 0.0, 0.1, 1e-9, 1e-9)
    np.testing.assert_array_equal(r1.times, r2.times)
    np.testing.assert_array_equal(r1.states, r2.states)
