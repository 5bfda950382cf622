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


def _need_ref(orc):
    if not orc.ref_available():
        pytest.skip("reference not compiled in place (oracle/_ref)")


def test_pi_controller_pinned_to_reference(orc):
    """The restated PI controller with Numerical Recipes' constants (safe
    0.9, alpha 0.2, beta 0, scale in [0.2, 10]) reproduces the reference's
    own Controller::success (NumericalRecipes/StepperDopr5.hpp:236-272,
    compiled in place) bit for bit on a sequence of error norms with
    successes, rejections, repeated rejections and a zero error."""
    _need_ref(orc)
    rng = np.random.default_rng(5)
    errs = np.concatenate([rng.uniform(0.01, 3.0, 200), [0.0, 2.5, 7.0, 0.3, 1e-9, 1.0, 1.0 + 1e-15,
                                                         50.0, 0.999, 1e-3]])
    got = orc.pi_sequence(0.9, 0.2, 0.0, 0.2, 10.0, errs, 1e-3)
    ref = orc.ref_dopri5_controller(errs, 1e-3)
    np.testing.assert_array_equal(got, ref)


def test_dopri5_dense_pinned_to_reference(orc):
    """The restated DOPRI5 dense output reproduces the reference's own
    prepare_dense / dense_out (NumericalRecipes/StepperDopr5.hpp:179-219,
    compiled in place) bit for bit, at interior points and both ends."""
    _need_ref(orc)
    rng = np.random.default_rng(6)
    n = 37
    y0, y1 = rng.standard_normal(n), rng.standard_normal(n)
    ks = rng.standard_normal(7 * n)
    h, t_new = 0.0137, 2.5
    ts = np.concatenate([[t_new - h], np.sort(rng.uniform(t_new - h, t_new, 9)), [t_new]])
    np.testing.assert_array_equal(orc.dopri5_dense(y0, y1, ks, h, t_new, ts),
                                  orc.ref_dopri5_dense(y0, y1, ks, h, t_new, ts))


def test_pi_session_integrates_reference_problems(orc):
    """The oracle loop with the PI controller (the reference integrator's
    constants, beta 0.04) reaches tf on x' = x (the reference's exponential
    problem) and on van der Pol with no more rejections than the elementary
    controller, accurate to the tolerance's order; with beta = 0 and no
    rejection it takes as many steps as the elementary controller."""
    ode = orc.small_ode(orc.ODE_EXPONENTIAL, 10)
    x0 = np.linspace(0.5, 1.5, 10)
    tol = 1e-10
    s = orc.Session("DOPRI5", ode, x0, 0.0, 1.0, tol, tol, controller="pi", pi_beta=0.04)
    times, states = s.run()
    st = s.stats()
    s.close()
    r = orc.integrate("DOPRI5", ode, x0, 0.0, 1.0, tol, tol)
    assert times[-1] == 1.0
    assert st["n_rejected"] <= r.stats["n_rejected"]
    assert np.max(np.abs(states[-1] - np.e * x0) / (np.e * x0)) <= 1e3 * tol
    s0 = orc.Session("DOPRI5", ode, x0, 0.0, 1.0, tol, tol, controller="pi", pi_beta=0.0)
    t0s, _ = s0.run()
    st0 = s0.stats()
    s0.close()
    if st0["n_rejected"] == 0 and r.stats["n_rejected"] == 0:
        # the same formula (evaluated as safe * err^-alpha instead of
        # safe / err^alpha): the same number of steps
        assert abs(len(t0s) - len(r.times)) <= 1
    vdp = orc.small_ode(orc.ODE_VANDERPOL, 2)
    P = GOLD["problems"]["vanderpol"]
    for tab in ("DOPRI5", "RKF78"):
        sv = orc.Session(tab, vdp, np.array(P["x0"]), P["t0"], P["tf"], P["tol"], P["tol"],
                         controller="pi")
        tv, xv = sv.run()
        stv = sv.stats()
        sv.close()
        rv = orc.integrate(tab, vdp, np.array(P["x0"]), P["t0"], P["tf"], P["tol"], P["tol"],
                           capacity=1 << 16)
        assert tv[-1] == P["tf"]
        assert stv["n_rejected"] <= rv.stats["n_rejected"]
        assert np.max(np.abs(xv[-1] - rv.states[-1])) <= 1e3 * P["tol"] * (1 + np.abs(xv[-1]).max())


def test_dense_session_on_the_exponential(orc):
    """Dense output from the oracle loop on x' = x (DOPRI5, tol 1e-10): the
    continuous extension is accurate to the tolerance's order at times
    between steps, and equals the step's own state at a step's end time."""
    ode = orc.small_ode(orc.ODE_EXPONENTIAL, 10)
    x0 = np.linspace(0.5, 1.5, 10)
    ts = np.linspace(0.01, 0.99, 23)
    s = orc.Session("DOPRI5", ode, x0, 0.0, 1.0, 1e-10, 1e-10, dense_times=ts)
    times, states = s.run()
    dense = s.dense()
    s.close()
    assert dense.shape == (len(ts), 10)
    exact = np.exp(ts)[:, None] * x0[None, :]
    assert np.max(np.abs(dense - exact) / exact) <= 1e-8
    s2 = orc.Session("DOPRI5", ode, x0, 0.0, 1.0, 1e-10, 1e-10, dense_times=times[3:6])
    s2.run()
    np.testing.assert_allclose(s2.dense(), states[3:6], rtol=1e-15, atol=0)
    s2.close()


def test_oracle_plummer_initial_conditions_match_library(orc, gb):
    """The CPU-baseline legs build their inputs with the oracle's copy of the
    seeded Plummer sampler; it gives the library's bits (host code only)."""
    for n, seed in ((1024, 1), (16384, 101), (333, 7)):
        np.testing.assert_array_equal(orc.ic_plummer(n, seed, 1.0), gb.ic_plummer(n, seed, 1.0))
