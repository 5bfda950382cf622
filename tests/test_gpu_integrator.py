"""GPU parity of the device-resident adaptive integrator against the
reference's golden values, the reference's own runs (fixtures) and the live
oracle.  Bars: same accepted-step count, final state within 10x the
tolerance (bitwise where stated)."""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu

GOLD = json.load(open(os.path.join(GOLDEN, "reference_goldens.json")))


def run(gb, tab, n, soft, mass, x0, t0, tf, tol, **exe_kw):
    exe = gb.Gb300Executor(**exe_kw)
    ode = gb.NBodyODE(n, soft, mass)
    out = gb.RawOutput()
    st = gb.RKEmbeddedParallel(tab).integrate(x0, t0, tf, tol, tol, ode, out, exe)
    return np.array(out.times()), np.array(out.states()), st


@pytest.mark.parametrize("exe_kw", [{}, {"exact": True}, {"fsal": False},
                                    {"attempts_per_sync": 1}, {"attempts_per_sync": 64}])
def test_five_body_rkf78_golden(gb, torch_cuda, exe_kw):
    """RKF78NBodyConsistencyTest (SingleThreadedRKEmbeddedTest.cpp:306-340) with
    the CUDA executor's tolerances (CudaRKEmbeddedTest.cu:309-354)."""
    P = GOLD["problems"]["nbody5"]
    case = GOLD["cases"]["RKF78NBodyConsistencyTest"]
    times, states, st = run(gb, "RKF78", 5, 0.0, 1.0, np.array(P["x0"]), P["t0"], P["tf"],
                            P["tol"], **exe_kw)
    assert len(times) == case["n_saved"] == 172
    tol = P["tol"]
    mid_tol = 1.657666 * tol * len(times) / 2
    assert times[0] == 0.0 and times[-1] == 6.3
    assert times[len(times) // 2] == pytest.approx(3.1699354066499978, abs=mid_tol)
    np.testing.assert_allclose(states[-1][[0, 3, 6, 9, 12]],
                               [1.6573213121279662, 0.46802604979077689, -1.2481480178176445,
                                -1.2883624086182086, 0.41116306451711232], atol=tol, rtol=0)
    assert st["n_accepted"] == 171


def test_spinning_cube_rkf78_golden(gb, orc, torch_cuda):
    """RKF78SpinningCubeNBodyTest (SingleThreadedRKEmbeddedTest.cpp:342-382) with
    CudaRKEmbeddedTest.cu:356-403's 10*DBL_EPSILON tolerance."""
    n = 1024
    x0 = orc.spinning_cube(n, 1.0, 0)
    soft = 4.0 / np.sqrt(n)
    times, states, _ = run(gb, "RKF78", n, soft, 1.0, x0, 0.0, np.sqrt(1.0 / n), soft)
    assert len(times) == 4
    eps10 = 10 * np.finfo(float).eps
    assert times[-1] == 0.03125
    assert times[2] == pytest.approx(0.0099564200160493655, abs=eps10)
    idx = [0, n // 4, n // 2, 3 * n // 4]
    np.testing.assert_allclose(states[2][idx], [0.36755281580363885, 0.85638183296447723,
                                                0.41417946857300797, 0.028148414608021005],
                               atol=eps10, rtol=0)
    np.testing.assert_allclose(states[-1][idx], [0.16121502269618729, 0.71404096847054921,
                                                 0.59500181799963803, 0.42875743462583493],
                               atol=eps10, rtol=0)


@pytest.mark.parametrize("tag", ["ball64_dopri5", "ball64_rkf78", "plummer256_rkf78",
                                 "config1_ball1024_dopri5"])
@pytest.mark.parametrize("exact", [False, True])
def test_matches_reference_runs(gb, torch_cuda, tag, exact):
    path = os.path.join(GOLDEN, f"nbody_{tag}.npz")
    if not os.path.exists(path):
        pytest.skip("fixture missing")
    d = np.load(path)
    n, soft, mass, t0, tf, tol = d["meta"]
    n = int(n)
    times, states, st = run(gb, str(d["tableau"]), n, soft, mass, d["x0"], t0, tf, tol,
                            exact=exact)
    # the parity bar: the same accepted-step count and a final state within
    # 10x the tolerance
    assert len(times) == len(d["times"]), (len(times), len(d["times"]))
    assert np.max(np.abs(states[-1] - d["final"])) <= 10 * tol
    if exact:
        # the reference's arithmetic: its step times bit for bit
        np.testing.assert_array_equal(times, d["times"])
    else:
        # FP64 stages with the refined-rsqrt pair term (a few ulp per term):
        # the step sizes follow err^(-1/(1+q)) of a near-cancelling error
        # estimate, so the accepted times drift from the reference's by
        # ~1e-7 relative over a run
        np.testing.assert_allclose(times, d["times"], rtol=1e-6, atol=10 * tol)


@pytest.mark.parametrize("n,tab,seed", [(48, "DOPRI5", 1), (100, "RKF78", 2), (33, "RKF45", 3),
                                        (70, "DVERK", 4), (20, "HE21", 5)])
def test_matches_live_oracle(gb, orc, torch_cuda, n, tab, seed):
    x0 = gb.ic_plummer(n, seed)
    soft, tol, tf = 0.05, 1e-8, 0.3 if tab != "HE21" else 0.02
    ode, _ = orc.nbody_ode(n, soft, 1.0 / n)
    r = orc.integrate(tab, ode, x0, 0.0, tf, tol, tol, capacity=1 << 16)
    times, states, _ = run(gb, tab, n, soft, 1.0 / n, x0, 0.0, tf, tol)
    assert len(times) == len(r.times)
    assert np.max(np.abs(states[-1] - r.states[-1])) <= 10 * tol


def test_fsal_is_bit_identical(gb, torch_cuda):
    n = 200
    x0 = gb.ic_uniform_ball(n, 9, 0.1)
    a = run(gb, "DOPRI5", n, 0.02, 1.0 / n, x0, 0.0, 0.2, 1e-9, fsal=True)
    b = run(gb, "DOPRI5", n, 0.02, 1.0 / n, x0, 0.0, 0.2, 1e-9, fsal=False)
    np.testing.assert_array_equal(a[0], b[0])
    np.testing.assert_array_equal(a[1], b[1])
    assert a[2]["n_rhs"] < b[2]["n_rhs"]
    assert a[2]["n_rhs_saved"] > 0


@pytest.mark.parametrize("n,zero_mass", [(2, False), (3, False), (300, True)])
def test_element_epilogue_is_bit_identical(gb, torch_cuda, n, zero_mass):
    """Kernels with two or more lanes per body finish a stage one state
    element per thread; one-lane kernels one body per thread.  Both do every
    element's FP64 arithmetic in the same order, so in exact mode (serial
    error norm), with pair sums that no partner order can change -- at most
    two partners per body, or zero masses -- one- and two-lane runs, with or
    without a cluster split, agree bit for bit.  N = 300 puts more elements
    in a CTA than it has threads."""
    rng = np.random.default_rng(17 + n)
    x0 = np.concatenate([rng.uniform(-1, 1, 3 * n), rng.uniform(-0.3, 0.3, 3 * n)])
    if zero_mass:
        ode = gb.NBodyODE(n, 0.05, masses=gb.to_device(np.zeros(n)))
    else:
        ode = gb.NBodyODE(n, 0.05, 1.0 / n)
    tab, tol, tf = "RKF78", 1e-10, 0.5
    runs = {}
    for split, lanes in [(1, 1), (1, 2), (4, 1), (4, 2)]:
        exe = gb.Gb300Executor(precision="f64", exact=True, tile=gb.tiling(split, lanes, 0))
        it = gb.Integrator(tab, ode, exe)
        it.start(x0, 0.0, tf, tol, tol)
        geo = it.geometry()
        it.close()
        assert (geo["j_split"], geo["lanes"]) == (split, lanes)
        out = gb.RawOutput()
        st = gb.RKEmbeddedParallel(tab).integrate(x0, 0.0, tf, tol, tol, ode, out, exe)
        runs[(split, lanes)] = (np.array(out.times()), np.array(out.states()), st["n_accepted"])
    t0, s0, a0 = runs[(1, 1)]
    assert a0 >= 2
    for key, (t, s, a) in runs.items():
        assert a == a0, key
        np.testing.assert_array_equal(t, t0, err_msg=str(key))
        np.testing.assert_array_equal(s, s0, err_msg=str(key))


def _mixed_run(gb, ode, x0, tf, tol, tile=None, variant=0, spatial_sort=0, tab="DOPRI5",
               attempts_per_sync=16):
    exe = gb.Gb300Executor(precision="mixed", tile=tile if tile is not None
                           else gb.tiling(mixed_variant=variant), spatial_sort=spatial_sort,
                           attempts_per_sync=attempts_per_sync)
    out = gb.RawOutput()
    st = gb.RKEmbeddedParallel(tab).integrate(x0, 0.0, tf, tol, tol, ode, out, exe)
    return np.array(out.times()), np.array(out.states()), st


@pytest.mark.parametrize("n,gen", [(16384, "plummer"), (8333, "cold"), (12000, "binary")])
def test_split_stage_tile_culling_is_bit_identical(gb, torch_cuda, n, gen):
    """The partner-chunk stage on Morton-sorted bodies skips the close-pair
    test for 64-partner quarter tiles whose boxes are far from every body of a
    warp; the terms it adds there are the ones the test would have kept, so whole RKF78 trajectories
    with and without the culling (re-sorted every 4 attempts) agree bit for
    bit, and both follow the FP64 integration to the mixed-precision bound."""
    x0 = {"plummer": lambda: gb.ic_plummer(n, 5), "cold": lambda: gb.ic_cold_sphere(n, 6, 0.01),
          "binary": lambda: gb.ic_binary_plummer(n, 7, 0.1, 1e-3, 1e-2)}[gen]()
    soft, tol, tf = 0.005, 1e-9, 0.05
    ode = gb.NBodyODE(n, soft, 1.0 / n)
    a = _mixed_run(gb, ode, x0, tf, tol, tab="RKF78", attempts_per_sync=4)
    b = _mixed_run(gb, ode, x0, tf, tol, tab="RKF78", attempts_per_sync=4, spatial_sort=2)
    np.testing.assert_array_equal(a[0], b[0])
    np.testing.assert_array_equal(a[1], b[1])
    out64 = gb.RawOutput()
    gb.RKEmbeddedParallel("RKF78").integrate(x0, 0.0, tf, tol, tol, ode, out64,
                                             gb.Gb300Executor(precision="f64"))
    assert abs(len(a[0]) - len(out64.times())) <= 2
    assert np.max(np.abs(a[1][-1] - np.array(out64.states()[-1]))) <= 1e-6


@pytest.mark.parametrize("n", [8192, 8333])
def test_split_stage_is_deterministic_and_tracks_fp64(gb, torch_cuda, n):
    """From N = 8192 the packed mixed stage runs as independent partner chunks
    whose sums the last-arriving CTA adds in chunk order.  Runs are bit for
    bit repeatable whatever the arrival order; the chunked form, the cluster
    form (8 x 2 lanes), an uneven chunk count (5) and the two-bodies-per-thread
    loop all follow the FP64 integration to the mixed-precision bound.
    N = 8333 leaves a ragged last tile and an odd partner count."""
    soft, tol, tf = 0.01, 1e-9, 0.02
    x0 = gb.ic_plummer(n, 77)
    ode = gb.NBodyODE(n, soft, 1.0 / n)
    exe = gb.Gb300Executor(precision="mixed")
    it = gb.Integrator("DOPRI5", ode, exe)
    it.start(x0, 0.0, tf, tol, tol)
    geo = it.geometry()
    it.close()
    assert (geo["j_split"], geo["lanes"]) == (8, 1)
    a = _mixed_run(gb, ode, x0, tf, tol)
    b = _mixed_run(gb, ode, x0, tf, tol)
    np.testing.assert_array_equal(a[0], b[0])
    np.testing.assert_array_equal(a[1], b[1])
    out64 = gb.RawOutput()
    gb.RKEmbeddedParallel("DOPRI5").integrate(x0, 0.0, tf, tol, tol, ode, out64,
                                              gb.Gb300Executor(precision="f64"))
    ref = np.array(out64.states()[-1])
    runs = {"split": a, "cluster": _mixed_run(gb, ode, x0, tf, tol, tile=gb.tiling(8, 2, 0)),
            "split5": _mixed_run(gb, ode, x0, tf, tol, tile=gb.tiling(5, 1, 0)),
            "pairs2": _mixed_run(gb, ode, x0, tf, tol, variant=2),
            "unsorted": _mixed_run(gb, ode, x0, tf, tol, spatial_sort=3)}
    for name, (t, s, st) in runs.items():
        assert t[-1] == tf, name
        assert abs(len(t) - len(out64.times())) <= 2, name
        assert np.max(np.abs(s[-1] - ref)) <= 1e-6, name


def test_vector_tolerances_match_scalar(gb, torch_cuda):
    n = 64
    x0 = gb.ic_plummer(n, 3)
    exe = gb.Gb300Executor()
    ode = gb.NBodyODE(n, 0.05, 1.0 / n)
    o1, o2 = gb.RawOutput(), gb.RawOutput()
    gb.RKEmbeddedParallel("DOPRI5").integrate(x0, 0.0, 0.2, 1e-9, 1e-9, ode, o1, exe)
    tv = np.full(6 * n, 1e-9)
    gb.RKEmbeddedParallel("DOPRI5").integrate(x0, 0.0, 0.2, tv, tv, ode, o2, exe)
    np.testing.assert_array_equal(np.array(o1.states()), np.array(o2.states()))


@pytest.mark.parametrize("variant", [0, 1, 2, 3])
def test_mixed_precision_integrator(gb, torch_cuda, variant):
    """Every mixed pair loop (auto, scalar, one or two packed pairs per
    thread) tracks the FP64 path."""
    n = 1024
    x0 = gb.ic_uniform_ball(n, 1, 0.1)
    tol = 1e-9
    t64, s64, st64 = run(gb, "DOPRI5", n, 0.01, 1.0 / n, x0, 0.0, 0.1, tol)
    tmx, smx, stmx = run(gb, "DOPRI5", n, 0.01, 1.0 / n, x0, 0.0, 0.1, tol, precision="mixed",
                         tile=gb.tiling(mixed_variant=variant))
    assert abs(len(tmx) - len(t64)) <= max(2, len(t64) // 20)
    assert np.max(np.abs(smx[-1] - s64[-1])) <= 1e-6


def test_budget_and_nonfinite_status(gb, torch_cuda):
    n = 32
    x0 = gb.ic_plummer(n, 1)
    exe = gb.Gb300Executor(max_attempts=5)
    it = gb.Integrator("DOPRI5", gb.NBodyODE(n, 0.05, 1.0 / n), exe)
    it.start(x0, 0.0, 10.0, 1e-12, 1e-12)
    assert it.advance() == gb.GB_ERR_BUDGET
    assert it.stats()["n_attempts"] == 5
    it.close()
    bad = x0.copy()
    bad[7] = np.nan
    it = gb.Integrator("DOPRI5", gb.NBodyODE(n, 0.05, 1.0 / n), gb.Gb300Executor())
    it.start(bad, 0.0, 1.0, 1e-9, 1e-9)
    assert it.advance() == gb.GB_ERR_NOT_FINITE
    it.close()


def test_pi_controller_runs(gb, torch_cuda):
    n = 256
    x0 = gb.ic_plummer(n, 6)
    t_ref, s_ref, st_ref = run(gb, "DOPRI5", n, 0.02, 1.0 / n, x0, 0.0, 0.3, 1e-9)
    t_pi, s_pi, st_pi = run(gb, "DOPRI5", n, 0.02, 1.0 / n, x0, 0.0, 0.3, 1e-9, controller="pi")
    assert t_pi[-1] == pytest.approx(0.3)
    assert np.max(np.abs(s_pi[-1] - s_ref[-1])) <= 1e-7


@pytest.mark.parametrize("tab,n,soft,tf,beta", [("DOPRI5", 64, 0.05, 0.5, 0.04),
                                                ("RKF78", 128, 0.02, 0.3, 0.04),
                                                ("DOPRI5", 100, 0.03, 0.4, 0.08)])
def test_pi_controller_matches_oracle(gb, orc, torch_cuda, tab, n, soft, tf, beta):
    """The device PI controller against the oracle's restatement of
    Controller::success (NumericalRecipes/StepperDopr5.hpp:236-272 with the
    reference integrator's constants, pinned to the reference's own
    controller on the CPU): same accepted-step count, final state within
    10x the tolerance (exact mode: serial pair sums, as the oracle)."""
    x0 = gb.ic_plummer(n, 17)
    tol = 1e-9
    times, states, st = run(gb, tab, n, soft, 1.0 / n, x0, 0.0, tf, tol, controller="pi",
                            pi_beta=beta, exact=True)
    ode, _ = orc.nbody_ode(n, soft, 1.0 / n)
    s = orc.Session(tab, ode, x0, 0.0, tf, tol, tol, controller="pi", pi_beta=beta)
    o_times, o_states = s.run()
    o_st = s.stats()
    s.close()
    assert len(times) == len(o_times)
    assert st["n_rejected"] == o_st["n_rejected"]
    assert times[-1] == o_times[-1] == tf
    assert np.max(np.abs(states[-1] - o_states[-1])) <= 10 * tol


def test_dopri5_dense_output_matches_oracle(gb, orc, torch_cuda):
    """Dense output on the device against the oracle's restatement of
    prepare_dense / dense_out (NumericalRecipes/StepperDopr5.hpp:179-219,
    pinned bit for bit to the reference's own code on the CPU) on the same
    accepted steps (exact mode: the trajectory is the reference's, bit for
    bit): every output within 1e-12 of the oracle's, relative to the state."""
    n, soft, tol, tf = 64, 0.05, 1e-9, 0.3
    x0 = gb.ic_plummer(n, 21)
    ode = gb.NBodyODE(n, soft, 1.0 / n)
    times = np.sort(np.concatenate([np.linspace(0.013, 0.29, 17), [0.3]]))
    it = gb.Integrator("DOPRI5", ode, gb.Gb300Executor(exact=True, attempts_per_sync=4))
    it.set_dense_output(times)
    it.start(x0, 0.0, tf, tol, tol)
    assert it.advance(0) == 0
    dense = it.dense_output()
    it.close()
    ode_o, _ = orc.nbody_ode(n, soft, 1.0 / n)
    s = orc.Session("DOPRI5", ode_o, x0, 0.0, tf, tol, tol, dense_times=times)
    s.run()
    o_dense = s.dense()
    s.close()
    assert dense.shape == o_dense.shape == (len(times), 6 * n)
    scale = np.max(np.abs(o_dense), axis=1, keepdims=True)
    assert np.max(np.abs(dense - o_dense) / scale) <= 1e-12


def test_enqueue_and_state(gb, torch_cuda):
    n = 128
    x0 = gb.ic_plummer(n, 2)
    it = gb.Integrator("RKF78", gb.NBodyODE(n, 0.02, 1.0 / n), gb.Gb300Executor())
    it.start(x0, 0.0, 0.1, 1e-9, 1e-9)
    it.enqueue(2)
    it.sync()
    s = it.stats()
    assert s["n_attempts"] >= 1
    x, t = it.state()
    assert t == s["t"] and x.shape[0] == 6 * n
    it.close()


@pytest.mark.parametrize("tag", ["ball64_dopri5", "ball64_rkf78", "plummer256_rkf78",
                                 "config1_ball1024_dopri5"])
def test_exact_mode_reproduces_reference_bits(gb, torch_cuda, tag):
    """Exact mode: serial partner order, serial norm, IEEE stage sums and a
    correctly rounded pow in the step-size formulas -- the whole accepted
    trajectory equals the reference's single-threaded run bit for bit."""
    path = os.path.join(GOLDEN, f"nbody_{tag}.npz")
    if not os.path.exists(path):
        pytest.skip("fixture missing")
    d = np.load(path)
    n, soft, mass, t0, tf, tol = d["meta"]
    n = int(n)
    times, states, _ = run(gb, str(d["tableau"]), n, soft, mass, d["x0"], t0, tf, tol,
                           exact=True)
    np.testing.assert_array_equal(times, d["times"])
    np.testing.assert_array_equal(states[-1], d["final"])
    np.testing.assert_array_equal(states[len(states) // 2], d["mid"])


def test_sorted_and_unsorted_mixed_paths_agree(gb, torch_cuda):
    n = 3000
    x0 = gb.ic_plummer(n, 12)
    tol = 1e-9
    t64, s64, _ = run(gb, "RKF78", n, 0.005, 1.0 / n, x0, 0.0, 0.05, tol)
    ta, sa, _ = run(gb, "RKF78", n, 0.005, 1.0 / n, x0, 0.0, 0.05, tol, precision="mixed",
                    spatial_sort=True, attempts_per_sync=4)
    tb, sb, _ = run(gb, "RKF78", n, 0.005, 1.0 / n, x0, 0.0, 0.05, tol, precision="mixed",
                    spatial_sort=False)
    assert abs(len(ta) - len(t64)) <= 2 and abs(len(tb) - len(t64)) <= 2
    assert np.max(np.abs(sa[-1] - s64[-1])) <= 1e-6
    assert np.max(np.abs(sb[-1] - s64[-1])) <= 1e-6


def test_dopri5_dense_output(gb, torch_cuda):
    """Dense output between steps (DOPRI5 continuous extension): states at the
    requested times agree with integrations stopped exactly there, and at a
    step's own end time with that step's state."""
    n, soft, tol, tf = 64, 0.05, 1e-9, 0.3
    x0 = gb.ic_plummer(n, 21)
    ode = gb.NBodyODE(n, soft, 1.0 / n)
    out = gb.RawOutput()
    it = gb.Integrator("DOPRI5", ode, gb.Gb300Executor(attempts_per_sync=4), record=True)
    probe = gb.RawOutput()
    gb.RKEmbeddedParallel("DOPRI5").integrate(x0, 0.0, tf, tol, tol, ode, probe,
                                              gb.Gb300Executor())
    step_t = np.array(probe.times())
    times = np.sort(np.concatenate([np.linspace(0.013, 0.29, 17), step_t[3:6]]))
    it.set_dense_output(times)
    it.start(x0, 0.0, tf, tol, tol, out)
    assert it.advance(0, out) == 0
    dense = it.dense_output()
    it.close()
    assert dense.shape == (len(times), 6 * n)
    for j, t in enumerate(times):
        ref = gb.RawOutput()
        gb.RKEmbeddedParallel("DOPRI5").integrate(x0, 0.0, t, 1e-12, 1e-12, ode, ref,
                                                  gb.Gb300Executor())
        assert np.max(np.abs(dense[j] - ref.states()[-1])) <= 100 * tol, t
    states = np.array(out.states())
    for t in step_t[3:6]:
        k = int(np.where(np.array(out.times()) == t)[0][0])
        j = int(np.where(times == t)[0][0])
        np.testing.assert_allclose(dense[j], states[k], rtol=0, atol=1e-13)


def test_mixed_integrator_per_body_masses(gb, torch_cuda):
    """Per-body masses run the scalar FP32 pair loop in the mixed path; the
    integration tracks the FP64 path with the same masses."""
    n = 700
    x0 = gb.ic_plummer(n, 31)
    m = np.random.default_rng(6).uniform(0.5, 1.5, n)
    m /= m.sum()
    md = gb.to_device(m)
    tol = 1e-9
    ode = gb.NBodyODE(n, 0.02, masses=md)
    out64, outmx = gb.RawOutput(), gb.RawOutput()
    gb.RKEmbeddedParallel("DOPRI5").integrate(x0, 0.0, 0.1, tol, tol, ode, out64,
                                              gb.Gb300Executor(precision="f64"))
    gb.RKEmbeddedParallel("DOPRI5").integrate(x0, 0.0, 0.1, tol, tol, ode, outmx,
                                              gb.Gb300Executor(precision="mixed"))
    assert abs(len(outmx.times()) - len(out64.times())) <= 2
    assert np.max(np.abs(np.array(outmx.states()[-1]) - np.array(out64.states()[-1]))) <= 1e-6


def test_dopri5_dense_output_mixed(gb, torch_cuda):
    """Dense output in mixed precision agrees with the FP64 path's."""
    n, soft, tol, tf = 512, 0.02, 1e-9, 0.1
    x0 = gb.ic_plummer(n, 22)
    ode = gb.NBodyODE(n, soft, 1.0 / n)
    times = np.linspace(0.01, 0.09, 9)
    dense = {}
    for prec in ("f64", "mixed"):
        it = gb.Integrator("DOPRI5", ode, gb.Gb300Executor(precision=prec, attempts_per_sync=4))
        it.set_dense_output(times)
        it.start(x0, 0.0, tf, tol, tol)
        assert it.advance(0) == 0
        dense[prec] = it.dense_output()
        it.close()
    assert dense["mixed"].shape == (len(times), 6 * n)
    assert np.max(np.abs(dense["mixed"] - dense["f64"])) <= 1e-6


@pytest.mark.parametrize("precision", ["f64", "mixed"])
def test_single_body_moves_uniformly(gb, torch_cuda, precision):
    """A lone body has zero acceleration: the integrator carries it along its
    velocity to tf."""
    x0 = np.array([0.1, -0.2, 0.3, 0.5, 0.25, -1.0])
    out = gb.RawOutput()
    gb.RKEmbeddedParallel("DOPRI5").integrate(x0, 0.0, 1.0, 1e-9, 1e-9, gb.NBodyODE(1, 0.05, 1.0),
                                              out, gb.Gb300Executor(precision=precision))
    xf = np.array(out.states()[-1])
    np.testing.assert_allclose(xf[:3], x0[:3] + x0[3:], rtol=0, atol=1e-12)
    np.testing.assert_array_equal(xf[3:], x0[3:])


def test_bounded_host_wait_times_out(gb, torch_cuda):
    """Every host wait for the device is bounded: a graph replay of 16 FP64
    RKF78 attempts at N = 8192 (about 1.3 s of device work) with a 0.2 s bound
    returns GB_ERR_TIMEOUT instead of blocking, and the integrator can still
    be closed (the failure is made on the host; nothing faults).  The bound
    leaves the start-up wait (two right-hand sides, ~13 ms) well inside it."""
    n = 8192
    x0 = gb.ic_plummer(n, 12)
    exe = gb.Gb300Executor(precision="f64", attempts_per_sync=16, host_wait_timeout_s=0.2)
    it = gb.Integrator("RKF78", gb.NBodyODE(n, 0.005, 1.0 / n), exe)
    it.start(x0, 0.0, 2.0, 1e-8, 1e-8)
    assert it.advance(0) == gb.GB_ERR_TIMEOUT
    it.close()
    torch_cuda.cuda.synchronize()
