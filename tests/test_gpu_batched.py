"""GPU: the batched integrator -- every system of a batch of uneven sizes
follows the reference's loop (oracle) and agrees with the single-system
integrator."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _systems(gb, sizes, seed0):
    # a one-body system is a lone body in uniform motion
    xs = [gb.ic_plummer(int(n), seed0 + k) if n > 1
          else np.array([0.1, -0.2, 0.3, 0.05, 0.02, -0.01]) for k, n in enumerate(sizes)]
    return xs, np.concatenate(xs)


@pytest.mark.parametrize("tab", ["DOPRI5", "RKF78"])
def test_batch_f64_matches_oracle_per_system(gb, orc, torch_cuda, tab):
    sizes = [33, 64, 100, 129, 7, 250, 1]
    soft, tol, tf = 0.05, 1e-9, 0.15
    xs, x0 = _systems(gb, sizes, 40)
    b = gb.Batch(tab, sizes, soft, precision="f64")
    b.start(x0, 0.0, tf, tol, tol)
    assert b.advance() == 0
    st = b.stats(per_system=True)
    x, t = b.state()
    x = x.cpu().numpy()
    for k, n in enumerate(sizes):
        ode, _ = orc.nbody_ode(n, soft, 1.0 / n)
        r = orc.integrate(tab, ode, xs[k], 0.0, tf, tol, tol)
        assert st["systems"][k]["n_accepted"] == len(r.times) - 1, k
        assert t[k] == r.times[-1]
        assert np.max(np.abs(b.system_state(x, k) - r.states[-1])) <= 10 * tol
    b.close()


def test_batch_mixed_and_autotune(gb, torch_cuda):
    rng = np.random.default_rng(5)
    sizes = np.round(np.exp(rng.uniform(np.log(64), np.log(1024), 24))).astype(int)
    soft = 0.04 / np.cbrt(sizes)
    tol, tf = 1e-9, 0.05
    xs, x0 = _systems(gb, sizes, 100)
    ref = gb.Batch("DOPRI5", sizes, soft, precision="f64")
    ref.start(x0, 0.0, tf, tol, tol)
    assert ref.advance() == 0
    xr, _ = ref.state()
    b = gb.Batch("DOPRI5", sizes, soft, precision="mixed")
    b.start(x0, 0.0, tf, tol, tol)
    choice = b.autotune(2)
    assert choice["stage_ms"] > 0
    assert b.advance() == 0
    xm, tm = b.state()
    np.testing.assert_allclose(tm, tf)
    assert (xm - xr).abs().max().item() <= 1e-6
    ref.close()
    b.close()


def test_batch_budget_status(gb, torch_cuda):
    sizes = [40, 50]
    xs, x0 = _systems(gb, sizes, 7)
    b = gb.Batch("DOPRI5", sizes, 0.05, precision="f64", max_attempts=3)
    b.start(x0, 0.0, 5.0, 1e-12, 1e-12)
    assert b.advance() == gb.GB_ERR_BUDGET
    st = b.stats(per_system=True)
    assert all(s["n_attempts"] == 3 for s in st["systems"])
    b.close()


def _zero_mlp(gb):
    """A network whose output is exactly zero: the learned proposal is then
    the elementary controller's formula in log form."""
    import ctypes as C
    m = gb.GbMlp()
    assert gb.lib().gb_mlp_init(C.byref(m), 9) == 0
    for k in range(64):
        m.w3[k] = 0.0
    m.b3 = 0.0
    m.out_bias = 0.0
    m.out_scale = 1.0
    for k in range(16):
        m.in_scale[k] = 1.0
    return m


@pytest.mark.parametrize("spc", [1, 2])
def test_batch_learned_controller(gb, torch_cuda, spc):
    """The batched control warp evaluates the proposer per system; with a
    zero-output network every system takes the same accepted steps as the
    single-system integrator under the same network, with one system per CTA
    or with the small ones sharing a CTA."""
    sizes = [48, 96, 160]
    soft, tol, tf = 0.05, 1e-9, 0.1
    xs, x0 = _systems(gb, sizes, 70)
    m = _zero_mlp(gb)
    b = gb.Batch("DOPRI5", sizes, soft, precision="f64", controller="learned", mlp=m,
                 tiling=gb.GbBatchTiling(128, 1, 1, 0, spc))
    b.start(x0, 0.0, tf, tol, tol)
    assert b.advance() == 0
    st = b.stats(per_system=True)
    assert st["n_learned_proposals"] > 0
    x, t = b.state()
    x = x.cpu().numpy()
    np.testing.assert_allclose(t, tf)
    for k, n in enumerate(sizes):
        exe = gb.Gb300Executor(precision="f64", controller="learned", mlp=m)
        it = gb.Integrator("DOPRI5", gb.NBodyODE(n, soft, 1.0 / n), exe)
        it.start(xs[k], 0.0, tf, tol, tol)
        assert it.advance(0) == 0
        s1 = it.stats()
        assert abs(st["systems"][k]["n_accepted"] - s1["n_accepted"]) <= 1, k
        xk, _ = it.state()
        assert np.max(np.abs(b.system_state(x, k) - xk.cpu().numpy())) <= 10 * tol
        it.close()
    b.close()


def test_batch_learned_requires_network(gb, torch_cuda):
    with pytest.raises(gb.GbError):
        gb.Batch("DOPRI5", [32], 0.05, precision="f64", controller="learned")


def test_batch_pi_controller_matches_single_system(gb, torch_cuda):
    """The PI controller in the batch's per-system control warp takes the same
    accepted steps as the single-system integrator's PI controller."""
    sizes = [40, 90, 150]
    soft, tol, tf = 0.05, 1e-9, 0.1
    xs, x0 = _systems(gb, sizes, 80)
    b = gb.Batch("DOPRI5", sizes, soft, precision="f64", controller="pi")
    b.start(x0, 0.0, tf, tol, tol)
    assert b.advance() == 0
    st = b.stats(per_system=True)
    x, t = b.state()
    x = x.cpu().numpy()
    np.testing.assert_allclose(t, tf)
    for k, n in enumerate(sizes):
        it = gb.Integrator("DOPRI5", gb.NBodyODE(n, soft, 1.0 / n),
                           gb.Gb300Executor(precision="f64", controller="pi"))
        it.start(xs[k], 0.0, tf, tol, tol)
        assert it.advance(0) == 0
        assert abs(st["systems"][k]["n_accepted"] - it.stats()["n_accepted"]) <= 1, k
        xk, _ = it.state()
        assert np.max(np.abs(b.system_state(x, k) - xk.cpu().numpy())) <= 10 * tol
        it.close()
    b.close()


@pytest.mark.parametrize("spc", [2, 4])
def test_batch_systems_sharing_a_cta_follow_the_oracle(gb, orc, torch_cuda, spc):
    """Several small systems per CTA (one warp group each): in FP64 every
    system follows the reference loop (oracle), and the whole batch is bit
    for bit the batch with one system per CTA (a lane's partner order does
    not depend on the group size)."""
    sizes = [33, 64, 100, 129, 7, 250, 1, 20, 50, 31, 64, 12]
    soft, tol, tf = 0.05, 1e-9, 0.1
    xs, x0 = _systems(gb, sizes, 140)
    runs = []
    for g in (1, spc):
        b = gb.Batch("DOPRI5", sizes, soft, precision="f64",
                     tiling=gb.GbBatchTiling(128, 1, 1, 0, g))
        geo = b.geometry()
        assert geo["systems_per_cta"] == g
        b.start(x0, 0.0, tf, tol, tol)
        assert b.advance() == 0
        x, t = b.state()
        runs.append((x.cpu().numpy(), t, b.stats(per_system=True)))
        b.close()
    (x1, t1, _), (xg, tg, st) = runs
    np.testing.assert_array_equal(xg, x1)
    np.testing.assert_array_equal(tg, t1)
    for k, n in enumerate(sizes):
        ode, _ = orc.nbody_ode(n, soft, 1.0 / n)
        r = orc.integrate("DOPRI5", ode, xs[k], 0.0, tf, tol, tol)
        assert st["systems"][k]["n_accepted"] == len(r.times) - 1, k
        assert np.max(np.abs(x1[6 * sum(sizes[:k]):6 * sum(sizes[:k + 1])] - r.states[-1])) \
            <= 10 * tol, k


def test_batch_mixed_systems_sharing_a_cta(gb, torch_cuda):
    """Mixed precision, two systems of up to 64 bodies per 128-thread CTA:
    each such system runs the 64-thread packed pair loop, so it is bit for
    bit the system of a 64-thread batch; every system tracks the FP64 batch
    to 1e-6."""
    sizes = [64, 40, 200, 17, 64, 130, 1, 50, 33]
    soft, tol, tf = 0.05, 1e-9, 0.05
    xs, x0 = _systems(gb, sizes, 160)
    ref = gb.Batch("DOPRI5", sizes, soft, precision="f64")
    ref.start(x0, 0.0, tf, tol, tol)
    assert ref.advance() == 0
    xr, _ = ref.state()
    ref.close()
    out = {}
    for key, til in (("grouped", gb.GbBatchTiling(128, 1, 1, 0, 2)),
                     ("t64", gb.GbBatchTiling(64, 1, 1, 0, 1))):
        b = gb.Batch("DOPRI5", sizes, soft, precision="mixed", tiling=til)
        b.start(x0, 0.0, tf, tol, tol)
        assert b.advance() == 0
        x, t = b.state()
        np.testing.assert_allclose(t, tf)
        assert (x - xr).abs().max().item() <= 1e-6, key
        out[key] = x.cpu().numpy()
        b.close()
    for k, n in enumerate(sizes):
        if n <= 64:
            sl = slice(6 * sum(sizes[:k]), 6 * sum(sizes[:k + 1]))
            np.testing.assert_array_equal(out["grouped"][sl], out["t64"][sl])
