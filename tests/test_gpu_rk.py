"""GPU parity of the element-wise embedded-RK kernels and of fixed-step
trajectories against the oracle."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TABS = ["HE21", "RKF45", "DOPRI5", "DVERK", "RKF78"]


def _np_stage(t, stage, dt, x0, ks, n):
    """rk_stage_kernel's operation order in numpy (IEEE, no contraction),
    zero coefficients skipped (they only change the sign of a zero)."""
    v = np.zeros(n)
    for j in range(stage):
        a = t.a[stage - 1][j]
        if a != 0.0:
            v = v + a * ks[j * n:(j + 1) * n]
    return x0 + v * dt


@pytest.mark.parametrize("name", TABS)
def test_stage_update_target_bitwise(gb, torch_cuda, name):
    torch = torch_cuda
    t = gb.tableau(name)
    S, n = t.n_stages, 1237
    rng = np.random.default_rng(S)
    x0 = rng.standard_normal(n)
    ks = rng.standard_normal(S * n)
    dt = 0.0137
    dx0, dks = gb.to_device(x0), gb.to_device(ks)
    out = torch.empty(n, dtype=torch.float64, device="cuda")
    for stage in range(1, S):
        gb.rk_stage(t, stage, dt, dx0, dks, out, n)
        np.testing.assert_array_equal(out.cpu().numpy(), _np_stage(t, stage, dt, x0, ks, n))
    x = torch.empty_like(out)
    err = torch.empty_like(out)
    gb.rk_update(t, dt, dx0, dks, x, err, n)
    xv = np.zeros(n)
    ev = np.zeros(n)
    for j in range(S):
        b, db = t.b[j], t.b[j] - t.bt[j]
        if b != 0.0:
            xv = xv + b * ks[j * n:(j + 1) * n]
        if db != 0.0:
            ev = ev + db * ks[j * n:(j + 1) * n]
    np.testing.assert_array_equal(x.cpu().numpy(), x0 + xv * dt)
    np.testing.assert_array_equal(err.cpu().numpy(), ev * dt)
    atol = gb.to_device(np.full(n, 1e-8))
    rtol = gb.to_device(np.full(n, 1e-6))
    tg = torch.empty_like(out)
    gb.rk_error_target(atol, rtol, x, dx0, tg, n)
    xn = x.cpu().numpy()
    np.testing.assert_array_equal(tg.cpu().numpy(),
                                  1e-8 + 1e-6 * np.maximum(np.abs(xn), np.abs(x0)))


@pytest.mark.parametrize("n", [1, 7, 256, 6144, 98304, 1000003])
def test_norm(gb, torch_cuda, n):
    rng = np.random.default_rng(n)
    v = rng.standard_normal(n)
    s = rng.uniform(0.5, 2.0, n)
    got = gb.rk_norm(gb.to_device(v), gb.to_device(s), n).item()
    serial = 0.0
    q = (v / s) ** 2
    ref = np.sqrt(np.sum(q) / n)
    assert got == pytest.approx(ref, rel=1e-14)
    again = gb.rk_norm(gb.to_device(v), gb.to_device(s), n).item()
    assert got == again  # deterministic


@pytest.mark.parametrize("name,tile", [("DOPRI5", (1, 1, 0)), ("RKF78", (1, 1, 0)),
                                       ("DOPRI5", (0, 0, 0)), ("RKF78", (4, 2, 0))])
def test_fixed_step_trajectory(gb, orc, torch_cuda, name, tile):
    """Fixed-step trajectories built from the GPU kernels agree with the
    oracle to <= 1e-12 (bitwise with the serial tiling)."""
    torch = torch_cuda
    n, soft, dt, steps = 256, 0.02, 1e-3, 20
    x0 = gb.ic_plummer(n, 4)
    ode, _ = orc.nbody_ode(n, soft, 1.0 / n)
    ref, _ = orc.fixed_steps(name, ode, x0, dt, steps)
    t = gb.tableau(name)
    S, nv = t.n_stages, 6 * n
    til = gb.tiling(*tile)
    x = gb.to_device(x0)
    ks = torch.empty(S * nv, dtype=torch.float64, device="cuda")
    tmp = torch.empty(nv, dtype=torch.float64, device="cuda")
    err = torch.empty(nv, dtype=torch.float64, device="cuda")
    xn = torch.empty(nv, dtype=torch.float64, device="cuda")
    for _ in range(steps):
        gb.nbody_rhs_f64(x, n, soft, 1.0 / n, tile=til, out=ks[:nv])
        for s in range(1, S):
            gb.rk_stage(t, s, dt, x, ks, tmp, nv)
            gb.nbody_rhs_f64(tmp, n, soft, 1.0 / n, tile=til, out=ks[s * nv:(s + 1) * nv])
        gb.rk_update(t, dt, x, ks, xn, err, nv)
        x.copy_(xn)
    got = x.cpu().numpy()
    if tile == (1, 1, 0):
        np.testing.assert_array_equal(got, ref)
    else:
        assert np.max(np.abs(got - ref) / np.maximum(np.abs(ref), 1.0)) <= 1e-12


@pytest.mark.parametrize("tile,exact", [((1, 1, 0), True), ((0, 0, 0), False)])
def test_leapfrog_matches_oracle(gb, orc, torch_cuda, tile, exact):
    """ParallelLeapfrogIntegrator (LeapfrogParallel.hpp:11-41): bit-identical
    with the serial tiling, <= 1e-12 otherwise."""
    n, soft, dt = 200, 0.02, 1e-3
    x0 = gb.ic_plummer(n, 17)
    ode, _ = orc.nbody_ode(n, soft, 1.0 / n)
    ref, steps_ref = orc.leapfrog(ode, x0, 0.0, 0.05, dt)
    out = gb.RawOutput()
    exe = gb.Gb300Executor(tile=gb.tiling(*tile))
    x, steps = gb.ParallelLeapfrogIntegrator.integrate(x0, 0.0, 0.05, dt,
                                                       gb.NBodyODE(n, soft, 1.0 / n), out, exe)
    assert steps == steps_ref and len(out.times()) == steps + 1
    got = x.cpu().numpy()
    if exact:
        np.testing.assert_array_equal(got, ref)
    else:
        assert np.max(np.abs(got - ref) / np.maximum(np.abs(ref), 1.0)) <= 1e-12
    np.testing.assert_array_equal(np.array(out.states()[-1]), got)


def test_leapfrog_mixed_tracks_f64(gb, torch_cuda):
    """Leapfrog on the mixed-precision force kernels stays within 1e-6 of the
    FP64 leapfrog over 50 steps."""
    n, soft, dt = 1024, 0.01, 1e-3
    x0 = gb.ic_plummer(n, 18)
    ode = gb.NBodyODE(n, soft, 1.0 / n)
    x64, s64 = gb.ParallelLeapfrogIntegrator.integrate(x0, 0.0, 0.05, dt, ode, None,
                                                       gb.Gb300Executor(precision="f64"))
    xmx, smx = gb.ParallelLeapfrogIntegrator.integrate(x0, 0.0, 0.05, dt, ode, None,
                                                       gb.Gb300Executor(precision="mixed"))
    assert s64 == smx
    assert (xmx - x64).abs().max().item() <= 1e-6
