"""GPU: the learned step-size proposer end to end.  Controller logs of the
plain integrator on seed set A, training with the library's own forward /
backward / Adam kernels, then integration of held-out seeds (set B) with the
reference controller (the method without the network), the PI controller
(its fallback) and the learned proposer.  The embedded error estimate
accepts or rejects every attempt in all three."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_learned_proposer_gain_on_held_out_systems(gb, torch_cuda, capsys):
    from ode_prototyping_gb300 import learned
    c = learned.CONFIGS["plummer4096_rkf78"]
    m, info = learned.train_config("plummer4096_rkf78", learned.SEEDS_A[:4], rounds=2)
    assert all(np.isfinite(r["val_loss"]) for r in info)
    ev = learned.evaluate_config("plummer4096_rkf78", m, learned.SEEDS_B[:4])
    ref, pi, lrn = ev["reference"], ev["pi"], ev["learned"]
    gain = ev["gain"]
    with capsys.disabled():
        print(f"\nlearned proposer on {c['n']}-body Plummer RKF78, seeds B: RHS "
              f"{lrn['rhs']:.0f} vs reference {ref['rhs']:.0f} "
              f"({100 * gain['rhs_saved_fraction']:.1f}% saved) and PI {pi['rhs']:.0f} "
              f"(energy error {pi['energy_rel_err_max']:.2e}); "
              f"rejected {100 * lrn['rejected_fraction']:.1f}% vs "
              f"{100 * ref['rejected_fraction']:.1f}%; energy error "
              f"{lrn['energy_rel_err_max']:.2e} vs {ref['energy_rel_err_max']:.2e}")
    # the network proposed the steps after accepted attempts
    assert lrn["learned_proposals"] >= 0.5 * lrn["accepted"]
    # what it gains: fewer RHS evaluations than the reference controller (the
    # proposals are residuals over the PI formula, its fallback) ...
    assert gain["rhs_saved_fraction"] > 0.0
    # ... at a comparable energy error (a 2x looser tolerance costs the reference
    # controller ~3x in energy error for ~10 % fewer RHS evaluations), and the
    # same trajectory to tolerance level
    assert gain["energy_err_ratio"] <= 3.0
    assert gain["max_state_diff_vs_reference"] <= 1e-2


def test_shipped_tight_tolerance_proposer_saves_rhs(gb, torch_cuda):
    """The proposer shipped for the headline system at tol 1e-11 (relative
    energy error below 1e-8 over t in [0, 2]) takes fewer RHS evaluations than
    the reference controller on held-out seeds, with both runs' energy error
    below 1e-8."""
    import os
    from ode_prototyping_gb300 import learned
    c = learned.CONFIGS["plummer16384_rkf78_tol1e-11"]
    path = os.path.join(os.path.dirname(gb.__file__), "weights",
                        "proposer_plummer16384_rkf78_tol1e-11.bin")
    mlp = gb.GbMlp.from_buffer_copy(open(path, "rb").read())
    n, eps, tol = c["n"], c["softening"], c["tol"]
    rhs = {"reference": 0, "learned": 0}
    for seed in learned.SEEDS_B[:2]:
        x0 = gb.to_device(gb.ic_plummer(n, seed))
        e0 = gb.energy(x0, n, eps, 1.0 / n)
        for ctrl in rhs:
            exe = gb.Gb300Executor(precision="mixed", controller=ctrl, attempts_per_sync=16,
                                   mlp=mlp if ctrl == "learned" else None)
            it = gb.Integrator(c["tab"], gb.NBodyODE(n, eps, 1.0 / n), exe)
            it.start(x0, 0.0, c["tf"], tol, tol)
            it.advance(0)
            xs, t = it.state()
            st = it.stats()
            it.close()
            assert t == c["tf"]
            e1 = gb.energy(xs, n, eps, 1.0 / n)
            assert abs(e1["e"] - e0["e"]) / abs(e0["e"]) <= 1e-8, (seed, ctrl)
            rhs[ctrl] += st["n_rhs"]
    assert rhs["learned"] < rhs["reference"], rhs


def test_tolerance_feature_in_the_controller_log(gb, torch_cuda):
    """Feature 14 of every logged attempt is log max(atol, rtol) for scalar
    tolerances and 0 for vector tolerances; the batch sets it per system."""
    n, soft = 128, 0.05
    x0 = gb.ic_plummer(n, 31)
    for atol, rtol in ((1e-9, 1e-9), (1e-10, 1e-8), (np.full(6 * n, 1e-9), 1e-9)):
        exe = gb.Gb300Executor(precision="f64", log_steps=20)
        it = gb.Integrator("DOPRI5", gb.NBodyODE(n, soft, 1.0 / n), exe)
        it.start(x0, 0.0, 0.05, atol, rtol)
        assert it.advance(0) == 0
        f14 = it.log()[:, 14]
        assert len(f14) > 0
        want = 0.0 if np.ndim(atol) else np.float32(np.log(max(atol, rtol)))
        assert np.all(f14 == want), (atol, rtol, f14[:3])
        it.close()
    # in a batch the feature reaches the control warp's network input: a
    # network that reads only feature 14 proposes log(tol)-dependent steps
    # (checked through the single-system integrator above; here the batch runs
    # with per-system tolerances and the same network without error)
    m = gb.GbMlp()
    import ctypes as C
    assert gb.lib().gb_mlp_init(C.byref(m), 3) == 0
    for k in range(16):
        m.in_scale[k] = 0.0
    m.in_scale[14] = 0.01
    b = gb.Batch("DOPRI5", [64, 96], soft, precision="f64", controller="learned", mlp=m)
    xs = np.concatenate([gb.ic_plummer(64, 32), gb.ic_plummer(96, 33)])
    b.start(xs, 0.0, 0.05, [1e-8, 1e-10], [1e-8, 1e-10])
    assert b.advance() == 0
    assert b.stats()["n_learned_proposals"] > 0
    b.close()


@pytest.mark.parametrize("tol", [1e-9, 1e-11])
def test_multi_tolerance_proposer_beats_pi_on_held_out_seeds(gb, torch_cuda, tol):
    """One network trained over tolerances 1e-8 .. 1e-12 (log max(atol, rtol)
    is a feature) against its own fallback, the PI controller, on held-out
    seeds of the headline system: fewer RHS evaluations, at an energy error
    within the run-to-run spread of PI's.  The relative energy error at tf is
    a sum of signed drifts: a last-bit change of the error norm's summation
    order moved the learned run at tol 1e-11 between 0.75x and 1.5x PI's, so
    the bound is 3x (the spread a 2x tolerance step gives one controller)."""
    import os
    from ode_prototyping_gb300 import learned
    c = learned.CONFIGS["plummer16384_rkf78_multitol"]
    path = os.path.join(os.path.dirname(gb.__file__), "weights",
                        "proposer_plummer16384_rkf78_multitol.bin")
    mlp = gb.GbMlp.from_buffer_copy(open(path, "rb").read())
    n, eps = c["n"], c["softening"]
    rhs = {"pi": 0, "learned": 0}
    err = {"pi": 0.0, "learned": 0.0}
    for seed in learned.SEEDS_B[:2]:
        x0 = gb.to_device(gb.ic_plummer(n, seed))
        e0 = gb.energy(x0, n, eps, 1.0 / n)
        for ctrl in rhs:
            exe = gb.Gb300Executor(precision="mixed", controller=ctrl, attempts_per_sync=16,
                                   mlp=mlp if ctrl == "learned" else None)
            it = gb.Integrator(c["tab"], gb.NBodyODE(n, eps, 1.0 / n), exe)
            it.start(x0, 0.0, c["tf"], tol, tol)
            assert it.advance(0) == 0
            rhs[ctrl] += it.stats()["n_rhs"]
            e1 = gb.energy(it.state()[0], n, eps, 1.0 / n)
            err[ctrl] = max(err[ctrl], abs(e1["e"] - e0["e"]) / abs(e0["e"]))
            it.close()
    assert rhs["learned"] < rhs["pi"], rhs
    assert err["learned"] <= 3.0 * err["pi"], err
