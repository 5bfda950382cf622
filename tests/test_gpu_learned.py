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
