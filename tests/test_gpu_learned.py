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
