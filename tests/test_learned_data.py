"""CPU: the training targets of the learned step-size proposer.

Each accepted attempt k followed by an attempt k+1 gives one sample: the
features the controller saw after attempt k, and the log step change that
would have put attempt k+1 at the error ratio rho under err ~ dt^(q+1),
taken relative to the PI controller's own proposal (the base the device adds
the network output to).  Rejected attempts, the last attempt and non-finite
targets give no sample."""
import numpy as np

from ode_prototyping_gb300 import learned


def _records(log_dt, log_err, accepted, log_err_prev):
    n = len(log_dt)
    rec = np.zeros((n, 19), dtype=np.float64)
    rec[:, :16] = np.arange(16)[None, :] + 100.0 * np.arange(n)[:, None]  # recognisable
    rec[:, 13] = log_err_prev
    rec[:, learned.LOG_DT] = log_dt
    rec[:, learned.LOG_ERR] = log_err
    rec[:, learned.ACCEPTED] = accepted
    return rec


def test_samples_only_from_accepted_attempts_with_a_successor():
    rec = _records(log_dt=[-3.0, -2.9, -2.8, -2.7], log_err=[-1.0, 0.5, -0.5, -0.2],
                   accepted=[1, 0, 1, 1], log_err_prev=[0.0, -1.0, -1.0, -0.5])
    x, y = learned.build_dataset([rec], q=4)
    # attempt 0 (accepted, successor 1), attempt 2 (accepted, successor 3);
    # attempt 1 was rejected, attempt 3 has no successor
    assert x.shape == (2, 16) and y.shape == (2,)
    np.testing.assert_array_equal(x[0], rec[0, :16].astype(np.float32))
    np.testing.assert_array_equal(x[1], rec[2, :16].astype(np.float32))


def test_target_is_the_ideal_step_change_over_the_pi_proposal():
    q, rho, beta = 4, 0.38, learned.PI_BETA
    # local error model err = c dt^(q+1): the ideal next step for error rho
    c = 10.0 ** 9
    log_dt = np.log([1e-2, 1.1e-2])
    log_err = np.log(c) + (q + 1) * log_dt
    rec = _records(log_dt=log_dt, log_err=log_err, accepted=[1, 1],
                   log_err_prev=[np.log(0.3), log_err[0]])
    x, y = learned.build_dataset([rec], q=q, rho=rho, pi_beta=beta)
    ideal = np.log((rho / c) ** (1.0 / (q + 1)))
    base = (np.log(0.38) / (1 + q) - (1.0 / (1 + q) - 0.75 * beta) * log_err[0]
            + beta * np.log(0.3))
    assert y.shape == (1,)
    assert abs(float(y[0]) - (ideal - log_dt[0] - base)) < 1e-5


def test_non_finite_targets_are_dropped():
    rec = _records(log_dt=[-3.0, -2.9, -2.8], log_err=[-1.0, -np.inf, -0.5],
                   accepted=[1, 1, 1], log_err_prev=[0.0, -1.0, -1.0])
    x, y = learned.build_dataset([rec], q=4)
    # attempt 0's successor has err = 0 (log -inf): no finite target; attempt
    # 1's own log err is -inf, so its PI base is not finite either
    assert len(y) == 0 and x.shape[0] == 0


def test_logs_are_concatenated_in_order():
    a = _records([-3.0, -2.9], [-1.0, -0.9], [1, 1], [0.0, -1.0])
    b = _records([-2.0, -1.9, -1.8], [-0.7, -0.6, -0.5], [1, 1, 1], [0.0, -0.7, -0.6])
    x, y = learned.build_dataset([a, b], q=4)
    assert len(y) == 1 + 2
    np.testing.assert_array_equal(x[1], b[0, :16].astype(np.float32))


def test_shipped_weights_match_the_struct_and_a_configuration():
    """Every shipped proposer is a raw gb_mlp of the current layout, named for
    a training configuration, with finite weights, non-negative input scales
    (0 switches off a feature that was constant in training) and a positive
    output scale."""
    import ctypes
    import glob
    import os
    import ode_prototyping_gb300 as gb
    files = sorted(glob.glob(os.path.join(os.path.dirname(gb.__file__), "weights", "*.bin")))
    assert files
    for path in files:
        name = os.path.basename(path)[len("proposer_"):-len(".bin")]
        assert name in learned.CONFIGS, name
        raw = open(path, "rb").read()
        assert len(raw) == ctypes.sizeof(gb.GbMlp), name
        m = gb.GbMlp.from_buffer_copy(raw)
        flat = np.frombuffer(raw, dtype=np.float32)
        assert np.all(np.isfinite(flat)), name
        assert all(s >= 0 for s in m.in_scale) and any(s > 0 for s in m.in_scale), name
        assert m.out_scale > 0, name


def test_shipped_single_tolerance_proposers_ignore_the_tolerance_feature(gb):
    """Proposers trained at one tolerance saw a constant feature 14 (log max
    of the tolerances) and carry a zero input scale for it; the
    multi-tolerance proposer uses it."""
    import glob
    import os
    wdir = os.path.join(os.path.dirname(gb.__file__), "weights")
    paths = sorted(glob.glob(os.path.join(wdir, "*.bin")))
    assert paths
    for path in paths:
        m = gb.GbMlp.from_buffer_copy(open(path, "rb").read())
        if "multitol" in os.path.basename(path):
            assert m.in_scale[14] > 0.0, path
        else:
            assert m.in_scale[14] == 0.0, path
