"""Trajectory files in the reference's binary format (src/demo/nbody_io.hpp:4-22):
written by the library's background writer, read back with the layout the
reference's reader expects (scripts/nbody_io/bin_reader.py:11-18)."""
import os

import numpy as np
import pytest


def test_writer_roundtrip_host_only(gb, tmp_path):
    path = str(tmp_path / "traj.bin")
    rng = np.random.default_rng(0)
    states = rng.standard_normal((300, 30))
    times = np.cumsum(rng.uniform(0, 0.1, 300))
    w = gb.TrajectoryWriter(path, 30, 0.25)
    for t, x in zip(times, states):
        w.save_state(t, x)
    assert w.close() == 300
    raw = open(path, "rb").read()
    assert len(raw) == 24 + 300 * 31 * 8
    t2, s2, soft = gb.read_trajectory(path)
    assert soft == 0.25
    np.testing.assert_array_equal(t2, times)
    np.testing.assert_array_equal(s2, states)
    # the reference reader's reshape: (n_times, n_var + 1)
    flat = np.frombuffer(raw[24:], dtype="<f8").reshape(300, 31)
    np.testing.assert_array_equal(flat[:, 0], times)


def test_empty_trajectory(gb, tmp_path):
    path = str(tmp_path / "empty.bin")
    w = gb.TrajectoryWriter(path, 6, 0.0)
    assert w.close() == 0
    t, s, soft = gb.read_trajectory(path)
    assert len(t) == 0 and s.shape == (0, 6)


@pytest.mark.gpu
def test_integrator_streams_to_file(gb, torch_cuda, tmp_path):
    n = 64
    x0 = gb.ic_plummer(n, 3)
    path = str(tmp_path / "run.bin")
    w = gb.TrajectoryWriter(path, 6 * n, 0.05)
    ram = gb.RawOutput()

    class Both:
        def save_state(self, t, x):
            ram.save_state(t, x)
            w.save_state(t, x)

    gb.RKEmbeddedParallel("DOPRI5").integrate(x0, 0.0, 0.2, 1e-9, 1e-9,
                                              gb.NBodyODE(n, 0.05, 1.0 / n), Both(),
                                              gb.Gb300Executor(attempts_per_sync=4))
    assert w.close() == len(ram.times())
    t, s, _ = gb.read_trajectory(path)
    np.testing.assert_array_equal(t, np.array(ram.times()))
    np.testing.assert_array_equal(s, np.array(ram.states()))
