"""GPU parity of the N-body right-hand side against the oracle (reference
restatement) and the reference's own outputs (fixtures)."""
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu


def _x(n, seed, spread=1.0):
    rng = np.random.default_rng(seed)
    x = rng.standard_normal(6 * n) * spread
    return x


def _rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def _force_scale(x, n, soft, rows=512):
    """Per body, the sum of the magnitudes of its pair terms, m sum_j
    |x_j - x_i| / (r^2 + eps^2)^(3/2) (FP64, torch on the GPU): the scale a
    per-body acceleration error is measured against when the pair terms
    nearly cancel (a body near the centre of mass has |a_i| << that sum)."""
    import torch
    p = torch.as_tensor(np.asarray(x[: 3 * n]).reshape(-1, 3), dtype=torch.float64,
                        device="cuda")
    out = torch.empty(n, dtype=torch.float64, device="cuda")
    for i0 in range(0, n, rows):
        d = p[None, :, :] - p[i0:i0 + rows, None, :]
        r = d.norm(dim=2)
        out[i0:i0 + rows] = (r / (r * r + soft * soft) ** 1.5).sum(dim=1)
    return out.cpu().numpy() / n


@pytest.mark.parametrize("n,soft", [(2, 0.1), (5, 0.0), (64, 0.05), (1000, 0.01), (1024, 0.01),
                                    (1031, 0.2)])
def test_rhs_f64_serial_tiling_is_bitwise_reference(gb, orc, torch_cuda, n, soft):
    """j_split = lanes = 1: every body sums its terms in ascending partner
    order with IEEE operations -- identical to the serial executor."""
    x = _x(n, n)
    mass = 1.0 / n
    ode, _ = orc.nbody_ode(n, soft, mass)
    ref = orc.rhs(ode, x)
    got = gb.nbody_rhs_f64(x, n, soft, mass, tile=gb.tiling(1, 1, 0)).cpu().numpy()
    np.testing.assert_array_equal(got, ref)


@pytest.mark.parametrize("pair", [2, 1])
@pytest.mark.parametrize("P,L,B", [(0, 0, 0), (2, 1, 0), (4, 2, 0), (8, 4, 0), (8, 8, 64),
                                   (1, 4, 32), (2, 2, 256), (1, 1, 0)])
def test_rhs_f64_tilings_within_1e12(gb, orc, torch_cuda, P, L, B, pair):
    """Every tiling, with the reference's pair term (pair 2) and with the
    refined-rsqrt pair term the integrator's FP64 stages use (pair 1)."""
    n, soft = 1531, 0.01
    x = _x(n, 7)
    ode, _ = orc.nbody_ode(n, soft, 1.0 / n)
    ref = orc.rhs(ode, x)
    got = gb.nbody_rhs_f64(x, n, soft, 1.0 / n,
                           tile=gb.tiling(P, L, B, f64_pair=pair)).cpu().numpy()
    acc_g, acc_r = got[3 * n:].reshape(-1, 3), ref[3 * n:].reshape(-1, 3)
    # FP64 parity bound for any tiling: accelerations agree to <= 1e-12 relative
    rel = np.linalg.norm(acc_g - acc_r, axis=1) / np.linalg.norm(acc_r, axis=1)
    assert rel.max() <= 1e-12, rel.max()
    np.testing.assert_array_equal(got[: 3 * n], ref[: 3 * n])


@pytest.mark.parametrize("pair", [2, 1])
@pytest.mark.parametrize("n,soft,gen,rows", [(16384, 0.005, "plummer", 4096),
                                             (262144, 0.002, "cold", 1024)])
def test_rhs_f64_config_sizes_sampled_rows(gb, orc, torch_cuda, n, soft, gen, rows, pair):
    """The FP64 right-hand side at the configurations' sizes with the default
    launch geometry (at N = 16384: 8 cluster ranks x 2 lanes; at 262144: 8 x 1)
    against the oracle's pair sum (NBodyODE.hpp:68-133 restated) on sampled
    rows: <= 1e-12 relative per body, velocities copied exactly; both pair
    terms (2: the reference's operation order, 1: the integrator's default)."""
    x = gb.ic_plummer(n, 101) if gen == "plummer" else gb.ic_cold_sphere(n, 5, 0.01)
    got = gb.nbody_rhs_f64(x, n, soft, 1.0 / n, tile=gb.tiling(f64_pair=pair)).cpu().numpy()
    np.testing.assert_array_equal(got[: 3 * n], x[3 * n:])
    sel = np.sort(np.random.default_rng(n).choice(n, rows, replace=False))
    ode, _ = orc.nbody_ode(n, soft, 1.0 / n)
    ref = orc.acc_rows(ode, x, sel)
    a = got[3 * n:].reshape(-1, 3)[sel]
    rel = np.linalg.norm(a - ref, axis=1) / np.linalg.norm(ref, axis=1)
    assert rel.max() <= 1e-12, rel.max()


def test_rhs_f64_deterministic(gb, torch_cuda):
    n = 2048
    x = _x(n, 3)
    a = gb.nbody_rhs_f64(x, n, 0.01, 1.0 / n).cpu().numpy()
    b = gb.nbody_rhs_f64(x, n, 0.01, 1.0 / n).cpu().numpy()
    np.testing.assert_array_equal(a, b)


@pytest.mark.parametrize("tag", ["ball64_dopri5", "plummer256_rkf78", "config1_ball1024_dopri5"])
def test_rhs_f64_equals_reference_fixture(gb, torch_cuda, tag):
    path = os.path.join(GOLDEN, f"nbody_{tag}.npz")
    if not os.path.exists(path):
        pytest.skip("fixture missing")
    d = np.load(path)
    n, soft, mass = int(d["meta"][0]), d["meta"][1], d["meta"][2]
    got = gb.nbody_rhs_f64(d["x0"], n, soft, mass, tile=gb.tiling(1, 1, 0)).cpu().numpy()
    np.testing.assert_array_equal(got, d["rhs"])


def test_rhs_f64_per_body_masses(gb, orc, torch_cuda):
    n = 300
    x = _x(n, 9)
    m = np.random.default_rng(1).uniform(0.5, 2.0, n) / n
    ode, keep = orc.nbody_ode(n, 0.02, masses=m)
    ref = orc.rhs(ode, x)
    mt = gb.to_device(m)
    got = gb.nbody_rhs_f64(x, n, 0.02, masses=mt, tile=gb.tiling(1, 1, 0)).cpu().numpy()
    np.testing.assert_array_equal(got, ref)


def test_acc_write_and_accumulate(gb, orc, torch_cuda):
    n = 129
    x = _x(n, 4)
    ode, _ = orc.nbody_ode(n, 0.1, 1.0)
    ref = orc.rhs(ode, x)[3 * n:]
    acc = gb.nbody_acc_f64(x[: 3 * n], n, 0.1, 1.0, tile=gb.tiling(1, 1, 0))
    np.testing.assert_array_equal(acc.cpu().numpy(), ref)
    gb.nbody_acc_f64(x[: 3 * n], n, 0.1, 1.0, accumulate=True, out=acc, tile=gb.tiling(1, 1, 0))
    np.testing.assert_array_equal(acc.cpu().numpy(), 2 * ref)


@pytest.mark.parametrize("variant", [0, 1, 2, 3])
@pytest.mark.parametrize("n,soft,gen", [(1024, 0.01, "ball"), (4096, 0.005, "plummer"),
                                        (16384, 0.005, "plummer"), (3001, 0.003, "binary"),
                                        (8192, 0.002, "cold"), (7, 0.05, "plummer"),
                                        (257, 0.02, "plummer")])
def test_rhs_mixed_within_1e6_of_fp64(gb, torch_cuda, n, soft, gen, variant):
    """Hi-only pair differences with hi/lo for close pairs, every pair loop:
    accelerations within 1e-6 of FP64 (normwise and for the median body)."""
    if gen == "ball":
        x = gb.ic_uniform_ball(n, 1, 0.1)
    elif gen == "plummer":
        x = gb.ic_plummer(n, 2)
    elif gen == "cold":
        x = gb.ic_cold_sphere(n, 4, 0.01)
    else:
        x = gb.ic_binary_plummer(n, 3, 0.1, 1e-3, 1e-2)
    ref = gb.nbody_rhs_f64(x, n, soft, 1.0 / n).cpu().numpy()
    got = gb.nbody_rhs_mixed(x, n, soft, 1.0 / n,
                             tile=gb.tiling(mixed_variant=variant)).cpu().numpy()
    np.testing.assert_array_equal(got[: 3 * n], ref[: 3 * n])
    a_g, a_r = got[3 * n:].reshape(-1, 3), ref[3 * n:].reshape(-1, 3)
    # normwise relative error of the acceleration field
    assert _rel(a_g, a_r) <= 1e-6, _rel(a_g, a_r)
    err = np.linalg.norm(a_g - a_r, axis=1)
    per = err / np.linalg.norm(a_r, axis=1)
    # per-body: the median body is far inside the bound, and 99.9 % of the
    # bodies are within it where there are enough bodies for that quantile
    assert np.median(per) <= 1e-6, np.median(per)
    if n >= 1024:
        assert np.quantile(per, 0.999) <= 1e-6, np.quantile(per, 0.999)
    # every body, against the sum of its pair terms' magnitudes (the error
    # bound of the pair differences is relative to each term)
    cond = err / _force_scale(x, n, soft)
    assert cond.max() <= 1e-6, cond.max()


def test_rhs_mixed_masses_and_shift_invariance(gb, torch_cuda):
    n = 2000
    x = gb.ic_plummer(n, 5)
    m = np.random.default_rng(2).uniform(0.5, 1.5, n)
    m /= m.sum()
    mt = gb.to_device(m)
    ref = gb.nbody_rhs_f64(x, n, 0.01, masses=mt).cpu().numpy()
    got = gb.nbody_rhs_mixed(x, n, 0.01, masses=mt).cpu().numpy()
    assert _rel(got[3 * n:], ref[3 * n:]) <= 1e-6
    # hi/lo positions relative to the centroid: a far-away system is as accurate
    xs = x.copy()
    xs[: 3 * n] += 1.0e4
    got2 = gb.nbody_rhs_mixed(xs, n, 0.01, masses=mt).cpu().numpy()
    assert _rel(got2[3 * n:], ref[3 * n:]) <= 2e-6


def test_energy_kernel_matches_oracle(gb, orc, torch_cuda):
    n = 777
    x = gb.ic_plummer(n, 8)
    ode, _ = orc.nbody_ode(n, 0.01, 1.0 / n)
    e_ref = orc.energy(ode, x)
    e = gb.energy(x, n, 0.01, 1.0 / n)
    assert e["ke"] == pytest.approx(e_ref["ke"], rel=1e-13)
    assert e["pe"] == pytest.approx(e_ref["pe"], rel=1e-12)
    np.testing.assert_allclose(e["p"], e_ref["p"], atol=1e-14)
    np.testing.assert_allclose(e["l"], e_ref["l"], atol=1e-13)


def test_invalid_mixed_softening_rejected(gb, torch_cuda):
    with pytest.raises(gb.GbError):
        gb.nbody_rhs_mixed(_x(10, 1), 10, 0.0, 0.1)


@pytest.mark.parametrize("n,soft,gen", [(1024, 0.01, "ball"), (4096, 0.005, "plummer"),
                                        (16384, 0.005, "plummer"), (3001, 0.003, "binary"),
                                        (130, 0.05, "plummer"), (65536, 0.002, "cold")])
def test_rhs_mixed_sorted_within_1e6_of_fp64(gb, torch_cuda, n, soft, gen):
    """Morton-sorted tiles with the tile-centroid far path: same bound as the
    hi/lo path, rows in body order."""
    x = {"ball": lambda: gb.ic_uniform_ball(n, 1, 0.1), "plummer": lambda: gb.ic_plummer(n, 2),
         "binary": lambda: gb.ic_binary_plummer(n, 3, 0.1, 1e-3, 1e-2),
         "cold": lambda: gb.ic_cold_sphere(n, 4, 0.01)}[gen]()
    ref = gb.nbody_rhs_f64(x, n, soft, 1.0 / n).cpu().numpy()
    got = gb.nbody_rhs_mixed_sorted(x, n, soft, 1.0 / n).cpu().numpy()
    np.testing.assert_array_equal(got[: 3 * n], ref[: 3 * n])
    a_g, a_r = got[3 * n:].reshape(-1, 3), ref[3 * n:].reshape(-1, 3)
    assert _rel(a_g, a_r) <= 1e-6, _rel(a_g, a_r)
    per = np.linalg.norm(a_g - a_r, axis=1) / np.linalg.norm(a_r, axis=1)
    assert np.median(per) <= 1e-6, np.median(per)


def test_rhs_mixed_sorted_masses_and_displaced(gb, torch_cuda):
    n = 2000
    x = gb.ic_plummer(n, 5)
    m = np.random.default_rng(2).uniform(0.5, 1.5, n)
    m /= m.sum()
    mt = gb.to_device(m)
    ref = gb.nbody_rhs_f64(x, n, 0.01, masses=mt).cpu().numpy()
    got = gb.nbody_rhs_mixed_sorted(x, n, 0.01, masses=mt).cpu().numpy()
    assert _rel(got[3 * n:], ref[3 * n:]) <= 1e-6
    xs = x.copy()
    xs[: 3 * n] += 1.0e4
    got2 = gb.nbody_rhs_mixed_sorted(xs, n, 0.01, masses=mt).cpu().numpy()
    assert _rel(got2[3 * n:], ref[3 * n:]) <= 2e-6


@pytest.mark.parametrize("n", [1, 2, 3])
def test_tiny_systems_both_precisions(gb, orc, torch_cuda, n):
    """Edge sizes: a lone body feels no force (its self-pair contributes an
    exact zero); two and three bodies match the oracle."""
    x = _x(n, 40 + n)
    ode, _ = orc.nbody_ode(n, 0.05, 1.0 / n)
    ref = orc.rhs(ode, x)
    got64 = gb.nbody_rhs_f64(x, n, 0.05, 1.0 / n, tile=gb.tiling(1, 1, 0)).cpu().numpy()
    np.testing.assert_array_equal(got64, ref)
    gotmx = gb.nbody_rhs_mixed(x, n, 0.05, 1.0 / n).cpu().numpy()
    np.testing.assert_array_equal(gotmx[: 3 * n], ref[: 3 * n])
    if n == 1:
        assert np.all(gotmx[3:] == 0.0)
    else:
        assert _rel(gotmx[3 * n:], ref[3 * n:]) <= 1e-6


def test_empty_system_rejected(gb, torch_cuda):
    with pytest.raises(gb.GbError):
        gb.nbody_rhs_f64(np.zeros(0), 0, 0.05, 1.0)


@pytest.mark.parametrize("n", [131072, 262144])
def test_rhs_mixed_large_system_properties(gb, torch_cuda, n):
    """Full-size checks up to configuration 5's N = 262144 (cold collapse,
    eps = 0.002): the mixed accelerations stay within 1e-6 of FP64 normwise
    and for 99.9 % of the bodies, and the total force vanishes (pair terms
    are antisymmetric) to FP32 summation accuracy."""
    torch = torch_cuda
    soft = 0.002
    x = gb.ic_cold_sphere(n, 9, 0.01)
    ref = gb.nbody_rhs_f64(x, n, soft, 1.0 / n, tile=gb.tiling(f64_pair=1))
    got = gb.nbody_rhs_mixed(x, n, soft, 1.0 / n)
    a64 = ref[3 * n:].view(-1, 3)
    amx = got[3 * n:].view(-1, 3)
    rel = ((amx - a64).norm() / a64.norm()).item()
    assert rel <= 1e-6, rel
    per = (amx - a64).norm(dim=1) / a64.norm(dim=1)
    assert per.quantile(0.999).item() <= 1e-6
    net = amx.sum(0).norm().item() / amx.norm(dim=1).sum().item()
    assert net <= 1e-6, net
    assert torch.equal(got[: 3 * n], ref[: 3 * n])
