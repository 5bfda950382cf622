"""CPU tests of the C ABI: the library loads without a GPU and exports every
symbol include/gbode.h declares; host-only entry points (initial conditions,
tableaus, MLP initialisation) behave."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from conftest import ROOT

HEADER = os.path.join(ROOT, "include", "gbode.h")


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    names = re.findall(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b(gb_\w+)\s*\(", src, re.M)
    return sorted(set(n for n in names if not n.endswith("_t")))


def test_header_declares_entry_points():
    names = declared_functions()
    assert "gb_nbody_rhs_f64" in names and "gb_integrator_create" in names
    assert len(names) >= 40


def test_library_exports_every_declared_symbol(gb):
    lib = gb.lib()
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_binding_covers_header(gb):
    assert set(declared_functions()) <= set(gb.SIGNATURES), \
        set(declared_functions()) - set(gb.SIGNATURES)


def test_struct_sizes_match_header(gb):
    # sizes the C side uses (gb_tableau has 3 ints + padding + 16x16 + 2x16 doubles)
    assert C.sizeof(gb.GbTableau) == 4 * 3 + 4 + 8 * (16 * 16 + 32)
    assert C.sizeof(gb.GbStepLog) == 20 * 4
    assert C.sizeof(gb.GbMlp) == 4 * (64 * 16 + 64 + 64 * 64 + 64 + 64 + 1 + 16 + 16 + 2)


def test_status_strings(gb):
    lib = gb.lib()
    assert lib.gb_status_string(0) == b"ok"
    assert lib.gb_status_string(-5) == b"attempt budget exhausted"
    assert lib.gb_version() >= 10000


@pytest.mark.parametrize("name", ["HE21", "RKF45", "DOPRI5", "DVERK", "RKF78"])
def test_builtin_tableaus_match_oracle(gb, orc, name):
    t = gb.tableau(name)
    o = orc.tableau(name)
    assert (t.n_stages, t.p, t.pt) == (o.n_stages, o.p, o.pt)
    for r in range(16):
        assert list(t.a[r]) == list(o.a[r])
    assert list(t.b) == list(o.b) and list(t.bt) == list(o.bt)
    # consistency: row sums of a are the nodes c_s, b and bt sum to one
    assert sum(t.b) == pytest.approx(1.0, abs=1e-14)
    assert sum(t.bt) == pytest.approx(1.0, abs=1e-14)


def test_invalid_arguments_rejected_without_gpu(gb):
    lib = gb.lib()
    t = gb.GbTableau()
    assert lib.gb_tableau_builtin(99, C.byref(t)) == -1
    assert lib.gb_nbody_rhs_f64(None, None, 10, 0.1, 1.0, None, None, None) == -1
    assert lib.gb_rk_norm_workspace_bytes(0) == 0


def test_initial_conditions_deterministic_and_centred(gb):
    a = gb.ic_uniform_ball(512, 5, 0.1)
    b = gb.ic_uniform_ball(512, 5, 0.1)
    c = gb.ic_uniform_ball(512, 6, 0.1)
    np.testing.assert_array_equal(a, b)
    assert not np.array_equal(a, c)
    pos = a[: 3 * 512].reshape(-1, 3)
    vel = a[3 * 512:].reshape(-1, 3)
    np.testing.assert_allclose(pos.mean(0), 0, atol=1e-15)
    np.testing.assert_allclose(vel.mean(0), 0, atol=1e-15)
    assert np.sqrt((pos ** 2).sum(1)).max() < 1.0 + 0.2
    assert vel.std() == pytest.approx(0.1, rel=0.1)


def test_plummer_mass_profile(gb):
    n = 16384
    x = gb.ic_plummer(n, 1)
    r = np.sqrt((x[: 3 * n].reshape(-1, 3) ** 2).sum(1))
    for rr in (0.5, 1.0, 2.0):
        analytic = rr ** 3 / (1 + rr ** 2) ** 1.5
        assert (r < rr).mean() == pytest.approx(analytic, abs=0.02)
    # virial equilibrium of the sampled DF: 2K ~ |W| (unsoftened estimate on a subsample)
    v = x[3 * n:].reshape(-1, 3)
    k = 0.5 * (v ** 2).sum() / n
    assert k == pytest.approx(3 * np.pi / 64, rel=0.05)  # K = 3 pi / 64 for a = 1


def test_virial_rescale_and_binaries(gb):
    x = gb.ic_plummer(256, 3)
    y = gb.ic_set_virial_ratio(x, 0.5, 0.01)
    assert not np.array_equal(x, y)
    z = gb.ic_binary_plummer(1000, 4, 0.1, 1e-3, 1e-2)
    pos = z[:3000].reshape(-1, 3)
    d = np.sqrt(((pos[0:100:2] - pos[1:100:2]) ** 2).sum(1))
    assert d.min() >= 1e-3 * 0.999 and d.max() <= 1e-2 * 1.001


def test_mlp_init_host(gb):
    m = gb.GbMlp()
    assert gb.lib().gb_mlp_init(C.byref(m), 123) == 0
    w1 = np.ctypeslib.as_array(m.w1)
    assert np.abs(w1).max() <= np.sqrt(6 / 80) + 1e-6 and np.abs(w1).std() > 0
    assert list(m.in_scale) == [1.0] * 16 and m.out_scale == 1.0


def _header_enum(name):
    src = re.sub(r"/\*.*?\*/", "", open(HEADER).read(), flags=re.S)
    m = re.search(r"\b" + name + r"\s*=\s*(\d+)", src)
    assert m, name
    return int(m.group(1))


def test_binding_enums_match_header(gb):
    assert gb.PREC == {"f64": _header_enum("GB_PREC_F64"), "mixed": _header_enum("GB_PREC_MIXED")}
    assert gb.CONTROLLERS == {"reference": _header_enum("GB_CTRL_REFERENCE"),
                              "pi": _header_enum("GB_CTRL_PI"),
                              "learned": _header_enum("GB_CTRL_LEARNED")}


def test_executor_options_reach_the_c_struct(gb):
    """Gb300Executor -> gb_integrate_opts, field by field (no GPU)."""
    mlp = gb.GbMlp()
    exe = gb.Gb300Executor(precision="mixed", controller="learned", exact=False, fsal=False,
                           attempts_per_sync=5, tile=gb.tiling(16, 1, 0, mixed_variant=3),
                           max_attempts=77, pi_beta=0.06, mlp=mlp, log_steps=9,
                           spatial_sort=True, host_wait_timeout_s=1.5)
    o = exe.opts(record=True)
    assert (o.precision, o.controller, o.fsal, o.exact) == (1, 2, 0, 0)
    assert (o.attempts_per_sync, o.record, o.max_attempts, o.log_steps, o.spatial_sort) == \
        (5, 1, 77, 9, 1)
    assert o.pi_beta == 0.06 and o.host_wait_timeout_s == 1.5
    assert (o.tiling.j_split, o.tiling.lanes, o.tiling.bodies_per_cta,
            o.tiling.mixed_variant) == (16, 1, 0, 3)
    assert o.mlp == C.addressof(mlp)
    d = gb.Gb300Executor().opts(record=False)
    assert (d.precision, d.controller, d.fsal, d.exact, d.record, d.mlp) == (0, 0, 1, 0, 0, None)
    assert gb.tiling(scalar=True).mixed_variant == 1


# ctypes mirror -> C typedef in include/gbode.h
_STRUCTS = {"GbTableau": "gb_tableau", "GbForceTiling": "gb_force_tiling",
            "GbMlp": "gb_mlp", "GbStepLog": "gb_step_log", "GbNBodySystem": "gb_nbody_system",
            "GbIntegrateOpts": "gb_integrate_opts", "GbIntegrateStats": "gb_integrate_stats",
            "GbBatchTiling": "gb_batch_tiling", "GbBatchOpts": "gb_batch_opts"}


def test_struct_layouts_match_the_c_compiler(gb, tmp_path):
    """Every ctypes mirror has the size and field offsets the C compiler
    gives the header's struct (a field added on one side only fails here)."""
    import shutil
    import subprocess
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    lines = ['#include <stddef.h>', '#include <stdio.h>', '#include "gbode.h"', "int main(void) {"]
    for py, c in _STRUCTS.items():
        lines.append(f'  printf("{py} size %zu\\n", sizeof({c}));')
        for f, _ in getattr(gb, py)._fields_:
            lines.append(f'  printf("{py} {f} %zu\\n", offsetof({c}, {f}));')
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run([cc, "-std=c11", f"-I{os.path.join(ROOT, 'include')}", str(src), "-o",
                    str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    for line in out.splitlines():
        py, field, value = line.split()
        cls = getattr(gb, py)
        got = C.sizeof(cls) if field == "size" else getattr(cls, field).offset
        assert got == int(value), (py, field, got, int(value))
