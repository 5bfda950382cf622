"""The allocation-free mixed-precision right-hand side.

Some callers cannot allocate device memory (a host that hands this library a
fixed slice of the GPU and refuses further cudaMalloc, or a per-stage caller
that cannot afford cudaMalloc/cudaFree around every call).  For them
gb_nbody_rhs_mixed_noalloc takes its scratch from a fixed array inside the
library.  This file is collected last on purpose: if it fails, a run that
stops at the first failure has already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _call_noalloc(gb, torch, x, n, soft, mass):
    out = torch.empty_like(x)
    rc = gb.lib().gb_nbody_rhs_mixed_noalloc(x.data_ptr(), out.data_ptr(), n, soft, mass, None,
                                             None, C.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == 0, gb.lib().gb_status_string(rc)
    torch.cuda.synchronize()
    return out.cpu().numpy()


def test_noalloc_matches_workspace_entry_point_twice(gb, torch_cuda):
    torch = torch_cuda
    # two calls in a row on different systems: the shared scratch keeps the
    # previous call's contents, which must not leak into the next result
    for n, seed, soft in ((4096, 21, 0.005), (1500, 22, 0.01)):
        x = gb.to_device(gb.ic_plummer(n, seed))
        ref = gb.nbody_rhs_mixed(x, n, soft, 1.0 / n).cpu().numpy()
        got = _call_noalloc(gb, torch, x, n, soft, 1.0 / n)
        # both entry points run the same packing and force kernels with the
        # same geometry: the results are identical bit for bit
        np.testing.assert_array_equal(got, ref)


def test_noalloc_rejects_what_the_workspace_entry_point_rejects(gb, torch_cuda):
    torch = torch_cuda
    n = 64
    x = torch.zeros(6 * n, dtype=torch.float64, device="cuda")
    out = torch.empty_like(x)
    for soft, mass in ((float("inf"), 1.0 / n), (float("nan"), 1.0 / n), (0.0, 1.0 / n),
                       (0.01, 0.0)):
        rc = gb.lib().gb_nbody_rhs_mixed_noalloc(x.data_ptr(), out.data_ptr(), n, soft, mass,
                                                 None, None, None)
        assert rc == -1, (soft, mass, rc)  # GB_ERR_INVALID_ARGUMENT
    assert gb.lib().gb_nbody_rhs_mixed_noalloc(None, out.data_ptr(), n, 0.01, 1.0 / n, None,
                                               None, None) == -1


def test_noalloc_rejects_sizes_beyond_its_scratch(gb, torch_cuda):
    torch = torch_cuda
    cap = gb.lib().gb_nbody_rhs_mixed_noalloc_max_bodies()
    assert cap == 65536
    n = cap + 1
    x = torch.zeros(6 * n, dtype=torch.float64, device="cuda")
    out = torch.empty_like(x)
    rc = gb.lib().gb_nbody_rhs_mixed_noalloc(x.data_ptr(), out.data_ptr(), n, 0.01, 1.0 / n, None,
                                             None, None)
    assert rc == -7  # GB_ERR_CAPACITY
