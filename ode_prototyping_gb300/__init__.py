"""GB300 (sm_103a) adaptive embedded Runge-Kutta N-body integrator.

Python binding of ``libgbode.so`` (C ABI declared in ``include/gbode.h``).
The names mirror the reference's C++ interface (noether17/ode_prototyping):

* ``RKEmbeddedParallel(tableau).integrate(x0, t0, tf, atol, rtol, ode,
  output, exe)`` -- ``src/integrator/RKEmbeddedParallel/RKEmbeddedParallel.hpp:15-19``
* ``NBodyODE(n_particles, softening)`` -- ``src/ode/NBodyODE.hpp:9-46``
* ``RawOutput`` with ``save_state(t, x)`` -- ``src/output/RawOutput.hpp:8-27``
* ``Gb300Executor`` -- the executor argument (``src/par_exec/*Executor``)

There is no CPU fallback: importing works without a GPU (for the symbol
checks), but every compute call goes through the CUDA library and raises if
it is missing or if no GPU is present.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass, field

import numpy as np

from . import build as _build

LIB_PATH = _build.LIB

# ----------------------------------------------------------------------------
# C structures (include/gbode.h)
# ----------------------------------------------------------------------------
MAX_STAGES = 16
MLP_IN = 16
MLP_HIDDEN = 64

GB_OK = 0
STATUS = {0: "ok", -1: "invalid argument", -2: "CUDA error", -3: "unsupported",
          -4: "not finite", -5: "budget exhausted", -6: "timeout", -7: "capacity",
          -8: "step underflow"}
GB_ERR_NOT_FINITE, GB_ERR_BUDGET, GB_ERR_TIMEOUT = -4, -5, -6
TABLEAU_IDS = {"HE21": 0, "RKF45": 1, "DOPRI5": 2, "DVERK": 3, "RKF78": 4}
PREC = {"f64": 0, "mixed": 1}
CONTROLLERS = {"reference": 0, "pi": 1, "learned": 2}


class GbTableau(C.Structure):
    _fields_ = [("n_stages", C.c_int32), ("p", C.c_int32), ("pt", C.c_int32),
                ("a", (C.c_double * MAX_STAGES) * MAX_STAGES),
                ("b", C.c_double * MAX_STAGES), ("bt", C.c_double * MAX_STAGES)]


class GbForceTiling(C.Structure):
    _fields_ = [("j_split", C.c_int32), ("lanes", C.c_int32), ("bodies_per_cta", C.c_int32),
                ("mixed_variant", C.c_int32), ("f64_pair", C.c_int32)]


class GbNBodySystem(C.Structure):
    _fields_ = [("n_particles", C.c_int64), ("softening", C.c_double), ("mass", C.c_double),
                ("masses_dev", C.c_void_p)]


class GbIntegrateOpts(C.Structure):
    _fields_ = [("precision", C.c_int32), ("controller", C.c_int32), ("fsal", C.c_int32),
                ("exact", C.c_int32), ("attempts_per_sync", C.c_int32), ("record", C.c_int32),
                ("max_attempts", C.c_int64), ("host_wait_timeout_s", C.c_double),
                ("pi_beta", C.c_double), ("tiling", GbForceTiling), ("mlp", C.c_void_p),
                ("log_steps", C.c_int32), ("spatial_sort", C.c_int32)]


class GbIntegrateStats(C.Structure):
    _fields_ = [("n_accepted", C.c_int64), ("n_rejected", C.c_int64), ("n_attempts", C.c_int64),
                ("n_rhs", C.c_int64), ("n_rhs_saved", C.c_int64), ("t", C.c_double),
                ("dt", C.c_double), ("dt_initial", C.c_double), ("err_last", C.c_double),
                ("interactions", C.c_double), ("status", C.c_int32), ("done", C.c_int32),
                ("n_learned_proposals", C.c_int64), ("n_learned_rejected", C.c_int64)]


class GbMlp(C.Structure):
    _fields_ = [("w1", (C.c_float * MLP_IN) * MLP_HIDDEN), ("b1", C.c_float * MLP_HIDDEN),
                ("w2", (C.c_float * MLP_HIDDEN) * MLP_HIDDEN), ("b2", C.c_float * MLP_HIDDEN),
                ("w3", C.c_float * MLP_HIDDEN), ("b3", C.c_float),
                ("in_mean", C.c_float * MLP_IN), ("in_scale", C.c_float * MLP_IN),
                ("out_scale", C.c_float), ("out_bias", C.c_float)]


class GbBatchTiling(C.Structure):
    _fields_ = [("threads_per_cta", C.c_int32), ("lanes", C.c_int32),
                ("bodies_per_thread", C.c_int32), ("grid_ctas", C.c_int32),
                ("systems_per_cta", C.c_int32)]


class GbBatchOpts(C.Structure):
    _fields_ = [("precision", C.c_int32), ("controller", C.c_int32), ("fsal", C.c_int32),
                ("attempts_per_sync", C.c_int32), ("max_attempts", C.c_int64),
                ("host_wait_timeout_s", C.c_double), ("pi_beta", C.c_double),
                ("tiling", GbBatchTiling), ("mlp", C.c_void_p)]


class GbStepLog(C.Structure):
    _fields_ = [("feat", C.c_float * MLP_IN), ("log_dt", C.c_float), ("log_err", C.c_float),
                ("accepted", C.c_float), ("log_dt_ideal", C.c_float)]


SAVE_FN = C.CFUNCTYPE(None, C.c_void_p, C.c_double, C.POINTER(C.c_double), C.c_int64)

_VP, _DP, _I64, _I32, _D = C.c_void_p, C.c_void_p, C.c_int64, C.c_int32, C.c_double

# name -> (restype, argtypes); every symbol include/gbode.h declares.
SIGNATURES = {
    "gb_status_string": (C.c_char_p, [C.c_int]),
    "gb_last_cuda_error": (C.c_int, []),
    "gb_version": (C.c_int, []),
    "gb_tableau_builtin": (C.c_int, [_I32, C.POINTER(GbTableau)]),
    "gb_device_alloc": (C.c_int, [C.POINTER(C.c_void_p), C.c_size_t]),
    "gb_device_free": (C.c_int, [_VP]),
    "gb_memcpy": (C.c_int, [_VP, _VP, C.c_size_t, _I32]),
    "gb_memset_zero": (C.c_int, [_VP, C.c_size_t]),
    "gb_fill_f64": (C.c_int, [_DP, _I64, _D, _VP]),
    "gb_stream_synchronize": (C.c_int, [_VP]),
    "gb_pointer_kind": (C.c_int, [_VP]),
    "gb_nbody_rhs_f64": (C.c_int, [_DP, _DP, _I64, _D, _D, _DP, C.POINTER(GbForceTiling), _VP]),
    "gb_nbody_acc_f64": (C.c_int, [_DP, _DP, _I64, _D, _D, _DP, _I32, C.POINTER(GbForceTiling),
                                   _VP]),
    "gb_nbody_mixed_workspace_bytes": (C.c_size_t, [_I64]),
    "gb_nbody_rhs_mixed": (C.c_int, [_DP, _DP, _I64, _D, _D, _DP, _VP, C.POINTER(GbForceTiling),
                                     _VP]),
    "gb_nbody_mixed_sorted_workspace_bytes": (C.c_size_t, [_I64]),
    "gb_nbody_rhs_mixed_sorted": (C.c_int, [_DP, _DP, _I64, _D, _D, _DP, _VP, C.c_size_t,
                                            C.POINTER(GbForceTiling), _VP]),
    "gb_nbody_rhs_mixed_noalloc_max_bodies": (C.c_int64, []),
    "gb_nbody_rhs_mixed_noalloc": (C.c_int, [_DP, _DP, _I64, _D, _D, _DP,
                                             C.POINTER(GbForceTiling), _VP]),
    "gb_rk_stage_f64": (C.c_int, [C.POINTER(GbTableau), _I32, _D, _DP, _DP, _DP, _I64, _VP]),
    "gb_rk_update_state_and_error_f64": (C.c_int, [C.POINTER(GbTableau), _D, _DP, _DP, _DP, _DP,
                                                   _I64, _VP]),
    "gb_rk_error_target_f64": (C.c_int, [_DP, _DP, _DP, _DP, _DP, _I64, _VP]),
    "gb_rk_norm_workspace_bytes": (C.c_size_t, [_I64]),
    "gb_rk_norm_f64": (C.c_int, [_DP, _DP, _I64, _VP, C.c_size_t, _DP, _VP]),
    "gb_rk_scaled_sq_sum_f64": (C.c_int, [_DP, _DP, _I64, _VP, C.c_size_t,
                                          C.POINTER(C.c_double), _VP]),
    "gb_mlp_init": (C.c_int, [C.POINTER(GbMlp), C.c_uint64]),
    "gb_mlp_act_floats": (C.c_int64, [_I64]),
    "gb_mlp_forward_f32": (C.c_int, [_VP, _VP, _VP, _I64, _VP, _VP]),
    "gb_mlp_backward_workspace_bytes": (C.c_size_t, [_I64]),
    "gb_mlp_backward_f32": (C.c_int, [_VP, _VP, _VP, _VP, _VP, _I64, _VP, _VP]),
    "gb_mlp_adam_step": (C.c_int, [_VP, _VP, _VP, _VP, C.c_float, C.c_float, C.c_float,
                                   C.c_float, _I32, _VP]),
    "gb_mlp_infer_bf16": (C.c_int, [_VP, _VP, _VP, _I64, _VP]),
    "gb_mlp_train": (C.c_int, [_VP, _VP, _VP, _I64, _I32, C.c_float, C.c_float,
                               C.POINTER(C.c_float), _VP]),
    "gb_integrator_create": (C.c_int, [C.POINTER(GbTableau), C.POINTER(GbNBodySystem),
                                       C.POINTER(GbIntegrateOpts), _VP, C.POINTER(C.c_void_p)]),
    "gb_integrator_start": (C.c_int, [_VP, _DP, _D, _D, _DP, _DP, _D, _D, SAVE_FN, _VP]),
    "gb_integrator_advance": (C.c_int, [_VP, _I64, SAVE_FN, _VP]),
    "gb_integrator_enqueue": (C.c_int, [_VP, _I64]),
    "gb_integrator_sync": (C.c_int, [_VP]),
    "gb_integrator_stats": (C.c_int, [_VP, C.POINTER(GbIntegrateStats)]),
    "gb_integrator_state": (C.c_int, [_VP, _DP, C.POINTER(C.c_double)]),
    "gb_integrator_destroy": (C.c_int, [_VP]),
    "gb_integrator_log": (C.c_int, [_VP, C.POINTER(GbStepLog), _I64, C.POINTER(C.c_int64)]),
    "gb_integrator_launch_stage": (C.c_int, [_VP, _I32]),
    "gb_integrator_set_dense_output": (C.c_int, [_VP, C.POINTER(C.c_double), _I64]),
    "gb_integrator_dense_output": (C.c_int, [_VP, C.POINTER(C.c_double), _I64,
                                             C.POINTER(C.c_int64)]),
    "gb_integrator_geometry": (C.c_int, [_VP, C.POINTER(GbForceTiling), C.POINTER(C.c_int64)]),
    "gb_integrate_nbody": (C.c_int, [C.POINTER(GbTableau), C.POINTER(GbNBodySystem),
                                     C.POINTER(GbIntegrateOpts), _DP, _D, _D, _DP, _DP, _D, _D,
                                     SAVE_FN, _VP, _DP, C.POINTER(GbIntegrateStats), _VP]),
    "gb_batch_create": (C.c_int, [C.POINTER(GbTableau), _I32, C.POINTER(C.c_int64),
                                  C.POINTER(C.c_double), C.POINTER(C.c_double),
                                  C.POINTER(GbBatchOpts), _VP, C.POINTER(C.c_void_p)]),
    "gb_batch_start": (C.c_int, [_VP, _DP, C.POINTER(C.c_double), C.POINTER(C.c_double),
                                 C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    "gb_batch_advance": (C.c_int, [_VP, _I64]),
    "gb_batch_enqueue": (C.c_int, [_VP, _I64]),
    "gb_batch_sync": (C.c_int, [_VP]),
    "gb_batch_stats": (C.c_int, [_VP, C.POINTER(GbIntegrateStats), C.POINTER(GbIntegrateStats)]),
    "gb_batch_state": (C.c_int, [_VP, _DP, C.POINTER(C.c_double)]),
    "gb_batch_launch_stage": (C.c_int, [_VP, _I32]),
    "gb_batch_autotune": (C.c_int, [_VP, _I32, C.POINTER(GbBatchTiling), C.POINTER(C.c_double)]),
    "gb_batch_geometry": (C.c_int, [_VP, C.POINTER(GbBatchTiling), C.POINTER(C.c_int64)]),
    "gb_batch_destroy": (C.c_int, [_VP]),
    "gb_leapfrog_nbody": (C.c_int, [C.POINTER(GbNBodySystem), _DP, _D, _D, _D, _I32,
                                    C.POINTER(GbForceTiling), SAVE_FN, _VP,
                                    C.POINTER(C.c_int64), _VP]),
    "gb_trajectory_open": (C.c_int, [C.c_char_p, _I64, _D, C.POINTER(C.c_void_p)]),
    "gb_trajectory_append": (C.c_int, [_VP, _D, C.POINTER(C.c_double)]),
    "gb_trajectory_save": (None, [_VP, _D, C.POINTER(C.c_double), _I64]),
    "gb_trajectory_close": (C.c_int, [_VP, C.POINTER(C.c_int64)]),
    "gb_nbody_energy_workspace_bytes": (C.c_size_t, [_I64]),
    "gb_nbody_energy_f64": (C.c_int, [_DP, _I64, _D, _D, _DP, _VP, C.c_size_t, _DP, _VP]),
    "gb_ic_uniform_ball": (C.c_int, [_I64, C.c_uint64, _D, C.POINTER(C.c_double)]),
    "gb_ic_plummer": (C.c_int, [_I64, C.c_uint64, _D, C.POINTER(C.c_double)]),
    "gb_ic_set_virial_ratio": (C.c_int, [_I64, _D, _D, C.POINTER(C.c_double)]),
    "gb_ic_cold_sphere": (C.c_int, [_I64, C.c_uint64, _D, C.POINTER(C.c_double)]),
    "gb_ic_binary_plummer": (C.c_int, [_I64, C.c_uint64, _D, _D, _D, C.POINTER(C.c_double)]),
}

_lib = None


class GbError(RuntimeError):
    def __init__(self, status: int, where: str):
        super().__init__(f"{where}: {STATUS.get(status, status)} (status {status}, "
                         f"cuda error {lib().gb_last_cuda_error() if _lib else '?'})")
        self.status = status


def lib() -> C.CDLL:
    """Loads libgbode.so (built in-tree); raises if it is missing."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"libgbode.so not built ({LIB_PATH}); run __graft_entry__.build()")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def check(status: int, where: str) -> None:
    if status != GB_OK:
        raise GbError(status, where)


# ----------------------------------------------------------------------------
# device helpers (torch provides device memory and streams)
# ----------------------------------------------------------------------------
def _torch():
    import torch
    if not torch.cuda.is_available():
        raise RuntimeError("no CUDA device: the GB300 library has no CPU fallback")
    return torch


def _ptr(t) -> int | None:
    return None if t is None else t.data_ptr()


def _stream(stream=None):
    torch = _torch()
    s = stream if stream is not None else torch.cuda.current_stream()
    return C.c_void_p(s.cuda_stream)


def to_device(x, dtype=None):
    torch = _torch()
    if isinstance(x, torch.Tensor):
        return x.to(device="cuda", dtype=dtype or x.dtype).contiguous()
    return torch.as_tensor(np.ascontiguousarray(x), dtype=dtype or torch.float64,
                           device="cuda").contiguous()


def tableau(name_or_struct) -> GbTableau:
    if isinstance(name_or_struct, GbTableau):
        return name_or_struct
    t = GbTableau()
    check(lib().gb_tableau_builtin(TABLEAU_IDS[name_or_struct], C.byref(t)), "gb_tableau_builtin")
    return t


def tiling(j_split=0, lanes=0, bodies_per_cta=0, scalar=False,
           mixed_variant=0, f64_pair=0) -> GbForceTiling:
    """Force-kernel tiling.  Mixed precision: scalar=True (or mixed_variant=1)
    selects the scalar FP32 pair loop, mixed_variant=2 / 3 the packed f32x2
    loop over pairs of partners with two bodies / one body per thread, 0 the
    library's choice (3).  FP64: f64_pair=1 the refined-rsqrt pair term,
    2 the reference's operation order, 0 the entry point's default."""
    return GbForceTiling(j_split, lanes, bodies_per_cta, 1 if scalar else mixed_variant, f64_pair)


# ----------------------------------------------------------------------------
# right-hand side
# ----------------------------------------------------------------------------
def nbody_rhs_f64(x, n_particles: int, softening: float, mass: float = 1.0, masses=None,
                  tile: GbForceTiling | None = None, out=None, stream=None):
    """dxdt = f(x) of NBodyODE (FP64, reference operation order)."""
    x = to_device(x)
    out = out if out is not None else _torch().empty_like(x)
    check(lib().gb_nbody_rhs_f64(_ptr(x), _ptr(out), n_particles, softening, mass,
                                 _ptr(masses), C.byref(tile) if tile else None, _stream(stream)),
          "gb_nbody_rhs_f64")
    return out


def nbody_acc_f64(pos, n_particles: int, softening: float, mass: float = 1.0, masses=None,
                  accumulate: bool = False, out=None, tile=None, stream=None):
    pos = to_device(pos)
    out = out if out is not None else _torch().zeros(3 * n_particles, dtype=_torch().float64,
                                                     device="cuda")
    check(lib().gb_nbody_acc_f64(_ptr(pos), _ptr(out), n_particles, softening, mass,
                                 _ptr(masses), 1 if accumulate else 0,
                                 C.byref(tile) if tile else None, _stream(stream)),
          "gb_nbody_acc_f64")
    return out


def nbody_rhs_mixed(x, n_particles: int, softening: float, mass: float = 1.0, masses=None,
                    tile: GbForceTiling | None = None, out=None, work=None, stream=None):
    torch = _torch()
    x = to_device(x)
    out = out if out is not None else torch.empty_like(x)
    if work is None:
        nb = lib().gb_nbody_mixed_workspace_bytes(n_particles)
        work = torch.empty(nb, dtype=torch.uint8, device="cuda")
    check(lib().gb_nbody_rhs_mixed(_ptr(x), _ptr(out), n_particles, softening, mass,
                                   _ptr(masses), _ptr(work), C.byref(tile) if tile else None,
                                   _stream(stream)), "gb_nbody_rhs_mixed")
    return out


def nbody_rhs_mixed_sorted(x, n_particles: int, softening: float, mass: float = 1.0,
                           masses=None, tile: GbForceTiling | None = None, out=None,
                           stream=None):
    """Mixed-precision RHS on Morton-sorted tiles with the far-field path."""
    torch = _torch()
    x = to_device(x)
    out = out if out is not None else torch.empty_like(x)
    nb = lib().gb_nbody_mixed_sorted_workspace_bytes(n_particles)
    work = torch.empty(nb + 256, dtype=torch.uint8, device="cuda")
    base = (work.data_ptr() + 255) // 256 * 256
    check(lib().gb_nbody_rhs_mixed_sorted(_ptr(x), _ptr(out), n_particles, softening, mass,
                                          _ptr(masses), base, nb,
                                          C.byref(tile) if tile else None, _stream(stream)),
          "gb_nbody_rhs_mixed_sorted")
    return out


def energy(x, n_particles: int, softening: float, mass: float = 1.0, masses=None, stream=None):
    torch = _torch()
    x = to_device(x)
    nb = lib().gb_nbody_energy_workspace_bytes(n_particles)
    work = torch.empty(nb, dtype=torch.uint8, device="cuda")
    out = torch.zeros(8, dtype=torch.float64, device="cuda")
    check(lib().gb_nbody_energy_f64(_ptr(x), n_particles, softening, mass, _ptr(masses),
                                    _ptr(work), nb, _ptr(out), _stream(stream)),
          "gb_nbody_energy_f64")
    o = out.cpu().numpy()
    return {"ke": o[0], "pe": o[1], "e": o[0] + o[1], "p": o[2:5].copy(), "l": o[5:8].copy()}


# ----------------------------------------------------------------------------
# element-wise RK kernels
# ----------------------------------------------------------------------------
def rk_stage(tab, stage: int, dt: float, x0, ks, out, n_var: int, stream=None):
    t = tableau(tab)
    check(lib().gb_rk_stage_f64(C.byref(t), stage, dt, _ptr(x0), _ptr(ks), _ptr(out), n_var,
                                _stream(stream)), "gb_rk_stage_f64")


def rk_update(tab, dt: float, x0, ks, x, err, n_var: int, stream=None):
    t = tableau(tab)
    check(lib().gb_rk_update_state_and_error_f64(C.byref(t), dt, _ptr(x0), _ptr(ks), _ptr(x),
                                                 _ptr(err), n_var, _stream(stream)),
          "gb_rk_update_state_and_error_f64")


def rk_error_target(atol, rtol, x, x0, out, n_var: int, stream=None):
    check(lib().gb_rk_error_target_f64(_ptr(atol), _ptr(rtol), _ptr(x), _ptr(x0), _ptr(out),
                                       n_var, _stream(stream)), "gb_rk_error_target_f64")


def rk_norm(v, scale, n: int, stream=None):
    """rk_norm of the reference: sqrt(sum (v/scale)^2 / n), result on device."""
    torch = _torch()
    nb = lib().gb_rk_norm_workspace_bytes(n)
    work = torch.empty(nb, dtype=torch.uint8, device="cuda")
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    check(lib().gb_rk_norm_f64(_ptr(v), _ptr(scale), n, _ptr(work), nb, _ptr(out),
                               _stream(stream)), "gb_rk_norm_f64")
    return out


# ----------------------------------------------------------------------------
# initial conditions
# ----------------------------------------------------------------------------
def _ic(fn, n, *args):
    x = np.zeros(6 * n)
    check(fn(n, *args, x.ctypes.data_as(C.POINTER(C.c_double))), fn.__name__)
    return x


def ic_uniform_ball(n: int, seed: int, sigma_v: float = 0.1) -> np.ndarray:
    return _ic(lib().gb_ic_uniform_ball, n, seed, sigma_v)


def ic_plummer(n: int, seed: int, a: float = 1.0) -> np.ndarray:
    return _ic(lib().gb_ic_plummer, n, seed, a)


def ic_cold_sphere(n: int, seed: int, noise: float = 0.01) -> np.ndarray:
    return _ic(lib().gb_ic_cold_sphere, n, seed, noise)


def ic_binary_plummer(n: int, seed: int, frac: float = 0.1, amin: float = 1e-3,
                      amax: float = 1e-2) -> np.ndarray:
    return _ic(lib().gb_ic_binary_plummer, n, seed, frac, amin, amax)


def ic_set_virial_ratio(x: np.ndarray, q: float, softening: float) -> np.ndarray:
    x = np.ascontiguousarray(x, dtype=np.float64).copy()
    n = len(x) // 6
    check(lib().gb_ic_set_virial_ratio(n, q, softening, x.ctypes.data_as(C.POINTER(C.c_double))),
          "gb_ic_set_virial_ratio")
    return x


# ----------------------------------------------------------------------------
# reference-shaped host API
# ----------------------------------------------------------------------------
@dataclass
class NBodyODE:
    """NBodyODE<double, 6N>{softening} (src/ode/NBodyODE.hpp:9-46), with an
    optional uniform mass (applied after the pair sum) or per-body masses."""
    n_particles: int
    softening: float = 0.0
    mass: float = 1.0
    masses: object = None  # device tensor of N doubles

    @property
    def n_var(self) -> int:
        return 6 * self.n_particles

    def __call__(self, exe, x, dxdt):
        exe.rhs(self, x, dxdt)

    def acc(self, exe, x, acc):
        nbody_acc_f64(x[: 3 * self.n_particles], self.n_particles, self.softening, self.mass,
                      self.masses, out=acc, tile=exe.tile)


class RawOutput:
    """RawOutput (src/output/RawOutput.hpp:8-27): time and host copy of each
    saved state."""

    def __init__(self, keep_states: bool = True):
        self._times: list[float] = []
        self._states: list[np.ndarray] = []
        self.keep_states = keep_states

    def save_state(self, t: float, x: np.ndarray) -> None:
        self._times.append(t)
        if self.keep_states:
            self._states.append(np.array(x, copy=True))
        else:
            self._states[:] = [np.array(x, copy=True)]

    def times(self):
        return self._times

    def states(self):
        return self._states


@dataclass
class Gb300Executor:
    """Executor for the GB300 path: carries the precision, controller and
    tiling choices (the reference's executor carries its thread count)."""
    precision: str = "f64"
    controller: str = "reference"
    exact: bool = False
    fsal: bool = True
    attempts_per_sync: int = 16
    tile: GbForceTiling | None = None
    max_attempts: int = 0
    pi_beta: float = 0.04
    mlp: GbMlp | None = None
    log_steps: int = 0
    # mixed precision: 0 = default (from N = 8192 the partner-chunk stage on
    # Morton-sorted bodies with tile culling), 1 = the tile-centroid far-field
    # path, 2 = the sorted chunk stage without culling (same bits as 0),
    # 3 = the chunk stage in body order
    spatial_sort: int = 0
    host_wait_timeout_s: float = 600.0  # bound on each host wait for the device

    def rhs(self, ode: NBodyODE, x, dxdt):
        if self.precision == "f64":
            nbody_rhs_f64(x, ode.n_particles, ode.softening, ode.mass, ode.masses,
                          tile=self.tile, out=dxdt)
        else:
            nbody_rhs_mixed(x, ode.n_particles, ode.softening, ode.mass, ode.masses,
                            tile=self.tile, out=dxdt)

    def opts(self, record: bool) -> GbIntegrateOpts:
        o = GbIntegrateOpts()
        o.precision = PREC[self.precision]
        o.controller = CONTROLLERS[self.controller]
        o.fsal = 1 if self.fsal else 0
        o.exact = 1 if self.exact else 0
        o.attempts_per_sync = self.attempts_per_sync
        o.record = 1 if record else 0
        o.max_attempts = self.max_attempts
        o.host_wait_timeout_s = self.host_wait_timeout_s
        o.pi_beta = self.pi_beta
        if self.tile is not None:
            o.tiling = self.tile
        if self.mlp is not None:
            self._mlp_keep = self.mlp
            o.mlp = C.cast(C.pointer(self.mlp), C.c_void_p)
        o.log_steps = self.log_steps
        o.spatial_sort = int(self.spatial_sort)
        return o


class Integrator:
    """Stateful device-resident integrator (gb_integrator_*)."""

    def __init__(self, tab, ode: NBodyODE, exe: Gb300Executor, record: bool = False,
                 stream=None):
        self.tab = tableau(tab)
        self.ode = ode
        self.exe = exe
        self.record = record
        self.sys = GbNBodySystem(ode.n_particles, ode.softening, ode.mass,
                                 _ptr(ode.masses) if ode.masses is not None else None)
        self.opts = exe.opts(record)
        h = C.c_void_p()
        check(lib().gb_integrator_create(C.byref(self.tab), C.byref(self.sys),
                                         C.byref(self.opts), _stream(stream), C.byref(h)),
              "gb_integrator_create")
        self.h = h
        self._cb = None

    def _make_cb(self, output):
        if output is None:
            return SAVE_FN(), None
        n_var = self.ode.n_var

        def cb(_user, t, xp, n):
            x = np.ctypeslib.as_array(xp, shape=(n,))
            output.save_state(t, x)

        f = SAVE_FN(cb)
        self._cb = f
        return f, None

    def start(self, x0, t0: float, tf: float, atol, rtol, output=None):
        torch = _torch()
        x0 = to_device(x0)
        self._x0 = x0
        av = rv = None
        a_s = r_s = 0.0
        if np.ndim(atol) == 0 and not isinstance(atol, torch.Tensor):
            a_s = float(atol)
        else:
            av = to_device(atol)
        if np.ndim(rtol) == 0 and not isinstance(rtol, torch.Tensor):
            r_s = float(rtol)
        else:
            rv = to_device(rtol)
        self._tol = (av, rv)
        cb, _ = self._make_cb(output)
        check(lib().gb_integrator_start(self.h, _ptr(x0), t0, tf, _ptr(av), _ptr(rv), a_s, r_s,
                                        cb, None), "gb_integrator_start")

    def advance(self, max_attempts: int = 0, output=None) -> int:
        cb, _ = self._make_cb(output)
        return lib().gb_integrator_advance(self.h, max_attempts, cb, None)

    def enqueue(self, n_replays: int):
        check(lib().gb_integrator_enqueue(self.h, n_replays), "gb_integrator_enqueue")

    def sync(self):
        check(lib().gb_integrator_sync(self.h), "gb_integrator_sync")

    def stats(self) -> dict:
        s = GbIntegrateStats()
        check(lib().gb_integrator_stats(self.h, C.byref(s)), "gb_integrator_stats")
        return {f: getattr(s, f) for f, _ in GbIntegrateStats._fields_}

    def state(self):
        torch = _torch()
        out = torch.empty(self.ode.n_var, dtype=torch.float64, device="cuda")
        t = C.c_double(0.0)
        check(lib().gb_integrator_state(self.h, _ptr(out), C.byref(t)), "gb_integrator_state")
        return out, t.value

    def log(self, capacity: int = 1 << 20) -> np.ndarray:
        cnt = C.c_int64(0)
        check(lib().gb_integrator_log(self.h, None, 0, C.byref(cnt)), "gb_integrator_log")
        n = int(cnt.value)
        recs = (GbStepLog * max(n, 1))()
        check(lib().gb_integrator_log(self.h, recs, n, C.byref(cnt)), "gb_integrator_log")
        arr = np.ctypeslib.as_array(C.cast(recs, C.POINTER(C.c_float)), shape=(max(n, 1), 20))
        return arr[:n].copy()

    def set_dense_output(self, times):
        self._dense_t = np.ascontiguousarray(times, dtype=np.float64)
        check(lib().gb_integrator_set_dense_output(
            self.h, self._dense_t.ctypes.data_as(C.POINTER(C.c_double)), len(self._dense_t)),
            "gb_integrator_set_dense_output")

    def dense_output(self) -> np.ndarray:
        cnt = C.c_int64(0)
        n = len(getattr(self, "_dense_t", []))
        out = np.zeros((max(n, 1), self.ode.n_var))
        check(lib().gb_integrator_dense_output(self.h, out.ctypes.data_as(C.POINTER(C.c_double)),
                                               n, C.byref(cnt)), "gb_integrator_dense_output")
        return out[: int(cnt.value)]

    def launch_stage(self, stage: int):
        check(lib().gb_integrator_launch_stage(self.h, stage), "gb_integrator_launch_stage")

    def geometry(self) -> dict:
        t = GbForceTiling()
        n = C.c_int64(0)
        check(lib().gb_integrator_geometry(self.h, C.byref(t), C.byref(n)),
              "gb_integrator_geometry")
        bpt = {1: 2, 2: 2, 3: 1}.get(t.mixed_variant, 1)
        return {"j_split": t.j_split, "lanes": t.lanes, "bodies_per_cta": t.bodies_per_cta,
                "threads": t.bodies_per_cta * t.lanes // bpt, "mixed_variant": t.mixed_variant,
                "ctas": int(n.value)}

    def close(self):
        if getattr(self, "h", None):
            lib().gb_integrator_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class RKEmbeddedParallel:
    """RKEmbeddedParallel<ButcherTableau> with the reference's integrate
    signature (RKEmbeddedParallel.hpp:15-19), run device-resident."""

    def __init__(self, tab):
        self.tab = tableau(tab)

    def integrate(self, x0, t0, tf, atol, rtol, ode: NBodyODE, output, exe: Gb300Executor):
        it = Integrator(self.tab, ode, exe, record=output is not None)
        try:
            it.start(x0, t0, tf, atol, rtol, output)
            rc = it.advance(0, output)
            st = it.stats()
            if rc not in (GB_OK,):
                raise GbError(rc, "integrate")
            return st
        finally:
            it.close()


def _dbl(values):
    arr = np.ascontiguousarray(values, dtype=np.float64)
    return arr, arr.ctypes.data_as(C.POINTER(C.c_double))


class Batch:
    """Many independent N-body systems advanced together (gb_batch_*)."""

    def __init__(self, tab, n_particles, softening, mass=None, precision="f64",
                 controller="reference", attempts_per_sync=8, fsal=True, max_attempts=0,
                 tiling: GbBatchTiling | None = None, stream=None, mlp: GbMlp | None = None):
        self.tab = tableau(tab)
        self.n = np.ascontiguousarray(n_particles, dtype=np.int64)
        self.ns = len(self.n)
        self.offsets = np.concatenate([[0], np.cumsum(self.n)]) * 6
        self._soft, sp = _dbl(np.broadcast_to(softening, (self.ns,)))
        m = 1.0 / self.n if mass is None else np.broadcast_to(mass, (self.ns,))
        self._mass, mp = _dbl(m)
        o = GbBatchOpts()
        o.precision = PREC[precision]
        o.controller = CONTROLLERS[controller]
        o.fsal = 1 if fsal else 0
        o.attempts_per_sync = attempts_per_sync
        o.max_attempts = max_attempts
        o.host_wait_timeout_s = 600.0
        if tiling is not None:
            o.tiling = tiling
        if mlp is not None:
            self._mlp_keep = mlp
            o.mlp = C.cast(C.pointer(mlp), C.c_void_p)
        self.opts = o
        h = C.c_void_p()
        check(lib().gb_batch_create(C.byref(self.tab), self.ns,
                                    self.n.ctypes.data_as(C.POINTER(C.c_int64)), sp, mp,
                                    C.byref(o), _stream(stream), C.byref(h)), "gb_batch_create")
        self.h = h

    def start(self, x0_concat, t0, tf, atol, rtol):
        x0 = to_device(x0_concat)
        self._x0 = x0
        a = [_dbl(np.broadcast_to(v, (self.ns,))) for v in (t0, tf, atol, rtol)]
        self._keep = a
        check(lib().gb_batch_start(self.h, _ptr(x0), *(p for _, p in a)), "gb_batch_start")

    def advance(self, max_replays: int = 0) -> int:
        return lib().gb_batch_advance(self.h, max_replays)

    def enqueue(self, n: int):
        check(lib().gb_batch_enqueue(self.h, n), "gb_batch_enqueue")

    def sync(self):
        check(lib().gb_batch_sync(self.h), "gb_batch_sync")

    def stats(self, per_system: bool = False):
        tot = GbIntegrateStats()
        per = (GbIntegrateStats * self.ns)() if per_system else None
        check(lib().gb_batch_stats(self.h, C.byref(tot), per), "gb_batch_stats")
        d = {f: getattr(tot, f) for f, _ in GbIntegrateStats._fields_}
        if per_system:
            d["systems"] = [{f: getattr(p, f) for f, _ in GbIntegrateStats._fields_}
                            for p in per]
        return d

    def state(self):
        torch = _torch()
        out = torch.empty(int(self.offsets[-1]), dtype=torch.float64, device="cuda")
        t = np.zeros(self.ns)
        check(lib().gb_batch_state(self.h, _ptr(out), t.ctypes.data_as(C.POINTER(C.c_double))),
              "gb_batch_state")
        return out, t

    def system_state(self, x, k):
        return x[self.offsets[k]:self.offsets[k + 1]]

    def launch_stage(self, s: int):
        check(lib().gb_batch_launch_stage(self.h, s), "gb_batch_launch_stage")

    def autotune(self, reps: int = 3) -> dict:
        t = GbBatchTiling()
        ms = C.c_double(0)
        check(lib().gb_batch_autotune(self.h, reps, C.byref(t), C.byref(ms)), "gb_batch_autotune")
        return {"threads_per_cta": t.threads_per_cta, "lanes": t.lanes,
                "bodies_per_thread": t.bodies_per_thread, "grid_ctas": t.grid_ctas,
                "systems_per_cta": t.systems_per_cta, "stage_ms": ms.value}

    def geometry(self) -> dict:
        t = GbBatchTiling()
        nu = C.c_int64(0)
        check(lib().gb_batch_geometry(self.h, C.byref(t), C.byref(nu)), "gb_batch_geometry")
        return {"threads_per_cta": t.threads_per_cta, "lanes": t.lanes,
                "bodies_per_thread": t.bodies_per_thread, "grid_ctas": t.grid_ctas,
                "systems_per_cta": t.systems_per_cta, "units": int(nu.value)}

    def close(self):
        if getattr(self, "h", None):
            lib().gb_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class ParallelLeapfrogIntegrator:
    """ParallelLeapfrogIntegrator::integrate(x0, t0, tf, dt, ode, output, exe)
    (src/integrator/leapfrog/LeapfrogParallel.hpp:11-41) on the device."""

    @staticmethod
    def integrate(x0, t0: float, tf: float, dt: float, ode: NBodyODE, output,
                  exe: Gb300Executor):
        x = to_device(x0).clone()
        sysd = GbNBodySystem(ode.n_particles, ode.softening, ode.mass,
                             _ptr(ode.masses) if ode.masses is not None else None)
        cb = SAVE_FN()
        if output is not None:
            def _cb(_u, t, xp, n):
                output.save_state(t, np.ctypeslib.as_array(xp, shape=(n,)))
            cb = SAVE_FN(_cb)
        steps = C.c_int64(0)
        check(lib().gb_leapfrog_nbody(C.byref(sysd), _ptr(x), t0, tf, dt, PREC[exe.precision],
                                      C.byref(exe.tile) if exe.tile else None, cb, None,
                                      C.byref(steps), _stream()), "gb_leapfrog_nbody")
        return x, int(steps.value)


class TrajectoryWriter:
    """Trajectory file in the reference's binary format (gb_trajectory_*).
    Usable as an integrator output: ``save_state(t, x)``; or pass
    ``writer.c_save`` / ``writer.handle`` to the C save callback slot."""

    def __init__(self, path: str, n_var: int, softening: float):
        h = C.c_void_p()
        check(lib().gb_trajectory_open(path.encode(), n_var, softening, C.byref(h)),
              "gb_trajectory_open")
        self.handle = h
        self.n_var = n_var

    def save_state(self, t: float, x) -> None:
        x = np.ascontiguousarray(x, dtype=np.float64)
        check(lib().gb_trajectory_append(self.handle, t, x.ctypes.data_as(C.POINTER(C.c_double))),
              "gb_trajectory_append")

    def close(self) -> int:
        n = C.c_int64(0)
        if self.handle:
            check(lib().gb_trajectory_close(self.handle, C.byref(n)), "gb_trajectory_close")
            self.handle = None
        return int(n.value)


def read_trajectory(path: str):
    """(times, states, softening) of a file in the reference's format."""
    with open(path, "rb") as f:
        n_times, n_var = np.frombuffer(f.read(16), dtype="<u8")
        softening = float(np.frombuffer(f.read(8), dtype="<f8")[0])
        data = np.frombuffer(f.read(), dtype="<f8").reshape(int(n_times), int(n_var) + 1)
    return data[:, 0].copy(), data[:, 1:].copy(), softening


def exported_symbols() -> list[str]:
    return list(SIGNATURES)
