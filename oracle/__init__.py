"""CPU oracle for the adaptive embedded Runge-Kutta N-body path.

Test infrastructure only.  The tests, ``__graft_entry__.smoke()`` and the
CPU-baseline leg of ``bench.py`` import this package to compare the GPU results
against (or as the timed CPU implementation of the reference); the GPU library
never does.

Two back ends:

* ``liboracle.so`` -- ``gbode_oracle.c``, a plain-C restatement of the
  reference's integrator, tableaus, N-body right-hand side and executors
  (single-threaded and thread pool).  Always built (``make -C oracle``).
* ``libref.so`` -- the reference itself, compiled in place from its headers
  by ``make -C oracle ref`` where its sources are present.  Optional.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "_build", "liboracle.so")
REF_SO = os.path.join(HERE, "_ref", "libref.so")
# Where the reference's sources are read from (this container only; they do
# not travel to the GPU machine).  Every recipe and test takes it from here.
REF_ROOT = os.environ.get("GBODE_REFERENCE_ROOT", "/root/reference")

TABLEAUS = {"HE21": 0, "RKF45": 1, "DOPRI5": 2, "DVERK": 3, "RKF78": 4}
ODE_NBODY, ODE_EXPONENTIAL, ODE_VANDERPOL = 0, 1, 2
MAX_STAGES = 16


class Tableau(C.Structure):
    _fields_ = [
        ("n_stages", C.c_int),
        ("p", C.c_int),
        ("pt", C.c_int),
        ("a", (C.c_double * MAX_STAGES) * MAX_STAGES),
        ("b", C.c_double * MAX_STAGES),
        ("bt", C.c_double * MAX_STAGES),
    ]


class NBody(C.Structure):
    _fields_ = [
        ("n_particles", C.c_int64),
        ("softening", C.c_double),
        ("mass", C.c_double),
        ("masses", C.POINTER(C.c_double)),
    ]


class Ode(C.Structure):
    _fields_ = [("kind", C.c_int), ("nb", NBody), ("n_var", C.c_int64)]


class Stats(C.Structure):
    _fields_ = [
        ("n_saved", C.c_int64),
        ("n_attempts", C.c_int64),
        ("n_rejected", C.c_int64),
        ("n_rhs", C.c_int64),
        ("dt_initial", C.c_double),
        ("t_final", C.c_double),
        ("status", C.c_int),
    ]


_DP = C.POINTER(C.c_double)


def build(ref: bool | None = None, quiet: bool = True) -> None:
    """Compile the C restatement, and the in-place reference build when the
    reference sources are present (``ref=None``) or when asked."""
    out = subprocess.DEVNULL if quiet else None
    subprocess.run(["make", "-C", HERE, "all"], check=True, stdout=out)
    want_ref = os.path.isdir(os.path.join(REF_ROOT, "src")) if ref is None else ref
    if want_ref:
        subprocess.run(["make", "-C", HERE, "ref", f"REF_ROOT={REF_ROOT}"], check=True, stdout=out)


_lib = None
_ref = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(ORACLE_SO):
            build(ref=False)
        _lib = C.CDLL(ORACLE_SO)
        _lib.orc_rk_integrate.restype = C.c_int
        _lib.orc_rk_integrate.argtypes = [
            C.POINTER(Tableau), C.POINTER(Ode), _DP, C.c_double, C.c_double, _DP, _DP, C.c_int,
            C.c_int64, _DP, _DP, C.c_int64, C.c_int, C.POINTER(Stats)]
        _lib.orc_rk_fixed_steps.argtypes = [
            C.POINTER(Tableau), C.POINTER(Ode), _DP, C.c_double, C.c_int64, _DP, _DP, C.c_int, _DP]
        _lib.orc_ode_rhs.argtypes = [C.POINTER(Ode), _DP, _DP, C.c_int]
        _lib.orc_ode_rhs_repeat.argtypes = [C.POINTER(Ode), _DP, _DP, C.c_int, C.c_int64]
        _lib.orc_nbody_acc_rows.argtypes = [C.POINTER(NBody), _DP, C.POINTER(C.c_int64),
                                            C.c_int64, _DP]
        _lib.orc_nbody_energy.argtypes = [C.POINTER(NBody), _DP, _DP]
        _lib.orc_leapfrog.argtypes = [C.POINTER(NBody), _DP, C.c_double, C.c_double, C.c_double,
                                      C.POINTER(C.c_int64)]
        _lib.orc_spinning_cube.argtypes = [C.c_int64, C.c_double, C.c_uint32, _DP]
        _lib.orc_tableau_builtin.argtypes = [C.c_int, C.POINTER(Tableau)]
        _lib.orc_dopri5_dense_eval.argtypes = [_DP, _DP, _DP, C.c_int64, C.c_double,
                                               C.c_double, _DP, C.c_int64, _DP]
        _lib.orc_ic_plummer.argtypes = [C.c_int64, C.c_uint64, C.c_double, _DP]
        _lib.orc_pi_sequence.argtypes = [C.c_double] * 5 + [_DP, C.c_int64, C.c_double, _DP]
        _lib.orc_session_set_controller.argtypes = [C.c_void_p, C.c_int, C.c_double]
        _lib.orc_session_set_dense.argtypes = [C.c_void_p, _DP, C.c_int64, _DP]
        _lib.orc_session_dense_count.argtypes = [C.c_void_p]
        _lib.orc_session_dense_count.restype = C.c_int64
        for name in ("orc_sizeof_tableau", "orc_sizeof_ode", "orc_sizeof_stats"):
            getattr(_lib, name).restype = C.c_size_t
        assert _lib.orc_sizeof_tableau() == C.sizeof(Tableau)
        assert _lib.orc_sizeof_ode() == C.sizeof(Ode)
        assert _lib.orc_sizeof_stats() == C.sizeof(Stats)
    return _lib


def ref_available() -> bool:
    return os.path.exists(REF_SO)


def ref() -> C.CDLL:
    global _ref
    if _ref is None:
        _ref = C.CDLL(REF_SO)
        _ref.ref_integrate_nbody.argtypes = [
            C.c_int, C.c_int64, C.c_double, C.c_double, C.c_int, _DP, C.c_double, C.c_double,
            _DP, _DP, _DP, _DP, C.c_int64, C.POINTER(C.c_int64)]
        _ref.ref_integrate_small.argtypes = [
            C.c_int, C.c_int, C.c_int, _DP, C.c_double, C.c_double, _DP, _DP, _DP, _DP,
            C.c_int64, C.POINTER(C.c_int64)]
        _ref.ref_nbody_rhs.argtypes = [C.c_int64, C.c_double, C.c_double, C.c_int, _DP, _DP,
                                       C.c_int64]
        _ref.ref_nbody_sizes.argtypes = [C.POINTER(C.c_int64), C.c_int]
        _ref.ref_nr_dopr5_dense.argtypes = [C.c_int64, _DP, _DP, _DP, C.c_double, C.c_double,
                                            _DP, C.c_int64, _DP]
        _ref.ref_nr_dopr5_controller.argtypes = [_DP, C.c_int64, C.c_double, _DP]
    return _ref


def ref_dopri5_dense(y0, y1, ks, h: float, t_new: float, ts) -> np.ndarray:
    """The reference's own DOPRI5 dense output (Numerical Recipes'
    prepare_dense / dense_out, compiled in place)."""
    y0, y1, ks, ts = (np.ascontiguousarray(a, dtype=np.float64) for a in (y0, y1, ks, ts))
    n = len(y0)
    out = np.zeros((len(ts), n))
    assert ref().ref_nr_dopr5_dense(n, _ptr(y0), _ptr(y1), _ptr(ks), h, t_new, _ptr(ts),
                                    len(ts), _ptr(out)) == 0
    return out


def ref_dopri5_controller(errs, h0: float) -> np.ndarray:
    """The reference's Controller::success (Numerical Recipes' DOPRI5
    stepper, compiled in place) on a sequence of error norms."""
    errs = np.ascontiguousarray(errs, dtype=np.float64)
    hs = np.zeros(len(errs))
    assert ref().ref_nr_dopr5_controller(_ptr(errs), len(errs), h0, _ptr(hs)) == 0
    return hs


def dopri5_dense(y0, y1, ks, h: float, t_new: float, ts) -> np.ndarray:
    """The restated DOPRI5 dense output (gbode_oracle.c orc_dopri5_dense)."""
    y0, y1, ks, ts = (np.ascontiguousarray(a, dtype=np.float64) for a in (y0, y1, ks, ts))
    n = len(y0)
    out = np.zeros((len(ts), n))
    assert lib().orc_dopri5_dense_eval(_ptr(y0), _ptr(y1), _ptr(ks), n, h, t_new, _ptr(ts),
                                       len(ts), _ptr(out)) == 0
    return out


def ic_plummer(n: int, seed: int, a: float = 1.0) -> np.ndarray:
    """Seeded Plummer sphere, the same bits as the library's gb_ic_plummer
    (for the CPU-baseline legs, which must not load the GPU library)."""
    x = np.zeros(6 * n)
    assert lib().orc_ic_plummer(n, seed, a, _ptr(x)) == 0
    return x


def pi_sequence(safe: float, alpha: float, beta: float, minscale: float, maxscale: float,
                errs, h0: float) -> np.ndarray:
    """The restated PI controller (gbode_oracle.c orc_pi_scale) with explicit
    constants on a sequence of error norms: the step after each decision."""
    errs = np.ascontiguousarray(errs, dtype=np.float64)
    hs = np.zeros(len(errs))
    assert lib().orc_pi_sequence(safe, alpha, beta, minscale, maxscale, _ptr(errs), len(errs),
                                 h0, _ptr(hs)) == 0
    return hs


def ref_sizes() -> list[int]:
    buf = (C.c_int64 * 64)()
    n = ref().ref_nbody_sizes(buf, 64)
    return [int(buf[i]) for i in range(min(n, 64))]


def _ptr(a: np.ndarray | None):
    if a is None:
        return None
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(_DP)


def tableau(name: str) -> Tableau:
    t = Tableau()
    rc = lib().orc_tableau_builtin(TABLEAUS[name], C.byref(t))
    assert rc == 0
    return t


def nbody_ode(n_particles: int, softening: float, mass: float = 1.0,
              masses: np.ndarray | None = None) -> tuple[Ode, object]:
    keep = None
    o = Ode()
    o.kind = ODE_NBODY
    o.n_var = 6 * n_particles
    o.nb.n_particles = n_particles
    o.nb.softening = softening
    o.nb.mass = mass
    if masses is not None:
        keep = np.ascontiguousarray(masses, dtype=np.float64)
        o.nb.masses = _ptr(keep)
    return o, keep


def small_ode(kind: int, n_var: int) -> Ode:
    o = Ode()
    o.kind = kind
    o.n_var = n_var
    return o


@dataclass
class Result:
    times: np.ndarray
    states: np.ndarray
    stats: dict


def integrate(tab: str, ode: Ode, x0: np.ndarray, t0: float, tf: float, atol, rtol,
              n_threads: int = 1, capacity: int = 4096, keep_all: bool = True,
              max_attempts: int = 0) -> Result:
    """RKEmbeddedParallel<tab>::integrate restated (one thread = the
    single-threaded executor, several = the thread pool)."""
    n_var = int(ode.n_var)
    x0 = np.ascontiguousarray(x0, dtype=np.float64)
    atol = np.ascontiguousarray(np.broadcast_to(atol, (n_var,)), dtype=np.float64)
    rtol = np.ascontiguousarray(np.broadcast_to(rtol, (n_var,)), dtype=np.float64)
    cap = capacity if keep_all else 1
    times = np.zeros(cap)
    states = np.zeros((cap, n_var))
    st = Stats()
    t = tableau(tab)
    rc = lib().orc_rk_integrate(C.byref(t), C.byref(ode), _ptr(x0), t0, tf, _ptr(atol),
                                _ptr(rtol), n_threads, max_attempts, _ptr(times), _ptr(states),
                                cap, 1 if keep_all else 0, C.byref(st))
    assert rc == 0, rc
    if st.status == 1:
        return integrate(tab, ode, x0, t0, tf, atol, rtol, n_threads,
                         capacity=int(st.n_saved) + 16, keep_all=keep_all,
                         max_attempts=max_attempts)
    n = int(st.n_saved) if keep_all else 1
    stats = {f: getattr(st, f) for f, _ in Stats._fields_}
    return Result(times[:n].copy(), states[:n].copy(), stats)


def fixed_steps(tab: str, ode: Ode, x0: np.ndarray, dt: float, n_steps: int,
                atol=None, rtol=None, n_threads: int = 1):
    n_var = int(ode.n_var)
    x = np.ascontiguousarray(x0, dtype=np.float64).copy()
    en = np.zeros(max(n_steps, 1))
    a = r = None
    if atol is not None:
        a = np.ascontiguousarray(np.broadcast_to(atol, (n_var,)), dtype=np.float64)
        r = np.ascontiguousarray(np.broadcast_to(rtol, (n_var,)), dtype=np.float64)
    t = tableau(tab)
    rc = lib().orc_rk_fixed_steps(C.byref(t), C.byref(ode), _ptr(x), dt, n_steps, _ptr(a),
                                  _ptr(r), n_threads, _ptr(en))
    assert rc == 0
    return x, en[:n_steps]


def rhs(ode: Ode, x: np.ndarray, n_threads: int = 1) -> np.ndarray:
    x = np.ascontiguousarray(x, dtype=np.float64)
    out = np.zeros_like(x)
    assert lib().orc_ode_rhs(C.byref(ode), _ptr(x), _ptr(out), n_threads) == 0
    return out


def rhs_repeat(ode: Ode, x: np.ndarray, n_threads: int, reps: int) -> np.ndarray:
    x = np.ascontiguousarray(x, dtype=np.float64)
    out = np.zeros_like(x)
    assert lib().orc_ode_rhs_repeat(C.byref(ode), _ptr(x), _ptr(out), n_threads, reps) == 0
    return out


def acc_rows(ode: Ode, x: np.ndarray, rows: np.ndarray) -> np.ndarray:
    x = np.ascontiguousarray(x, dtype=np.float64)
    rows = np.ascontiguousarray(rows, dtype=np.int64)
    out = np.zeros((len(rows), 3))
    rc = lib().orc_nbody_acc_rows(C.byref(ode.nb), _ptr(x), rows.ctypes.data_as(C.POINTER(C.c_int64)),
                                  len(rows), _ptr(out))
    assert rc == 0
    return out


def energy(ode: Ode, x: np.ndarray) -> dict:
    x = np.ascontiguousarray(x, dtype=np.float64)
    out = np.zeros(8)
    assert lib().orc_nbody_energy(C.byref(ode.nb), _ptr(x), _ptr(out)) == 0
    return {"ke": out[0], "pe": out[1], "e": out[0] + out[1], "p": out[2:5].copy(),
            "l": out[5:8].copy()}


def leapfrog(ode: Ode, x0: np.ndarray, t0: float, tf: float, dt: float):
    x = np.ascontiguousarray(x0, dtype=np.float64).copy()
    n = C.c_int64(0)
    assert lib().orc_leapfrog(C.byref(ode.nb), _ptr(x), t0, tf, dt, C.byref(n)) == 0
    return x, int(n.value)


def spinning_cube(n: int, L: float = 1.0, seed: int = 0) -> np.ndarray:
    x = np.zeros(6 * n)
    assert lib().orc_spinning_cube(n, L, seed, _ptr(x)) == 0
    return x


# --- the reference itself (oracle/_ref), where it was compiled -------------
def ref_integrate_nbody(tab: str, n_particles: int, softening: float, mass: float,
                        x0: np.ndarray, t0: float, tf: float, atol, rtol, n_threads: int = 1,
                        capacity: int = 4096) -> Result:
    n_var = 6 * n_particles
    x0 = np.ascontiguousarray(x0, dtype=np.float64)
    atol = np.ascontiguousarray(np.broadcast_to(atol, (n_var,)), dtype=np.float64)
    rtol = np.ascontiguousarray(np.broadcast_to(rtol, (n_var,)), dtype=np.float64)
    times = np.zeros(capacity)
    states = np.zeros((capacity, n_var))
    n_saved = C.c_int64(0)
    rc = ref().ref_integrate_nbody(TABLEAUS[tab], n_particles, softening, mass, n_threads,
                                   _ptr(x0), t0, tf, _ptr(atol), _ptr(rtol), _ptr(times),
                                   _ptr(states), capacity, C.byref(n_saved))
    if rc == 1:
        return ref_integrate_nbody(tab, n_particles, softening, mass, x0, t0, tf, atol, rtol,
                                   n_threads, int(n_saved.value) + 16)
    assert rc == 0, f"size {n_particles} not instantiated in libref.so"
    n = int(n_saved.value)
    return Result(times[:n].copy(), states[:n].copy(), {"n_saved": n})


def ref_integrate_small(tab: str, kind: int, x0, t0, tf, atol, rtol, n_threads: int = 1,
                        capacity: int = 1 << 18) -> Result:
    x0 = np.ascontiguousarray(x0, dtype=np.float64)
    n_var = len(x0)
    atol = np.ascontiguousarray(np.broadcast_to(atol, (n_var,)), dtype=np.float64)
    rtol = np.ascontiguousarray(np.broadcast_to(rtol, (n_var,)), dtype=np.float64)
    times = np.zeros(capacity)
    states = np.zeros((capacity, n_var))
    n_saved = C.c_int64(0)
    rc = ref().ref_integrate_small(TABLEAUS[tab], kind, n_threads, _ptr(x0), t0, tf, _ptr(atol),
                                   _ptr(rtol), _ptr(times), _ptr(states), capacity,
                                   C.byref(n_saved))
    assert rc == 0, rc
    n = int(n_saved.value)
    return Result(times[:n].copy(), states[:n].copy(), {"n_saved": n})


def ref_rhs(n_particles: int, softening: float, mass: float, x: np.ndarray, n_threads: int = 1,
            reps: int = 1) -> np.ndarray:
    x = np.ascontiguousarray(x, dtype=np.float64)
    out = np.zeros_like(x)
    rc = ref().ref_nbody_rhs(n_particles, softening, mass, n_threads, _ptr(x), _ptr(out), reps)
    assert rc == 0, f"size {n_particles} not instantiated in libref.so"
    return out


class Session:
    """Resumable reference loop (orc_session_*): attempts one at a time, for
    timing the reference's CPU implementation on bounded samples."""

    def __init__(self, tab: str, ode: Ode, x0, t0: float, tf: float, atol, rtol,
                 n_threads: int = 1, controller: str = "reference", pi_beta: float = 0.04,
                 dense_times=None):
        L = lib()
        if not getattr(L, "_session_bound", False):
            L.orc_session_create.restype = C.c_void_p
            L.orc_session_create.argtypes = [C.POINTER(Tableau), C.POINTER(Ode), _DP, C.c_double,
                                             C.c_double, _DP, _DP, C.c_int]
            L.orc_session_attempt.argtypes = [C.c_void_p, C.POINTER(C.c_int)]
            L.orc_session_attempt.restype = C.c_int
            L.orc_session_stats.argtypes = [C.c_void_p, C.POINTER(Stats)]
            L.orc_session_state.argtypes = [C.c_void_p, C.POINTER(C.c_double)]
            L.orc_session_state.restype = _DP
            L.orc_session_destroy.argtypes = [C.c_void_p]
            L._session_bound = True
        n_var = int(ode.n_var)
        self._ode = ode
        self._tab = tableau(tab)
        x0 = np.ascontiguousarray(x0, dtype=np.float64)
        self._a = np.ascontiguousarray(np.broadcast_to(atol, (n_var,)), dtype=np.float64)
        self._r = np.ascontiguousarray(np.broadcast_to(rtol, (n_var,)), dtype=np.float64)
        self.h = L.orc_session_create(C.byref(self._tab), C.byref(ode), _ptr(x0), t0, tf,
                                      _ptr(self._a), _ptr(self._r), n_threads)
        assert self.h
        self.n_var = n_var
        if controller == "pi":
            assert L.orc_session_set_controller(self.h, 1, pi_beta) == 0
        else:
            assert controller == "reference", controller
        self._dense_t = None
        if dense_times is not None:
            self._dense_t = np.ascontiguousarray(dense_times, dtype=np.float64)
            self._dense = np.zeros((len(self._dense_t), n_var))
            assert L.orc_session_set_dense(self.h, _ptr(self._dense_t), len(self._dense_t),
                                           _ptr(self._dense)) == 0

    def attempt(self) -> tuple[bool, bool]:
        acc = C.c_int(0)
        done = lib().orc_session_attempt(self.h, C.byref(acc))
        return bool(done), bool(acc.value)

    def stats(self) -> dict:
        st = Stats()
        lib().orc_session_stats(self.h, C.byref(st))
        return {f: getattr(st, f) for f, _ in Stats._fields_}

    def dense(self) -> np.ndarray:
        """Dense outputs produced so far (DOPRI5 sessions with dense_times)."""
        if self._dense_t is None:
            return np.zeros((0, self.n_var))
        return self._dense[: int(lib().orc_session_dense_count(self.h))].copy()

    def run(self):
        """Attempts until t reaches tf: (times, states) of t0 and every
        accepted step, as the reference's RawOutput records them."""
        x, t = self.state()
        times, states = [t], [x]
        while True:
            done, acc = self.attempt()
            if done:
                break
            if acc:
                x, t = self.state()
                times.append(t)
                states.append(x)
        return np.array(times), np.array(states)

    def state(self):
        t = C.c_double(0)
        p = lib().orc_session_state(self.h, C.byref(t))
        return np.ctypeslib.as_array(p, shape=(self.n_var,)).copy(), t.value

    def close(self):
        if self.h:
            lib().orc_session_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
