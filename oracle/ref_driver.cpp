// ref_driver.cpp -- C entry points around the reference implementation,
// compiled in place from the reference's own headers (oracle/Makefile, target
// `ref`) into oracle/_ref/libref.so.  TEST INFRASTRUCTURE ONLY: it exists to
// validate the C restatement (gbode_oracle.c), to generate the golden fixtures
// under tests/golden/, and as the "reference" CPU baseline where it was built.
//
// The reference's state size is a template parameter, so each supported
// system size is instantiated explicitly (kNBodySizes below).  Masses 1/N are
// applied by a wrapper ODE that scales the acceleration half after the
// reference's unit-mass NBodyODE (NBodyODE.hpp:31-39 has no masses).
#include <cstdint>
#include <cstring>
#include <span>
#include <utility>

#include "BTDOPRI5.hpp"
#include "BTDVERK.hpp"
#include "BTHE21.hpp"
#include "BTRKF45.hpp"
#include "BTRKF78.hpp"
#include "ExponentialODE.hpp"
#include "HeapState.hpp"
#include "NBodyODE.hpp"
#include "ParallelExecutor.hpp"
#include "RKEmbeddedParallel.hpp"
#include "RawOutput.hpp"
#include "StepperDopr5.hpp"
#include "SingleThreadedExecutor.hpp"
#include "ThreadPoolExecutor.hpp"
#include "VanDerPolODE.hpp"

namespace {

template <std::size_t n_var>
struct MassScaledNBody {
  NBodyODE<double, n_var> ode;
  double mass;
  static constexpr void scale_kernel(std::size_t i, double* acc, double m) { acc[i] *= m; }
  void operator()(auto& exe, std::span<double const, n_var> x,
                  std::span<double, n_var> dxdt) const {
    ode(exe, x, dxdt);
    if (mass != 1.0) {
      call_parallel_kernel<scale_kernel>(exe, n_var / 2, dxdt.data() + n_var / 2, mass);
    }
  }
};

template <std::size_t n_var>
struct ExpoWrap {
  void operator()(auto& exe, std::span<double const, n_var> x, std::span<double, n_var> dxdt) {
    ExponentialODE<double, n_var>{}(exe, x, dxdt);
  }
};

struct VdpWrap {
  void operator()(auto& exe, std::span<double const, 2> x, std::span<double, 2> dxdt) {
    VanDerPolODE<double>{}(exe, x, dxdt);
  }
};

struct Sink {
  double* times;
  double* states;
  std::int64_t capacity;
  std::int64_t n_saved;
};

template <typename BT, std::size_t n_var, typename ODE, typename Exe>
int run(ODE ode, Exe& exe, double const* x0p, double t0, double tf, double const* atolp,
        double const* rtolp, Sink& sink) {
  using State = HeapState<double, n_var>;
  auto x0 = State{std::span<double const, n_var>{x0p, n_var}};
  auto atol = State{std::span<double const, n_var>{atolp, n_var}};
  auto rtol = State{std::span<double const, n_var>{rtolp, n_var}};
  auto output = RawOutput<State>{};
  RKEmbeddedParallel<BT>::integrate(x0, t0, tf, atol, rtol, ode, output, exe);
  auto const& times = output.times();
  auto const& states = output.states();
  sink.n_saved = static_cast<std::int64_t>(times.size());
  auto k_max = std::min<std::int64_t>(sink.n_saved, sink.capacity);
  for (std::int64_t k = 0; k < k_max; ++k) {
    if (sink.times) sink.times[k] = times[k];
    if (sink.states) std::memcpy(sink.states + k * n_var, states[k].data(), n_var * sizeof(double));
  }
  return sink.n_saved > sink.capacity ? 1 : 0;
}

template <typename BT, std::size_t n_var, typename ODE>
int run_exe(ODE ode, int n_threads, double const* x0, double t0, double tf, double const* atol,
            double const* rtol, Sink& sink) {
  if (n_threads <= 1) {
    auto exe = SingleThreadedExecutor{};
    return run<BT, n_var>(ode, exe, x0, t0, tf, atol, rtol, sink);
  }
  auto exe = ThreadPoolExecutor{n_threads};
  return run<BT, n_var>(ode, exe, x0, t0, tf, atol, rtol, sink);
}

template <std::size_t n_var, typename ODE>
int run_tableau(int tableau, ODE ode, int n_threads, double const* x0, double t0, double tf,
                double const* atol, double const* rtol, Sink& sink) {
  switch (tableau) {
    case 0: return run_exe<BTHE21, n_var>(ode, n_threads, x0, t0, tf, atol, rtol, sink);
    case 1: return run_exe<BTRKF45, n_var>(ode, n_threads, x0, t0, tf, atol, rtol, sink);
    case 2: return run_exe<BTDOPRI5, n_var>(ode, n_threads, x0, t0, tf, atol, rtol, sink);
    case 3: return run_exe<BTDVERK, n_var>(ode, n_threads, x0, t0, tf, atol, rtol, sink);
    case 4: return run_exe<BTRKF78, n_var>(ode, n_threads, x0, t0, tf, atol, rtol, sink);
    default: return -1;
  }
}

template <std::size_t N>
int nbody_integrate(int tableau, double softening, double mass, int n_threads, double const* x0,
                    double t0, double tf, double const* atol, double const* rtol, Sink& sink) {
  constexpr std::size_t n_var = 6 * N;
  auto ode = MassScaledNBody<n_var>{NBodyODE<double, n_var>{softening}, mass};
  return run_tableau<n_var>(tableau, ode, n_threads, x0, t0, tf, atol, rtol, sink);
}

template <std::size_t N>
int nbody_rhs(double softening, double mass, int n_threads, double const* x, double* dxdt,
              std::int64_t reps) {
  constexpr std::size_t n_var = 6 * N;
  auto ode = MassScaledNBody<n_var>{NBodyODE<double, n_var>{softening}, mass};
  auto xs = std::span<double const, n_var>{x, n_var};
  auto ds = std::span<double, n_var>{dxdt, n_var};
  if (n_threads <= 1) {
    auto exe = SingleThreadedExecutor{};
    for (std::int64_t r = 0; r < reps; ++r) ode(exe, xs, ds);
  } else {
    auto exe = ThreadPoolExecutor{n_threads};
    for (std::int64_t r = 0; r < reps; ++r) ode(exe, xs, ds);
  }
  return 0;
}

// Stand-ins for the derivative functor and output policy of the Numerical
// Recipes DOPRI5 stepper; only prepare_dense, dense_out and
// Controller::success are called, which use neither.
struct NoDerivs {
  void operator()(double, std::vector<double>&, std::vector<double>&) {}
};
struct NoSave {};
using NrDopr5 = StepperDopr5<NoDerivs, NoSave>;

#define GB_REF_SIZES(X) X(5) X(16) X(64) X(128) X(256) X(1024) X(4096) X(16384)

}  // namespace

extern "C" {

// Number of bodies this build was instantiated for; sizes[k] for k < count.
int ref_nbody_sizes(std::int64_t* sizes, int capacity) {
  int k = 0;
#define GB_LIST(n) \
  if (k < capacity) sizes[k] = n; \
  ++k;
  GB_REF_SIZES(GB_LIST)
#undef GB_LIST
  return k;
}

// RKEmbeddedParallel<BT>::integrate on the N-body problem (tableau ids: 0 HE21,
// 1 RKF45, 2 DOPRI5, 3 DVERK, 4 RKF78).  Returns 0, 1 when more states were
// saved than `capacity` (n_saved still holds the count), -1 for an unsupported
// size or tableau.
int ref_integrate_nbody(int tableau, std::int64_t n_particles, double softening, double mass,
                        int n_threads, double const* x0, double t0, double tf,
                        double const* atol, double const* rtol, double* times, double* states,
                        std::int64_t capacity, std::int64_t* n_saved) {
  Sink sink{times, states, capacity, 0};
  int rc = -1;
  switch (n_particles) {
#define GB_CASE(n)                                                                         \
  case n:                                                                                  \
    rc = nbody_integrate<n>(tableau, softening, mass, n_threads, x0, t0, tf, atol, rtol, \
                            sink);                                                         \
    break;
    GB_REF_SIZES(GB_CASE)
#undef GB_CASE
    default: return -1;
  }
  if (n_saved) *n_saved = sink.n_saved;
  return rc;
}

// ode_kind 1: ExponentialODE<double, 10>; ode_kind 2: VanDerPolODE (n_var 2).
int ref_integrate_small(int tableau, int ode_kind, int n_threads, double const* x0, double t0,
                        double tf, double const* atol, double const* rtol, double* times,
                        double* states, std::int64_t capacity, std::int64_t* n_saved) {
  Sink sink{times, states, capacity, 0};
  int rc = -1;
  if (ode_kind == 1) {
    rc = run_tableau<10>(tableau, ExpoWrap<10>{}, n_threads, x0, t0, tf, atol, rtol, sink);
  } else if (ode_kind == 2) {
    rc = run_tableau<2>(tableau, VdpWrap{}, n_threads, x0, t0, tf, atol, rtol, sink);
  }
  if (n_saved) *n_saved = sink.n_saved;
  return rc;
}

// `reps` evaluations of the (mass-scaled) NBodyODE right-hand side.
int ref_nbody_rhs(std::int64_t n_particles, double softening, double mass, int n_threads,
                  double const* x, double* dxdt, std::int64_t reps) {
  switch (n_particles) {
#define GB_CASE(n) \
  case n: return nbody_rhs<n>(softening, mass, n_threads, x, dxdt, reps);
    GB_REF_SIZES(GB_CASE)
#undef GB_CASE
    default: return -1;
  }
}

// The reference's DOPRI5 dense output (NumericalRecipes/StepperDopr5.hpp:
// 179-219): prepare_dense from y0 (at t_new - h), y1 (at t_new) and the seven
// stage derivatives ks[j * n + i], then dense_out at each time ts[k] into
// out[k * n + i].
int ref_nr_dopr5_dense(std::int64_t n, double const* y0, double const* y1, double const* ks,
                       double h, double t_new, double const* ts, std::int64_t nt, double* out) {
  std::vector<double> y(y0, y0 + n), dydx(ks, ks + n);
  double x = t_new;
  NoDerivs d;
  NrDopr5 st(y, dydx, x, 0.0, 0.0, d);
  st.yout.assign(y1, y1 + n);
  st.k3.assign(ks + 2 * n, ks + 3 * n);
  st.k4.assign(ks + 3 * n, ks + 4 * n);
  st.k5.assign(ks + 4 * n, ks + 5 * n);
  st.k6.assign(ks + 5 * n, ks + 6 * n);
  st.dydxnew.assign(ks + 6 * n, ks + 7 * n);
  Dopr5DenseData dd;
  st.prepare_dense(h, dd);
  for (std::int64_t k = 0; k < nt; ++k)
    for (std::int64_t i = 0; i < n; ++i) out[k * n + i] = st.dense_out((int)i, ts[k], h, dd);
  return 0;
}

// The reference's step-size controller (Controller::success,
// NumericalRecipes/StepperDopr5.hpp:236-272) on a sequence of error norms,
// as StepperDopr5::step drives it: after a success the next step is hnext,
// after a rejection the reduced h.  hs[k] = the step after decision k.
int ref_nr_dopr5_controller(double const* errs, std::int64_t m, double h0, double* hs) {
  NrDopr5::Controller con;
  double h = h0;
  for (std::int64_t k = 0; k < m; ++k) {
    if (con.success(errs[k], h)) h = con.hnext;
    hs[k] = h;
  }
  return 0;
}

}  // extern "C"
