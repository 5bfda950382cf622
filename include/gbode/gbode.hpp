// gbode.hpp -- C++20 drop-in types for the GB300 path, built only on the C ABI
// (gbode.h); no CUDA header is needed unless generic kernels are launched.
//
// They mirror the reference's template interface (noether17/ode_prototyping):
//   Gb300State<T, N>      -- an ODEState (src/state/ODEState.hpp:25-43) owning
//                            device memory, like CudaState (src/state/CudaState.cuh:10-64)
//   Gb300Executor         -- an executor with call_parallel_kernel /
//                            transform_reduce (src/par_exec/ParallelExecutor.hpp:7-24)
//   RKEmbeddedGb300<BT>   -- same integrate() signature as RKEmbeddedParallel<BT>
//                            (src/integrator/RKEmbeddedParallel/RKEmbeddedParallel.hpp:15-19)
//   NBodyODE<T, n_var>    -- same shape as the reference's NBodyODE
//                            (src/ode/NBodyODE.hpp:9-46) plus optional masses
//   tableau::DOPRI5 ...   -- tags for the built-in tableaus
//
// RKEmbeddedGb300<BT>::integrate accepts the reference's own types too: any
// BT with static a, b, bt, p, pt, n_stages; any ODE with a `softening`
// member and 6N state variables is integrated by the device-resident N-body
// integrator; any other ODE runs the reference's loop on the device through
// Gb300Executor (that path launches the ODE's own kernels and needs nvcc).
#pragma once

#include <algorithm>
#include <array>
#include <cmath>
#include <concepts>
#include <cstddef>
#include <cstdint>
#include <cstring>
#include <span>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>

#include "../gbode.h"

#ifdef __CUDACC__
#include <cuda_runtime.h>
#endif

namespace gbode {

struct Error : std::runtime_error {
  int status;
  Error(int s, const char* where)
      : std::runtime_error(std::string(where) + ": " + gb_status_string(s)), status(s) {}
};

inline void check(int status, const char* where) {
  if (status != GB_OK) throw Error(status, where);
}

// ---------------------------------------------------------------------------
// Gb300State: fixed-size owning device vector (CudaState semantics: default
// construction zero-fills, copies are deep, moves swap storage).
// ---------------------------------------------------------------------------
template <std::floating_point T, std::size_t N>
class Gb300State {
 public:
  static constexpr auto size() { return N; }

  Gb300State() {
    alloc();
    check(gb_memset_zero(ptr_, N * sizeof(T)), "Gb300State()");
  }
  explicit Gb300State(std::span<T const, N> host) {
    alloc();
    check(gb_memcpy(ptr_, host.data(), N * sizeof(T), 0), "Gb300State(span)");
  }
  Gb300State(Gb300State const& o) {
    alloc();
    check(gb_memcpy(ptr_, o.ptr_, N * sizeof(T), 2), "Gb300State(copy)");
  }
  Gb300State(Gb300State&& o) noexcept : ptr_{o.ptr_} {
    o.ptr_ = nullptr;
    o.alloc_nothrow();
  }
  Gb300State& operator=(Gb300State const& o) {
    if (this != &o) check(gb_memcpy(ptr_, o.ptr_, N * sizeof(T), 2), "Gb300State=");
    return *this;
  }
  Gb300State& operator=(Gb300State&& o) noexcept {
    std::swap(ptr_, o.ptr_);
    return *this;
  }
  ~Gb300State() { gb_device_free(ptr_); }

  auto* data() { return ptr_; }
  auto const* data() const { return ptr_; }

  void copy_to_span(std::span<T, N> dest) const {
    check(gb_memcpy(dest.data(), ptr_, N * sizeof(T), 1), "Gb300State::copy_to_span");
  }
  friend auto span(Gb300State& s) { return std::span<T, N>{s.data(), N}; }
  friend auto span(Gb300State const& s) { return std::span<T const, N>{s.data(), N}; }

 private:
  void alloc() {
    void* p = nullptr;
    check(gb_device_alloc(&p, N * sizeof(T)), "Gb300State alloc");
    ptr_ = static_cast<T*>(p);
  }
  void alloc_nothrow() noexcept {
    void* p = nullptr;
    if (gb_device_alloc(&p, N * sizeof(T)) == GB_OK) ptr_ = static_cast<T*>(p);
  }
  T* ptr_ = nullptr;
};

// Non-owning view of a host buffer, an ODEState handed to Output::save_state.
template <std::floating_point T, std::size_t N>
class HostStateView {
 public:
  static constexpr auto size() { return N; }
  HostStateView() = default;
  explicit HostStateView(T* p) : p_{p} {}
  auto* data() { return p_; }
  auto const* data() const { return p_; }
  void copy_to_span(std::span<T, N> dest) const { std::memcpy(dest.data(), p_, N * sizeof(T)); }
  friend auto span(HostStateView& s) { return std::span<T, N>{s.p_, N}; }
  friend auto span(HostStateView const& s) { return std::span<T const, N>{s.p_, N}; }

 private:
  T* p_ = nullptr;
};

// Device view of a ring slot: an ODEState whose copy_to_span reads the device.
template <std::floating_point T, std::size_t N>
class DeviceStateView {
 public:
  static constexpr auto size() { return N; }
  DeviceStateView() = default;
  explicit DeviceStateView(T* p) : p_{p} {}
  auto* data() { return p_; }
  auto const* data() const { return p_; }
  void copy_to_span(std::span<T, N> dest) const {
    check(gb_memcpy(dest.data(), p_, N * sizeof(T), 1), "DeviceStateView::copy_to_span");
  }
  friend auto span(DeviceStateView& s) { return std::span<T, N>{s.p_, N}; }
  friend auto span(DeviceStateView const& s) { return std::span<T const, N>{s.p_, N}; }

 private:
  T* p_ = nullptr;
};

// ---------------------------------------------------------------------------
// Tableau tags and conversion of any reference-style tableau to gb_tableau.
// ---------------------------------------------------------------------------
namespace tableau {
struct HE21 { static constexpr int32_t id = GB_HE21; };
struct RKF45 { static constexpr int32_t id = GB_RKF45; };
struct DOPRI5 { static constexpr int32_t id = GB_DOPRI5; };
struct DVERK { static constexpr int32_t id = GB_DVERK; };
struct RKF78 { static constexpr int32_t id = GB_RKF78; };
}  // namespace tableau

template <typename BT>
gb_tableau to_gb_tableau() {
  gb_tableau t;
  std::memset(&t, 0, sizeof t);
  if constexpr (requires { BT::id; }) {
    check(gb_tableau_builtin(BT::id, &t), "gb_tableau_builtin");
  } else {
    // the reference's butcher_tableaus/BT*.hpp layout
    static_assert(BT::n_stages <= GB_MAX_STAGES, "too many stages");
    t.n_stages = BT::n_stages;
    t.p = BT::p;
    t.pt = BT::pt;
    for (std::size_t r = 0; r < BT::a.size(); ++r)
      for (std::size_t c = 0; c < BT::a[r].size(); ++c) t.a[r][c] = BT::a[r][c];
    for (int j = 0; j < BT::n_stages; ++j) {
      t.b[j] = BT::b[j];
      t.bt[j] = BT::bt[j];
    }
  }
  return t;
}

// ---------------------------------------------------------------------------
// NBodyODE: the reference's shape (softening member, n_var = 6N) with an
// optional uniform mass (applied after the pair sum) or per-body masses.
// ---------------------------------------------------------------------------
struct Gb300Executor;

template <typename ValueType, std::size_t n_var>
struct NBodyODE {
  static_assert(n_var % 6 == 0, "N-body state is [positions 3N | velocities 3N]");
  static constexpr auto n_dof = n_var / 2;
  static constexpr auto n_particles = n_var / 6;
  double softening{};
  double mass = 1.0;
  double const* masses_dev = nullptr;

  void operator()(Gb300Executor& exe, std::span<ValueType const, n_var> x,
                  std::span<ValueType, n_var> dxdt) const;
  void acc(Gb300Executor& exe, std::span<ValueType const, n_var> x,
           std::span<ValueType, n_dof> acc) const;
};

template <typename ODE>
concept NBodyLike = requires(ODE const& o) {
  { o.softening } -> std::convertible_to<double>;
  { ODE::n_particles } -> std::convertible_to<std::size_t>;
};

template <typename ODE>
double ode_mass(ODE const& o) {
  if constexpr (requires { o.mass; }) return o.mass;
  return 1.0;  // the reference's NBodyODE has unit masses
}
template <typename ODE>
double const* ode_masses(ODE const& o) {
  if constexpr (requires { o.masses_dev; }) return o.masses_dev;
  return nullptr;
}

// ---------------------------------------------------------------------------
// Gb300Executor
// ---------------------------------------------------------------------------
#ifdef __CUDACC__
namespace detail {
template <auto kernel, typename... Args>
__global__ void parallel_kernel_launcher(std::size_t n, Args... args) {
  for (std::size_t i = blockIdx.x * (std::size_t)blockDim.x + threadIdx.x; i < n;
       i += (std::size_t)gridDim.x * blockDim.x)
    kernel(i, args...);
}
template <typename T, auto reduce, auto transform, typename... Args>
__global__ void transform_partial(T* out, std::size_t n, Args... args) {
  __shared__ T sh[256];
  T acc{};
  for (std::size_t i = blockIdx.x * (std::size_t)blockDim.x + threadIdx.x; i < n;
       i += (std::size_t)gridDim.x * blockDim.x)
    acc = reduce(acc, transform(i, args...));
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s /= 2) {
    if ((int)threadIdx.x < s) sh[threadIdx.x] = reduce(sh[threadIdx.x], sh[threadIdx.x + s]);
    __syncthreads();
  }
  if (threadIdx.x == 0) out[blockIdx.x] = sh[0];
}
}  // namespace detail
#endif

struct Gb300Executor {
  gb_stream_t stream = nullptr;
  int32_t precision = GB_PREC_F64;
  int32_t controller = GB_CTRL_REFERENCE;
  bool exact = false;
  bool fsal = true;
  int32_t attempts_per_sync = 16;
  int64_t max_attempts = 0;
  gb_force_tiling tiling{};
  const gb_mlp* mlp = nullptr;

  // Element-wise kernel over n items: kernel(i, args...) for i < n.  The
  // reference's executors run this on the host or with a CUDA grid-stride
  // launch; here it is a grid-stride launch of the caller's constexpr
  // kernel (needs nvcc).
  template <auto kernel, typename... Args>
  void call_parallel_kernel(std::size_t n_items, Args... args) {
#ifdef __CUDACC__
    if (n_items == 0) return;
    const unsigned blocks = (unsigned)std::min<std::size_t>((n_items + 255) / 256, 152 * 32);
    detail::parallel_kernel_launcher<kernel, Args...>
        <<<blocks, 256, 0, reinterpret_cast<cudaStream_t>(stream)>>>(n_items, args...);
    check(cudaGetLastError() == cudaSuccess ? GB_OK : GB_ERR_CUDA, "call_parallel_kernel");
#else
    static_assert(sizeof...(Args) < 0,
                  "generic kernels need nvcc; N-body ODEs go through RKEmbeddedGb300 directly");
#endif
  }

  // reduce(init, reduce over i of transform(i, args...)) with a deterministic
  // two-level tree; returns the host value (synchronises).
  template <typename T, auto reduce, auto transform, typename... Args>
  T transform_reduce(T init, std::size_t n_items, Args... args) {
#ifdef __CUDACC__
    const unsigned blocks = (unsigned)std::max<std::size_t>(
        1, std::min<std::size_t>((n_items + 1023) / 1024, 1024));
    T* part = nullptr;
    check(gb_device_alloc((void**)&part, blocks * sizeof(T)), "transform_reduce");
    auto s = reinterpret_cast<cudaStream_t>(stream);
    detail::transform_partial<T, reduce, transform, Args...><<<blocks, 256, 0, s>>>(part, n_items,
                                                                                    args...);
    std::vector<T> host(blocks);
    cudaMemcpyAsync(host.data(), part, blocks * sizeof(T), cudaMemcpyDeviceToHost, s);
    cudaStreamSynchronize(s);
    gb_device_free(part);
    T r = init;
    for (auto const& v : host) r = reduce(r, v);
    return r;
#else
    static_assert(sizeof...(Args) < 0, "generic reductions need nvcc");
    return init;
#endif
  }

  gb_integrate_opts opts(bool record) const {
    gb_integrate_opts o;
    std::memset(&o, 0, sizeof o);
    o.precision = precision;
    o.controller = controller;
    o.fsal = fsal ? 1 : 0;
    o.exact = exact ? 1 : 0;
    o.attempts_per_sync = attempts_per_sync;
    o.record = record ? 1 : 0;
    o.max_attempts = max_attempts;
    o.tiling = tiling;
    o.mlp = mlp;
    return o;
  }
};

template <typename ValueType, std::size_t n_var>
void NBodyODE<ValueType, n_var>::operator()(Gb300Executor& exe, std::span<ValueType const, n_var> x,
                                            std::span<ValueType, n_var> dxdt) const {
  static_assert(std::is_same_v<ValueType, double>, "FP64 state");
  if (exe.precision == GB_PREC_MIXED) {
    void* work = nullptr;
    const std::size_t wb = gb_nbody_mixed_workspace_bytes(n_particles);
    check(gb_device_alloc(&work, wb), "NBodyODE workspace");
    int rc = gb_nbody_rhs_mixed(x.data(), dxdt.data(), n_particles, softening, mass, masses_dev,
                                work, &exe.tiling, exe.stream);
    gb_stream_synchronize(exe.stream);
    gb_device_free(work);
    check(rc, "gb_nbody_rhs_mixed");
  } else {
    check(gb_nbody_rhs_f64(x.data(), dxdt.data(), n_particles, softening, mass, masses_dev,
                           &exe.tiling, exe.stream),
          "gb_nbody_rhs_f64");
  }
}

template <typename ValueType, std::size_t n_var>
void NBodyODE<ValueType, n_var>::acc(Gb300Executor& exe, std::span<ValueType const, n_var> x,
                                     std::span<ValueType, n_dof> a) const {
  check(gb_nbody_acc_f64(x.data(), a.data(), n_particles, softening, mass, masses_dev, 0,
                         &exe.tiling, exe.stream),
        "gb_nbody_acc_f64");
}

// ---------------------------------------------------------------------------
// RKEmbeddedGb300<BT>
// ---------------------------------------------------------------------------
template <typename State>
struct state_info;
template <template <typename, std::size_t> typename M, typename T, std::size_t N>
struct state_info<M<T, N>> {
  using value_type = T;
  static constexpr std::size_t size = N;
};

// Whether a state object's storage is device memory: Gb300State always;
// other types (the reference's HeapState / CudaState) are told apart by
// asking the library where the pointer lives.
int32_t pointer_kind(const void* p);

template <typename ButcherTableau>
struct RKEmbeddedGb300 {
  template <typename ODE, typename Output, typename Executor, typename StateType>
  static void integrate(StateType x0, typename state_info<StateType>::value_type t0,
                        typename state_info<StateType>::value_type tf, StateType atol,
                        StateType rtol, ODE ode, Output& output, Executor& exe) {
    constexpr std::size_t n_var = state_info<StateType>::size;
    if constexpr (NBodyLike<ODE>) {
      integrate_nbody<n_var>(x0, t0, tf, atol, rtol, ode, output, exe);
    } else {
      integrate_generic<n_var>(x0, t0, tf, atol, rtol, ode, output, exe);
    }
  }

 private:
  // Device copies of a state argument (host or device storage).
  struct DevBuf {
    double* p = nullptr;
    explicit DevBuf(std::size_t n) { check(gb_device_alloc((void**)&p, n * sizeof(double)), "buf"); }
    ~DevBuf() { gb_device_free(p); }
  };
  template <std::size_t n_var, typename State>
  static void to_device(State const& s, double* dst) {
    const int32_t kind = gb_pointer_kind(s.data());
    check(gb_memcpy(dst, s.data(), n_var * sizeof(double), kind == 0 ? 0 : 2), "state copy");
  }

  template <typename Output, std::size_t n_var>
  struct SaveCtx {
    Output* out;
  };
  template <typename Output, std::size_t n_var>
  static void save_cb(void* user, double t, const double* x, int64_t) {
    auto* c = static_cast<SaveCtx<Output, n_var>*>(user);
    HostStateView<double, n_var> v{const_cast<double*>(x)};
    c->out->save_state(t, v);
  }

  template <std::size_t n_var, typename StateType, typename ODE, typename Output,
            typename Executor>
  static void integrate_nbody(StateType const& x0, double t0, double tf, StateType const& atol,
                              StateType const& rtol, ODE const& ode, Output& output,
                              Executor& exe) {
    static_assert(n_var % 6 == 0, "N-body state is [positions 3N | velocities 3N]");
    const gb_tableau tab = to_gb_tableau<ButcherTableau>();
    gb_nbody_system sys{(int64_t)(n_var / 6), (double)ode.softening, ode_mass(ode),
                        ode_masses(ode)};
    gb_integrate_opts opts;
    gb_stream_t stream = nullptr;
    if constexpr (std::is_same_v<Executor, Gb300Executor>) {
      opts = exe.opts(true);
      stream = exe.stream;
    } else {
      opts = Gb300Executor{}.opts(true);
    }
    DevBuf dx(n_var), da(n_var), dr(n_var);
    to_device<n_var>(x0, dx.p);
    to_device<n_var>(atol, da.p);
    to_device<n_var>(rtol, dr.p);
    gb_integrator it = nullptr;
    check(gb_integrator_create(&tab, &sys, &opts, stream, &it), "gb_integrator_create");
    SaveCtx<Output, n_var> ctx{&output};
    int rc = gb_integrator_start(it, dx.p, t0, tf, da.p, dr.p, 0.0, 0.0,
                                 &save_cb<Output, n_var>, &ctx);
    if (rc == GB_OK) rc = gb_integrator_advance(it, 0, &save_cb<Output, n_var>, &ctx);
    gb_integrator_destroy(it);
    check(rc, "RKEmbeddedGb300::integrate");
  }

#ifdef __CUDACC__
  template <std::size_t n_var>
  struct Kernels {
    using Span = std::span<double, n_var>;
    using CSpan = std::span<double const, n_var>;
    static constexpr void scaled_sq(std::size_t i, double const* v, double const* s, double* out) {
      const double q = v[i] / s[i];
      out[i] = q * q;
    }
  };
#endif

  // Any other ODE: the reference's loop (RKEmbeddedParallel.hpp:13-81) with
  // the ODE's kernels launched by Gb300Executor, the stage, update, target
  // and norm kernels from the library, and the step-size decision on the
  // host (one 8-byte read per attempt, as the reference's CUDA executor).
  template <std::size_t n_var, typename StateType, typename ODE, typename Output,
            typename Executor>
  static void integrate_generic(StateType const& x0s, double t0, double tf,
                                StateType const& atols, StateType const& rtols, ODE ode,
                                Output& output, Executor& exe) {
#ifdef __CUDACC__
    const gb_tableau tab = to_gb_tableau<ButcherTableau>();
    const int S = tab.n_stages;
    const int q = std::min(tab.p, tab.pt);
    const double safety = std::pow(0.38, 1.0 / (1.0 + q));
    gb_stream_t st = exe.stream;
    DevBuf x0(n_var), x(n_var), ks(S * n_var), temp(n_var), err(n_var), target(n_var),
        atol(n_var), rtol(n_var), f0(n_var), x1(n_var), df(n_var);
    to_device<n_var>(x0s, x0.p);
    to_device<n_var>(atols, atol.p);
    to_device<n_var>(rtols, rtol.p);
    const std::size_t wb = gb_rk_norm_workspace_bytes(n_var);
    void* work = nullptr;
    check(gb_device_alloc(&work, wb), "norm workspace");
    auto norm = [&](double const* v, double const* s) {
      double sum = 0.0;
      check(gb_rk_scaled_sq_sum_f64(v, s, n_var, work, wb, &sum, st), "norm");
      return std::sqrt(sum / (double)n_var);
    };
    auto rhs = [&](double const* in, double* out) {
      ode(exe, std::span<double const, n_var>{in, n_var}, std::span<double, n_var>{out, n_var});
    };
    // estimate_initial_step (:170-200)
    {
      std::vector<double> h(n_var), ha(n_var), hr(n_var), tg(n_var);
      check(gb_memcpy(h.data(), x0.p, n_var * 8, 1), "copy");
      check(gb_memcpy(ha.data(), atol.p, n_var * 8, 1), "copy");
      check(gb_memcpy(hr.data(), rtol.p, n_var * 8, 1), "copy");
      for (std::size_t i = 0; i < n_var; ++i) tg[i] = std::abs(h[i]) * hr[i] + ha[i];
      check(gb_memcpy(target.p, tg.data(), n_var * 8, 0), "copy");
    }
    rhs(x0.p, f0.p);
    const double d0 = norm(x0.p, target.p), d1 = norm(f0.p, target.p);
    const double dt0 = (d0 < 1.0e-5 || d1 < 1.0e-5) ? 1.0e-6 : 0.01 * (d0 / d1);
    {
      gb_tableau euler;
      std::memset(&euler, 0, sizeof euler);
      euler.n_stages = 2;
      euler.p = euler.pt = 1;
      euler.a[0][0] = 1.0;
      check(gb_rk_stage_f64(&euler, 1, dt0, x0.p, f0.p, x1.p, n_var, st), "euler");
    }
    rhs(x1.p, df.p);
    {
      std::vector<double> a(n_var), b(n_var);
      check(gb_memcpy(a.data(), df.p, n_var * 8, 1), "copy");
      check(gb_memcpy(b.data(), f0.p, n_var * 8, 1), "copy");
      for (std::size_t i = 0; i < n_var; ++i) a[i] -= b[i];
      check(gb_memcpy(df.p, a.data(), n_var * 8, 0), "copy");
    }
    const double d2 = norm(df.p, target.p) / dt0;
    const double dmax = std::max(d1, d2);
    const double dt1 = dmax <= 1.0e-15 ? std::max(1.0e-6, dt0 * 1.0e-3)
                                       : std::pow(0.01 / dmax, 1.0 / (1.0 + tab.p));
    double dt = std::min(100.0 * dt0, dt1);
    double t = t0;
    check(gb_memcpy(x.p, x0.p, n_var * 8, 2), "copy");
    DeviceStateView<double, n_var> xv{x.p};
    output.save_state(t, xv);
    while (t < tf) {
      rhs(x0.p, ks.p);
      for (int s = 1; s < S; ++s) {
        check(gb_rk_stage_f64(&tab, s, dt, x0.p, ks.p, temp.p, n_var, st), "stage");
        rhs(temp.p, ks.p + s * n_var);
      }
      check(gb_rk_update_state_and_error_f64(&tab, dt, x0.p, ks.p, x.p, err.p, n_var, st),
            "update");
      check(gb_rk_error_target_f64(atol.p, rtol.p, x.p, x0.p, target.p, n_var, st), "target");
      const double e = norm(err.p, target.p);
      if (e <= 1.0) {
        t += dt;
        check(gb_memcpy(x0.p, x.p, n_var * 8, 2), "copy");
        output.save_state(t, xv);
      }
      const double dtnew = dt * safety / std::pow(e, 1.0 / (1.0 + q));
      if (std::abs(dtnew) > 6.0 * std::abs(dt)) {
        dt *= 6.0;
      } else if (std::abs(dtnew) < 0.33 * std::abs(dt)) {
        dt *= 0.33;
      } else if (dtnew / (tf - t0) < 1.0e-12) {
        dt = (tf - t0) * 1.0e-12;
      } else {
        dt = dtnew;
      }
      if (t + dt > tf) dt = tf - t;
    }
    gb_device_free(work);
#else
    static_assert(n_var == 0 && false, "non-N-body ODEs need nvcc (generic kernels)");
#endif
  }
};

inline int32_t pointer_kind(const void* p) { return gb_pointer_kind(p); }

}  // namespace gbode
