// The drop-in under nvcc: Gb300State / Gb300Executor behave like the
// reference's CudaState / CudaExecutor (the cases of src/test/CudaStateTest.cu
// and src/test/CudaExecutorTest.cu), and RKEmbeddedGb300 runs the reference's
// golden problems: van der Pol and exponential ODEs (defined here the way the
// reference's ODEs are, kernels launched through Gb300Executor) and the
// five-body system through the device-resident N-body integrator.
#include <array>
#include <numeric>

#include "dropin_common.hpp"

// ODEs with the reference's call shape (src/ode/VanDerPolODE.hpp,
// src/ode/ExponentialODE.hpp), written for this test.
struct VdP {
  static constexpr auto n_var = 2;
  static constexpr void kernel(std::size_t i, std::span<double const, 2> x,
                               std::span<double, 2> dxdt) {
    if (i == 0) {
      dxdt[0] = x[1];
    } else if (i == 1) {
      dxdt[1] = 1.0 * (1.0 - x[0] * x[0]) * x[1] - x[0];
    }
  }
  void operator()(gbode::Gb300Executor& exe, std::span<double const, 2> x,
                  std::span<double, 2> dxdt) {
    exe.call_parallel_kernel<kernel>(2, x, dxdt);
  }
};

struct Expo {
  static constexpr void kernel(std::size_t i, std::span<double const, 10> x,
                               std::span<double, 10> dxdt) {
    dxdt[i] = x[i];
  }
  void operator()(gbode::Gb300Executor& exe, std::span<double const, 10> x,
                  std::span<double, 10> dxdt) {
    exe.call_parallel_kernel<kernel>(10, x, dxdt);
  }
};

using Arr10 = std::array<double, 10>;

constexpr void add_kernel(std::size_t i, double* c, double const* a, double const* b) {
  c[i] = a[i] + b[i];
}
constexpr double binary_add(double a, double b) { return a + b; }
constexpr double multiply(std::size_t i, double const* a, double const* b) { return a[i] * b[i]; }
constexpr void iota_kernel(std::size_t i, double* a) { a[i] = (double)i; }
constexpr void fill_kernel(std::size_t i, double* a, double v) { a[i] = v; }

template <typename BT, typename ODE, std::size_t N>
void run_case(const char* name, ODE ode, std::array<double, N> x0h, double tf, double tol,
              bool& first) {
  using State = gbode::Gb300State<double, N>;
  auto x0 = State{std::span<double const, N>{x0h}};
  std::array<double, N> t{};
  t.fill(tol);
  auto atol = State{std::span<double const, N>{t}};
  auto rtol = atol;
  auto exe = gbode::Gb300Executor{};
  Collect<N> out;
  gbode::RKEmbeddedGb300<BT>::integrate(x0, 0.0, tf, atol, rtol, ode, out, exe);
  print_case(name, out, first);
}

int main() {
  bool first = true;
  int failures = 0;
  std::printf("{\n");
  // --- Gb300State (CudaStateTest.cu:18-92) ---------------------------------
  {
    constexpr std::size_t N = 10;
    std::array<double, N> h{};
    auto s0 = gbode::Gb300State<double, N>{};
    s0.copy_to_span(h);
    for (double v : h) failures += v != 0.0;
    std::array<double, N> src{};
    std::iota(src.begin(), src.end(), 0.0);
    auto s1 = gbode::Gb300State<double, N>{std::span<double const, N>{src}};
    auto s2 = s1;
    std::array<double, N> h1{}, h2{};
    s1.copy_to_span(h1);
    s2.copy_to_span(h2);
    failures += h1 != src || h2 != src;
    auto zero = gbode::Gb300State<double, N>{};
    auto copy = zero;
    auto exe = gbode::Gb300Executor{};
    exe.call_parallel_kernel<iota_kernel>(N, copy.data());
    zero.copy_to_span(h1);
    copy.copy_to_span(h2);
    for (std::size_t i = 0; i < N; ++i) failures += h1[i] != 0.0 || h2[i] != (double)i;
    exe.call_parallel_kernel<fill_kernel>(N, zero.data(), 3.0);
    zero.copy_to_span(h1);
    for (double v : h1) failures += v != 3.0;
    // --- Gb300Executor (CudaExecutorTest.cu:31-61) -------------------------
    std::array<double, N> a{}, b{};
    std::iota(a.begin(), a.end(), 0.0);
    std::iota(b.begin(), b.end(), 1.0);
    auto da = gbode::Gb300State<double, N>{std::span<double const, N>{a}};
    auto db = gbode::Gb300State<double, N>{std::span<double const, N>{b}};
    auto dc = gbode::Gb300State<double, N>{};
    exe.call_parallel_kernel<add_kernel>(N, dc.data(), da.data(), db.data());
    dc.copy_to_span(h1);
    for (std::size_t i = 0; i < N; ++i) failures += h1[i] != 2.0 * i + 1.0;
    const double ip =
        exe.transform_reduce<double, binary_add, multiply>(0.0, N, da.data(), db.data());
    failures += ip != 330.0;
    // move semantics keep both objects valid
    auto moved = std::move(da);
    moved.copy_to_span(h1);
    failures += h1 != a;
    std::printf("\"state_executor_failures\": %d", failures);
    first = false;
  }
  // --- golden problems through RKEmbeddedGb300 -------------------------------
  std::array<double, 2> vdp0{2.0, 0.0};
  const Arr10 e0 = {0.0, 1.0, 2.0, 3.0, 4.0, 5.0, 6.0, 7.0, 8.0, 9.0};
  run_case<gbode::tableau::RKF45>("RKF45VanDerPolConsistencyTest", VdP{}, vdp0, 2.0, 1e-10, first);
  run_case<gbode::tableau::DOPRI5>("DOPRI5VanDerPolConsistencyTest", VdP{}, vdp0, 2.0, 1e-10,
                                   first);
  run_case<gbode::tableau::DVERK>("DVERKVanDerPolConsistencyTest", VdP{}, vdp0, 2.0, 1e-10, first);
  run_case<gbode::tableau::RKF78>("RKF78VanDerPolConsistencyTest", VdP{}, vdp0, 2.0, 1e-10, first);
  run_case<gbode::tableau::HE21>("HE21ExponentialConsistencyTest", Expo{}, e0, 10.0, 1e-6, first);
  run_case<gbode::tableau::RKF45>("RKF45ExponentialConsistencyTest", Expo{}, e0, 10.0, 1e-6,
                                  first);
  run_case<gbode::tableau::DOPRI5>("DOPRI5ExponentialConsistencyTest", Expo{}, e0, 10.0, 1e-6,
                                   first);
  run_case<gbode::tableau::DVERK>("DVERKExponentialConsistencyTest", Expo{}, e0, 10.0, 1e-6,
                                  first);
  run_case<gbode::tableau::RKF78>("RKF78ExponentialConsistencyTest", Expo{}, e0, 10.0, 1e-6,
                                  first);
  std::array<double, 30> nb = {};
  std::copy(kFiveBody, kFiveBody + 30, nb.begin());
  run_case<gbode::tableau::RKF78>("RKF78NBodyConsistencyTest", gbode::NBodyODE<double, 30>{0.0},
                                  nb, 6.3, 1e-10, first);
  std::printf("\n}\n");
  return 0;
}
