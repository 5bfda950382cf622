// Host-compiler-only use of the drop-in (g++, no CUDA headers): the
// device-resident N-body integrator behind RKEmbeddedGb300 with Gb300State.
#include <array>
#include <span>

#include "dropin_common.hpp"

int main() {
  constexpr std::size_t n_var = 30;
  using State = gbode::Gb300State<double, n_var>;
  auto x0 = State{std::span<double const, n_var>{kFiveBody, n_var}};
  std::array<double, n_var> tol{};
  tol.fill(1.0e-10);
  auto atol = State{std::span<double const, n_var>{tol}};
  auto rtol = atol;
  auto exe = gbode::Gb300Executor{};
  bool first = true;
  std::printf("{\n");
  {
    Collect<n_var> out;
    gbode::RKEmbeddedGb300<gbode::tableau::RKF78>::integrate(
        x0, 0.0, 6.3, atol, rtol, gbode::NBodyODE<double, n_var>{0.0}, out, exe);
    print_case("RKF78NBodyConsistencyTest", out, first);
  }
  {
    Collect<n_var> a, b;
    gbode::RKEmbeddedGb300<gbode::tableau::HE21>::integrate(
        x0, 0.0, 0.05, atol, rtol, gbode::NBodyODE<double, n_var>{0.0}, a, exe);
    gbode::RKEmbeddedGb300<RefStyleHE21>::integrate(x0, 0.0, 0.05, atol, rtol,
                                                    gbode::NBodyODE<double, n_var>{0.0}, b, exe);
    print_case("he21_tag", a, first);
    print_case("he21_refstyle", b, first);
  }
  std::printf("\n}\n");
  return 0;
}
