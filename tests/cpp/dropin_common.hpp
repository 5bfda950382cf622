// Shared pieces of the C++ drop-in tests: a RawOutput-like collector and
// JSON printing of the rows the reference's golden tests look at
// (front, size/2, back).
#pragma once
#include <cstdio>
#include <span>
#include <string>
#include <vector>

#include "gbode/gbode.hpp"

// Same contract as the reference's RawOutput (src/output/RawOutput.hpp:15-19):
// save_state(t, x) appends t and a host copy of x.
template <std::size_t N>
struct Collect {
  std::vector<double> times;
  std::vector<std::vector<double>> states;
  template <typename State>
  void save_state(double t, State const& x) {
    times.push_back(t);
    states.emplace_back(N);
    x.copy_to_span(std::span<double, N>{states.back().data(), N});
  }
};

inline void print_row(const std::vector<double>& v) {
  std::printf("[");
  for (std::size_t i = 0; i < v.size(); ++i) std::printf(i ? ",%.17g" : "%.17g", v[i]);
  std::printf("]");
}

template <std::size_t N>
void print_case(const char* name, const Collect<N>& c, bool& first) {
  const std::size_t n = c.times.size();
  std::printf("%s\"%s\": {\"n_saved\": %zu, \"times\": [%.17g, %.17g, %.17g], \"rows\": [",
              first ? "" : ",\n", name, n, c.times[0], c.times[n / 2], c.times[n - 1]);
  print_row(c.states[0]);
  std::printf(",");
  print_row(c.states[n / 2]);
  std::printf(",");
  print_row(c.states[n - 1]);
  std::printf("]}");
  first = false;
}

// The five-body planar system of the reference's N-body test
// (src/test/NBodyTest.hpp:13-18), epsilon = 0, unit masses.
inline constexpr double kFiveBody[30] = {
    1.657666,  0.0,       0.0, 0.439775,  -0.169717, 0.0, -1.268608, -0.267651, 0.0,
    -1.268608, 0.267651,  0.0, 0.439775,  0.169717,  0.0, 0.0,       -0.593786, 0.0,
    1.822785,  0.128248,  0.0, 1.271564,  0.168645,  0.0, -1.271564, 0.168645,  0.0,
    -1.822785, 0.128248,  0.0};

// A tableau in the reference's butcher_tableaus/BT*.hpp layout (Heun-Euler
// 2(1)), to show that reference-style tableau types are accepted.
struct RefStyleHE21 {
  static constexpr auto a = std::array<std::array<double, 1>, 1>{{1.0}};
  static constexpr auto b = std::array{1.0 / 2.0, 1.0 / 2.0};
  static constexpr auto bt = std::array{1.0, 0.0};
  static constexpr auto p = 2;
  static constexpr auto pt = 1;
  static constexpr auto n_stages = static_cast<int>(b.size());
};
