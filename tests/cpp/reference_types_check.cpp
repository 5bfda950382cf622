// Compile-only check (where the reference's headers are available): the
// reference's own state, ODE, output and tableau types plug into
// gbode::RKEmbeddedGb300 unchanged, and Gb300State satisfies the reference's
// ODEState concept (src/state/ODEState.hpp:25-43).
#include "BTDOPRI5.hpp"
#include "BTRKF78.hpp"
#include "HeapState.hpp"
#include "NBodyODE.hpp"
#include "ODEState.hpp"
#include "RawOutput.hpp"
#include "gbode/gbode.hpp"

static_assert(ODEState<gbode::Gb300State<double, 6144>>);
static_assert(ODEState<gbode::HostStateView<double, 6144>>);

void drop_in(HeapState<double, 6144> const& x0, HeapState<double, 6144> const& tol,
             RawOutput<HeapState<double, 6144>>& output) {
  auto exe = gbode::Gb300Executor{};
  gbode::RKEmbeddedGb300<BTDOPRI5>::integrate(x0, 0.0, 1.0, tol, tol,
                                             NBodyODE<double, 6144>{0.01}, output, exe);
  auto dx0 = gbode::Gb300State<double, 6144>{std::span<double const, 6144>{x0.data(), 6144}};
  gbode::RKEmbeddedGb300<BTRKF78>::integrate(dx0, 0.0, 1.0, dx0, dx0,
                                            NBodyODE<double, 6144>{0.01}, output, exe);
}
