// Declaration-only stand-in for Kokkos::UnorderedMap: the AXIS weight
// generator names it only in its device-space paths, which the host build
// of the reference libraries under oracle/_ref does not instantiate.
// Test infrastructure.
#pragma once

#include <Kokkos_Core.hpp>

namespace Kokkos {
template <class Key, class Value, class Device = HostSpace>
class UnorderedMap;
}  // namespace Kokkos
