// Stand-in for KokkosSparse::spmv (KokkosKernels 5.1.1, fetched by the
// reference's CMake and absent here). The reference libraries under
// oracle/_ref call only the team-policy and COO paths of
// include/axis/solver/apply.hpp, which do not use it; a call throws.
// Test infrastructure.
#pragma once

#include <KokkosSparse_CrsMatrix.hpp>
#include <stdexcept>

namespace KokkosSparse {
template <class A, class X, class Y>
void spmv(const char *, double, const A &, const X &, double, const Y &) {
    throw std::logic_error("KokkosSparse::spmv is not part of the host shim");
}
}  // namespace KokkosSparse
