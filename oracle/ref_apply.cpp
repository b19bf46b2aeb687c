// Driver that runs the reference's OWN NaN-aware batch apply and masked
// apply (AXIS include/axis/solver/apply.hpp:349-413 and :441-520, the CSR
// team-policy paths, compiled unchanged through the host shims in ref_shim/)
// on a CSR matrix built by the reference's InterpolationMatrix::to_csr, so
// that the oracle's restatements of those loops are pinned bit for bit.
//
// TEST INFRASTRUCTURE ONLY: built by oracle/build.py into
// oracle/_ref/libaxisref_apply.so when the reference checkout exists, and
// loaded only by tests/.

#include <Kokkos_Core.hpp>
#include <axis/solver/apply.hpp>
#include <axis/solver/interpolation_matrix.hpp>
#include <cstdint>
#include <stdexcept>

using HS = Kokkos::HostSpace;
using IM = axis::solver::InterpolationMatrix<HS>;
using i64 = std::int64_t;

namespace {

IM make_matrix(i64 n_src, i64 n_dst, i64 nnz, const i64 *row, const i64 *col, const double *val) {
    Kokkos::View<double *, HS> w("w", nnz), fa("fa", n_src), fb("fb", n_dst), aa("aa", n_src), ab("ab", n_dst);
    Kokkos::View<axis::index_t *, HS> r("r", nnz), c("c", nnz);
    for (i64 k = 0; k < nnz; ++k) {
        w(k) = val[k];
        r(k) = row[k];
        c(k) = col[k];
    }
    IM m(w, r, c, fa, fb, aa, ab, static_cast<std::size_t>(n_src), static_cast<std::size_t>(n_dst));
    m.to_csr();
    return m;
}

}  // namespace

extern "C" {

// nan_batch_apply (apply.hpp:349-413) on LayoutLeft fields x [n_src, nvars]
// and y [n_dst, nvars]. Returns 0, or -3 when it threw.
int ref_nan_batch_apply(i64 n_src, i64 n_dst, i64 nnz, const i64 *row, const i64 *col, const double *val,
                        const double *x, double *y, i64 nvars, double na_thres) {
    try {
        IM m = make_matrix(n_src, n_dst, nnz, row, col, val);
        axis::field_view<const double, 2> src(x, static_cast<std::size_t>(n_src), static_cast<std::size_t>(nvars));
        axis::field_view<double, 2> dst(y, static_cast<std::size_t>(n_dst), static_cast<std::size_t>(nvars));
        axis::solver::nan_batch_apply<HS>(m, src, dst, na_thres);
    } catch (const std::exception &) {
        return -3;
    }
    return 0;
}

// Masked apply (apply.hpp:441-520): rows whose mask is 0 are left as they
// are in y. Returns 0, or -3 when it threw.
int ref_apply_masked(i64 n_src, i64 n_dst, i64 nnz, const i64 *row, const i64 *col, const double *val,
                     const double *x, double *y, const int *mask) {
    try {
        IM m = make_matrix(n_src, n_dst, nnz, row, col, val);
        axis::field_view<const double, 1> src(x, static_cast<std::size_t>(n_src));
        axis::field_view<double, 1> dst(y, static_cast<std::size_t>(n_dst));
        axis::field_view<const int, 1> msk(mask, static_cast<std::size_t>(n_dst));
        axis::solver::apply<HS>(m, src, dst, msk);
    } catch (const std::exception &) {
        return -3;
    }
    return 0;
}

}  // extern "C"
