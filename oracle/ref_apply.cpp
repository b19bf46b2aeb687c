// Driver that runs the reference's OWN header-only solver code, compiled
// unchanged through the host shims in ref_shim/: the NaN-aware batch apply
// and masked apply (AXIS include/axis/solver/apply.hpp:349-413 and
// :441-520, the CSR team-policy paths) on a CSR matrix built by the
// reference's InterpolationMatrix::to_csr, so that the oracle's restatements
// of those loops are pinned bit for bit; WeightCache::serialize
// (include/axis/solver/weight_cache.hpp:76-139), whose blob pins the device
// library's weight-cache writer and reader byte for byte; and
// check_conservation (src/solver/conservation.cpp, its reductions run in
// index order by the shim).
//
// TEST INFRASTRUCTURE ONLY: built by oracle/build.py into
// oracle/_ref/libaxisref_apply.so when the reference checkout exists, and
// loaded only by tests/.

#include <Kokkos_Core.hpp>
#include <axis/solver/apply.hpp>
#include <axis/solver/conservation.hpp>
#include <axis/solver/interpolation_matrix.hpp>
#include <axis/solver/weight_cache.hpp>
#include <cstdint>
#include <stdexcept>

using HS = Kokkos::HostSpace;
using IM = axis::solver::InterpolationMatrix<HS>;
using i64 = std::int64_t;

namespace {

IM make_coo(i64 n_src, i64 n_dst, i64 nnz, const i64 *row, const i64 *col, const double *val, const double *pfa,
             const double *pfb, const double *paa, const double *pab) {
    Kokkos::View<double *, HS> w("w", nnz), fa("fa", n_src), fb("fb", n_dst), aa("aa", n_src), ab("ab", n_dst);
    Kokkos::View<axis::index_t *, HS> r("r", nnz), c("c", nnz);
    for (i64 k = 0; k < nnz; ++k) {
        w(k) = val[k];
        r(k) = row[k];
        c(k) = col[k];
    }
    for (i64 i = 0; i < n_src; ++i) {
        fa(i) = pfa ? pfa[i] : 0.0;
        aa(i) = paa ? paa[i] : 0.0;
    }
    for (i64 j = 0; j < n_dst; ++j) {
        fb(j) = pfb ? pfb[j] : 0.0;
        ab(j) = pab ? pab[j] : 0.0;
    }
    return IM(w, r, c, fa, fb, aa, ab, static_cast<std::size_t>(n_src), static_cast<std::size_t>(n_dst));
}

IM make_matrix(i64 n_src, i64 n_dst, i64 nnz, const i64 *row, const i64 *col, const double *val) {
    IM m = make_coo(n_src, n_dst, nnz, row, col, val, nullptr, nullptr, nullptr, nullptr);
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

// check_conservation (src/solver/conservation.cpp) for a matrix's frac/area
// arrays and one source and destination field; norm_type 0 DstArea,
// 1 FracArea. out = (src_integral, dst_integral, absolute_error,
// relative_error). Returns 0, or -3 when it threw.
int ref_conservation(i64 n_src, const double *src, const double *area_a, const double *frac_a, i64 n_dst,
                     const double *dst, const double *area_b, const double *frac_b, int norm_type, double *out) {
    try {
        const i64 zero = 0;
        IM m = make_coo(n_src, n_dst, 0, &zero, &zero, nullptr, frac_a, frac_b, area_a, area_b);
        axis::field_view<const double, 1> s(src, static_cast<std::size_t>(n_src));
        axis::field_view<const double, 1> d(dst, static_cast<std::size_t>(n_dst));
        auto r = axis::solver::check_conservation<HS>(
            s, d, m, norm_type ? axis::solver::NormType::FracArea : axis::solver::NormType::DstArea);
        out[0] = r.src_integral;
        out[1] = r.dst_integral;
        out[2] = r.absolute_error;
        out[3] = r.relative_error;
    } catch (const std::exception &) {
        return -3;
    }
    return 0;
}

// WeightCache::serialize of the COO matrix (row, col, val in the given
// order) with its frac/area arrays. Query with buf = null: *size receives
// the blob size. Returns 0, or -3 when it threw (buffer too small).
int ref_cache_serialize(i64 n_src, i64 n_dst, i64 nnz, const i64 *row, const i64 *col, const double *val,
                        const double *fa, const double *fb, const double *aa, const double *ab, unsigned char *buf,
                        i64 cap, i64 *size) {
    try {
        IM m = make_coo(n_src, n_dst, nnz, row, col, val, fa, fb, aa, ab);
        *size = static_cast<i64>(axis::solver::WeightCache::serialize(m, buf, static_cast<std::size_t>(cap)));
    } catch (const std::exception &) {
        return -3;
    }
    return 0;
}

}  // extern "C"
