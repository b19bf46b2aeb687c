// Host stand-in for the part of ArborX v2.1 that the AXIS weight generator
// uses (src/solver/weight_generator.cpp): Point, Box, intersects(), nearest(),
// Experimental::attach_indices, PairValueIndex and BoundingVolumeHierarchy
// with query(space, predicates, values, offsets). ArborX is fetched by the
// reference's CMake (CMakeLists.txt:177-188) and is absent here, so this
// restates its published query semantics by exhaustive search:
//   * intersects(box): every indexed value whose box meets the query box
//     (closed intervals on every axis), in index order;
//   * nearest(point, k): the k values nearest the point by ArborX's distance
//     (float sum of squared coordinate differences, then its square root),
//     closest first; equal distances are ordered by index (ArborX leaves
//     that order unspecified).
// Test infrastructure: used only to build the reference libraries under
// oracle/_ref.
#pragma once

#include <Kokkos_Core.hpp>
#include <algorithm>
#include <cmath>
#include <utility>
#include <vector>

namespace ArborX {

template <int D, class T = float>
struct Point {
    T _c[D];
    T &operator[](int i) { return _c[i]; }
    const T &operator[](int i) const { return _c[i]; }
};

template <int D, class T = float>
struct Box {
    Point<D, T> _min, _max;
    Point<D, T> &minCorner() { return _min; }
    const Point<D, T> &minCorner() const { return _min; }
    Point<D, T> &maxCorner() { return _max; }
    const Point<D, T> &maxCorner() const { return _max; }
};

template <class G>
struct Intersects {
    G geometry;
};
template <class G>
struct Nearest {
    G geometry;
    int k = 1;
};

template <int D, class T>
Intersects<Box<D, T>> intersects(const Box<D, T> &b) {
    return {b};
}
template <int D, class T>
Nearest<Point<D, T>> nearest(const Point<D, T> &p, int k = 1) {
    return {p, k};
}

template <class V, class I = unsigned int>
struct PairValueIndex {
    V value;
    I index;
};

namespace Experimental {
template <class View>
struct AttachedIndices {
    View data;
};
template <class View>
AttachedIndices<View> attach_indices(const View &v) {
    return {v};
}
}  // namespace Experimental

namespace detail {
template <int D, class T>
bool meets(const Box<D, T> &a, const Box<D, T> &b) {
    for (int d = 0; d < D; ++d)
        if (a._max[d] < b._min[d] || b._max[d] < a._min[d]) return false;
    return true;
}
template <int D, class T>
T distance(const Point<D, T> &a, const Point<D, T> &b) {
    T s = 0;
    for (int d = 0; d < D; ++d) {
        const T t = b[d] - a[d];
        s = s + t * t;
    }
    return std::sqrt(s);
}
}  // namespace detail

template <class View>
class BoundingVolumeHierarchy {
   public:
    using geometry_type = typename View::nc_value;
    using value_type = PairValueIndex<geometry_type, unsigned int>;

    BoundingVolumeHierarchy() = default;
    template <class ExecSpace>
    BoundingVolumeHierarchy(const ExecSpace &, const Experimental::AttachedIndices<View> &a) {
        items_.assign(a.data.data(), a.data.data() + a.data.size());
    }
    std::size_t size() const { return items_.size(); }

    template <class ExecSpace, class Queries, class Values, class Offsets>
    void query(const ExecSpace &, const Queries &queries, Values &values, Offsets &offsets) const {
        using Q = typename Queries::nc_value;
        const std::size_t nq = queries.size();
        std::vector<value_type> out;
        std::vector<int> off(nq + 1, 0);
        for (std::size_t q = 0; q < nq; ++q) {
            off[q] = static_cast<int>(out.size());
            run(queries(q), out, static_cast<Q *>(nullptr));
        }
        off[nq] = static_cast<int>(out.size());
        values = Values("values", out.size());
        for (std::size_t i = 0; i < out.size(); ++i) values(i) = out[i];
        offsets = Offsets("offsets", nq + 1);
        for (std::size_t i = 0; i <= nq; ++i) offsets(i) = off[i];
    }

   private:
    std::vector<geometry_type> items_;

    template <class G>
    void run(const Intersects<G> &p, std::vector<value_type> &out, Intersects<G> *) const {
        for (std::size_t i = 0; i < items_.size(); ++i)
            if (detail::meets(items_[i], p.geometry)) out.push_back({items_[i], static_cast<unsigned int>(i)});
    }
    template <class G>
    void run(const Nearest<G> &p, std::vector<value_type> &out, Nearest<G> *) const {
        using T = std::remove_cv_t<std::remove_reference_t<decltype(p.geometry[0])>>;
        std::vector<std::pair<T, unsigned int>> d(items_.size());
        for (std::size_t i = 0; i < items_.size(); ++i)
            d[i] = {detail::distance(p.geometry, items_[i]), static_cast<unsigned int>(i)};
        const std::size_t k = std::min<std::size_t>(static_cast<std::size_t>(std::max(p.k, 0)), d.size());
        std::partial_sort(d.begin(), d.begin() + k, d.end());
        for (std::size_t i = 0; i < k; ++i) out.push_back({items_[d[i].second], d[i].second});
    }
};

template <class ExecSpace, class View>
BoundingVolumeHierarchy(const ExecSpace &, const Experimental::AttachedIndices<View> &) -> BoundingVolumeHierarchy<View>;

}  // namespace ArborX
