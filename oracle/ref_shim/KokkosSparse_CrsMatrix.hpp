// Stand-in for the KokkosKernels CrsMatrix type named by the reference's
// InterpolationMatrix (a lazily built apply operator that the fast-path
// oracle never builds): only a default-constructible type with the graph
// typedef. Test infrastructure for oracle/_ref.
#pragma once

namespace KokkosSparse {

template <class Value, class Ordinal, class Device, class Traits, class Size>
struct CrsMatrix {
    struct staticcrsgraph_type {
        template <class E, class R>
        staticcrsgraph_type(const E &, const R &) {}
    };
    CrsMatrix() = default;
    template <class V, class G>
    CrsMatrix(const char *, Ordinal, const V &, const G &) {}
};

}  // namespace KokkosSparse
