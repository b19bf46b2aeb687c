// Minimal layout_left mdspan stand-in (rank 1 and 2) so that the AXIS
// types header compiles with g++ 13, which has no <mdspan>. Test
// infrastructure for oracle/_ref only.
#pragma once

#include <cstddef>
#include <span>

namespace Kokkos {

template <class IndexType, std::size_t... Exts>
struct extents {
    static constexpr std::size_t rank() { return sizeof...(Exts); }
};
template <class IndexType, std::size_t Rank>
struct dextents_helper;
template <class IndexType>
struct dextents_helper<IndexType, 1> {
    using type = extents<IndexType, std::dynamic_extent>;
};
template <class IndexType>
struct dextents_helper<IndexType, 2> {
    using type = extents<IndexType, std::dynamic_extent, std::dynamic_extent>;
};
template <class IndexType, std::size_t Rank>
using dextents = typename dextents_helper<IndexType, Rank>::type;

struct layout_left {};
struct layout_right {};
struct layout_stride {};
template <class T>
struct default_accessor {};

template <class T, class Ext, class Layout = layout_right, class Acc = default_accessor<T>>
class mdspan {
    T *p_ = nullptr;
    std::size_t e_[4] = {0, 0, 0, 0};

   public:
    mdspan() = default;
    template <class... I>
    mdspan(T *p, I... ex) : p_(p) {
        std::size_t a[] = {static_cast<std::size_t>(ex)..., 0};
        for (std::size_t k = 0; k < sizeof...(I); ++k) e_[k] = a[k];
    }
    T *data_handle() const { return p_; }
    std::size_t extent(std::size_t d) const { return e_[d]; }
    T &operator[](std::size_t i) const { return p_[i]; }
    T &operator()(std::size_t i) const { return p_[i]; }
    T &operator()(std::size_t i, std::size_t j) const { return p_[i + j * e_[0]]; }
};

}  // namespace Kokkos
