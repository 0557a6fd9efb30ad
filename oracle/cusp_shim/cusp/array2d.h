// 2-D containers and views of the CUSP interface subset (row-major only),
// for the CPU build of the reference.  Test infrastructure only.
#pragma once

#include <cusp/array1d.h>

namespace cusp {

template <typename ArrayView, typename Orientation = row_major>
class array2d_view;

template <typename T, typename MemorySpace = device_memory, typename Orientation = row_major>
class array2d {
 public:
  using value_type = T;
  using memory_space = MemorySpace;
  using orientation = Orientation;
  using values_array_type = array1d<T, MemorySpace>;
  using container = array2d<T, MemorySpace, Orientation>;
  using view = array2d_view<typename values_array_type::view, Orientation>;
  using const_view = array2d_view<typename values_array_type::const_view, Orientation>;

  std::size_t num_rows = 0, num_cols = 0, num_entries = 0, pitch = 0;
  values_array_type values;

  array2d() = default;
  array2d(std::size_t r, std::size_t c)
      : num_rows(r), num_cols(c), num_entries(r * c), pitch(c), values(r * c) {}
  array2d(std::size_t r, std::size_t c, const T& v)
      : num_rows(r), num_cols(c), num_entries(r * c), pitch(c), values(r * c, v) {}

  typename values_array_type::view row(std::size_t i) {
    return typename values_array_type::view(values.begin() + i * pitch,
                                            values.begin() + i * pitch + num_cols);
  }
  typename values_array_type::const_view row(std::size_t i) const {
    return typename values_array_type::const_view(values.begin() + i * pitch,
                                                  values.begin() + i * pitch + num_cols);
  }
};

template <typename ArrayView, typename Orientation>
class array2d_view {
 public:
  using values_array_type = ArrayView;
  using value_type = typename ArrayView::value_type;
  using memory_space = device_memory;
  using orientation = Orientation;
  using container =
      array2d<typename std::remove_const<value_type>::type, device_memory, Orientation>;
  using view = array2d_view<ArrayView, Orientation>;

  std::size_t num_rows = 0, num_cols = 0, num_entries = 0, pitch = 0;
  ArrayView values;

  array2d_view() = default;
  array2d_view(std::size_t r, std::size_t c, std::size_t p, const ArrayView& v)
      : num_rows(r), num_cols(c), num_entries(r * c), pitch(p), values(v) {}
  template <typename T, typename M>
  array2d_view(array2d<T, M, Orientation>& a)
      : num_rows(a.num_rows), num_cols(a.num_cols), num_entries(a.num_entries), pitch(a.pitch),
        values(a.values) {}
  template <typename T, typename M>
  array2d_view(const array2d<T, M, Orientation>& a)
      : num_rows(a.num_rows), num_cols(a.num_cols), num_entries(a.num_entries), pitch(a.pitch),
        values(a.values) {}
  template <typename Other>
  array2d_view(const array2d_view<Other, Orientation>& o)
      : num_rows(o.num_rows), num_cols(o.num_cols), num_entries(o.num_entries), pitch(o.pitch),
        values(o.values) {}

  ArrayView row(std::size_t i) const {
    return ArrayView(values.begin() + i * pitch, values.begin() + i * pitch + num_cols);
  }
};

template <typename ArrayView, typename Orientation>
array2d_view<ArrayView, Orientation> make_array2d_view(std::size_t r, std::size_t c,
                                                       std::size_t pitch, const ArrayView& v,
                                                       Orientation) {
  return array2d_view<ArrayView, Orientation>(r, c, pitch, v);
}

}  // namespace cusp
