// Minimal container/view subset of the CUSP interface, written for the CPU
// build of the reference (oracle/refbuild.py).  Only what the segmentation
// path's sources use: owning 1-D arrays over thrust vectors, non-owning
// iterator-range views, and their conversions.  Test infrastructure only.
#pragma once

#include <cstddef>
#include <iterator>
#include <type_traits>

#include <thrust/adjacent_difference.h>
#include <thrust/binary_search.h>
#include <thrust/copy.h>
#include <thrust/device_vector.h>
#include <thrust/equal.h>
#include <thrust/fill.h>
#include <thrust/for_each.h>
#include <thrust/functional.h>
#include <thrust/gather.h>
#include <thrust/host_vector.h>
#include <thrust/iterator/constant_iterator.h>
#include <thrust/iterator/counting_iterator.h>
#include <thrust/iterator/discard_iterator.h>
#include <thrust/iterator/iterator_traits.h>
#include <thrust/iterator/permutation_iterator.h>
#include <thrust/iterator/transform_iterator.h>
#include <thrust/iterator/zip_iterator.h>
#include <thrust/reduce.h>
#include <thrust/remove.h>
#include <thrust/replace.h>
#include <thrust/scan.h>
#include <thrust/scatter.h>
#include <thrust/sequence.h>
#include <thrust/sort.h>
#include <thrust/tabulate.h>
#include <thrust/transform.h>
#include <thrust/tuple.h>
#include <thrust/unique.h>

namespace cusp {

struct device_memory {};
struct host_memory {};
struct row_major {};
struct column_major {};

template <typename Iterator>
class array1d_view;

template <typename T, typename MemorySpace>
class array1d;

namespace shim_detail {
template <typename T, typename M>
struct vector_of {
  using type = thrust::device_vector<T>;
};
template <typename T>
struct vector_of<T, host_memory> {
  using type = thrust::host_vector<T>;
};
}  // namespace shim_detail

template <typename Iterator>
class array1d_view {
 public:
  using iterator = Iterator;
  using value_type = typename thrust::iterator_value<Iterator>::type;
  using reference = typename thrust::iterator_reference<Iterator>::type;
  using size_type = std::size_t;
  using difference_type = typename thrust::iterator_difference<Iterator>::type;
  using memory_space = device_memory;
  using container = array1d<typename std::remove_const<value_type>::type, device_memory>;
  using view = array1d_view<Iterator>;

  array1d_view() : first_(), last_() {}
  array1d_view(Iterator first, Iterator last) : first_(first), last_(last) {}
  template <typename Other,
            typename = typename std::enable_if<std::is_convertible<Other, Iterator>::value>::type>
  array1d_view(const array1d_view<Other>& o) : first_(o.begin()), last_(o.end()) {}
  template <typename T, typename M>
  array1d_view(array1d<T, M>& a) : first_(a.begin()), last_(a.end()) {}
  template <typename T, typename M>
  array1d_view(const array1d<T, M>& a) : first_(a.begin()), last_(a.end()) {}

  Iterator begin() const { return first_; }
  Iterator end() const { return last_; }
  size_type size() const { return static_cast<size_type>(last_ - first_); }
  reference operator[](size_type i) const { return first_[i]; }
  reference back() const { return first_[size() - 1]; }
  array1d_view subarray(size_type start, size_type n) const {
    return array1d_view(first_ + start, first_ + start + n);
  }

 private:
  Iterator first_, last_;
};

template <typename T, typename MemorySpace = device_memory>
class array1d {
  using vec = typename shim_detail::vector_of<T, MemorySpace>::type;

 public:
  using value_type = T;
  using memory_space = MemorySpace;
  using iterator = typename vec::iterator;
  using const_iterator = typename vec::const_iterator;
  using reference = typename vec::reference;
  using const_reference = typename vec::const_reference;
  using size_type = std::size_t;
  using container = array1d<T, MemorySpace>;
  using view = array1d_view<iterator>;
  using const_view = array1d_view<const_iterator>;

  array1d() = default;
  explicit array1d(size_type n) : v_(n) {}
  array1d(size_type n, const T& value) : v_(n, value) {}

  iterator begin() { return v_.begin(); }
  iterator end() { return v_.end(); }
  const_iterator begin() const { return v_.begin(); }
  const_iterator end() const { return v_.end(); }
  size_type size() const { return v_.size(); }
  reference operator[](size_type i) { return v_[i]; }
  const_reference operator[](size_type i) const { return v_[i]; }
  reference back() { return v_[v_.size() - 1]; }
  view subarray(size_type start, size_type n) { return view(begin() + start, begin() + start + n); }
  void resize(size_type n) { v_.resize(n); }

 private:
  vec v_;
};

template <typename Iterator>
array1d_view<Iterator> make_array1d_view(Iterator first, Iterator last) {
  return array1d_view<Iterator>(first, last);
}

}  // namespace cusp
