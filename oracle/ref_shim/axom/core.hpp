// Stand-in for axom::Array / axom::ArrayView: row-major, host-only storage.
#pragma once
#include <array>
#include <cstddef>
#include <cstdint>
#include <vector>

namespace axom {
enum class MemorySpace { Dynamic, Host, Device, Unified };
using IndexType = std::ptrdiff_t;

template <typename T, int DIM = 1, MemorySpace SPACE = MemorySpace::Dynamic>
class Array {
 public:
  Array() { shape_.fill(0); }
  template <typename... I>
  explicit Array(I... n) : shape_{IndexType(n)...} {
    static_assert(sizeof...(I) == DIM, "shape rank");
    std::size_t total = 1;
    for (auto s : shape_) total *= std::size_t(s);
    data_.resize(total);
  }
  T* data() { return data_.data(); }
  const T* data() const { return data_.data(); }
  IndexType size() const { return IndexType(data_.size()); }
  const std::array<IndexType, DIM>& shape() const { return shape_; }
  bool empty() const { return data_.empty(); }
  template <typename... I>
  T& operator()(I... i) { return data_[offset(i...)]; }
  template <typename... I>
  std::size_t offset(I... i) const {
    IndexType idx[] = {IndexType(i)...};
    std::size_t o = 0;
    for (int k = 0; k < int(sizeof...(I)); k++) o = o * std::size_t(shape_[k]) + std::size_t(idx[k]);
    for (int k = int(sizeof...(I)); k < DIM; k++) o *= std::size_t(shape_[k]);
    return o;
  }
 private:
  std::array<IndexType, DIM> shape_;
  std::vector<T> data_;
};

template <typename T, int DIM = 1, MemorySpace SPACE = MemorySpace::Dynamic>
class ArrayView {
 public:
  ArrayView() : ptr_(nullptr) { shape_.fill(0); }
  ArrayView(Array<T, DIM, SPACE>& a) : ptr_(a.data()), shape_(a.shape()) {}
  ArrayView(T* p, std::array<IndexType, DIM> s) : ptr_(p), shape_(s) {}
  const std::array<IndexType, DIM>& shape() const { return shape_; }
  T* data() const { return ptr_; }
  template <typename... I>
  T& operator()(I... i) const {
    IndexType idx[] = {IndexType(i)...};
    std::size_t o = 0;
    for (int k = 0; k < int(sizeof...(I)); k++) o = o * std::size_t(shape_[k]) + std::size_t(idx[k]);
    for (int k = int(sizeof...(I)); k < DIM; k++) o *= std::size_t(shape_[k]);
    return ptr_[o];
  }
 private:
  T* ptr_;
  std::array<IndexType, DIM> shape_;
};
}  // namespace axom
