// Minimal stand-in for the parts of <torch/extension.h> the reference kernel
// sources touch: packed tensor accessors over plain host arrays.
#pragma once
#include <cstdint>

namespace at {
struct DefaultPtrTraits {};
struct RestrictPtrTraits {};
struct Tensor;

template <typename T, int N>
struct TensorAccessorH {
  T* data;
  const int32_t* sizes;
  const int32_t* strides;
  TensorAccessorH<T, N - 1> operator[](int64_t i) const {
    return TensorAccessorH<T, N - 1>{data + i * strides[0], sizes + 1, strides + 1};
  }
  int32_t size(int d) const { return sizes[d]; }
};
template <typename T>
struct TensorAccessorH<T, 1> {
  T* data;
  const int32_t* sizes;
  const int32_t* strides;
  T& operator[](int64_t i) const { return data[i * strides[0]]; }
  int32_t size(int d) const { return sizes[d]; }
};

template <typename T, int N, typename Traits = DefaultPtrTraits, typename index_t = int32_t>
struct PackedTensorAccessor32 {
  T* data = nullptr;
  int32_t sizes_[N] = {};
  int32_t strides_[N] = {};
  PackedTensorAccessor32() = default;
  template <typename Tr2>
  PackedTensorAccessor32(const PackedTensorAccessor32<T, N, Tr2, index_t>& o) : data(o.data) {
    for (int d = 0; d < N; ++d) {
      sizes_[d] = o.sizes_[d];
      strides_[d] = o.strides_[d];
    }
  }
  TensorAccessorH<T, N - 1> operator[](int64_t i) const {
    return TensorAccessorH<T, N - 1>{data + i * strides_[0], sizes_ + 1, strides_ + 1};
  }
  int32_t size(int d) const { return sizes_[d]; }
};

// Contiguous accessor over a host array with the given shape.
template <typename T, int N>
PackedTensorAccessor32<T, N> make_accessor(T* data, const int64_t (&shape)[N]) {
  PackedTensorAccessor32<T, N> a;
  a.data = data;
  int64_t stride = 1;
  for (int d = N - 1; d >= 0; --d) {
    a.sizes_[d] = (int32_t)shape[d];
    a.strides_[d] = (int32_t)stride;
    stride *= shape[d];
  }
  return a;
}
}  // namespace at

namespace torch {
using at::DefaultPtrTraits;
using at::RestrictPtrTraits;
}  // namespace torch
