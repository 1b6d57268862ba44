// Argument validation helpers for the C ABI.
#pragma once

#include <string>

#include "common.cuh"

namespace totri {

inline const char* dtype_name(int d) {
  switch (d) {
    case TOTRI_FLOAT32: return "float32";
    case TOTRI_FLOAT64: return "float64";
    case TOTRI_INT32: return "int32";
    case TOTRI_INT64: return "int64";
    default: return "unknown";
  }
}

inline std::string shape_str(const totri_array_t* a) {
  std::string s = "[";
  for (int i = 0; i < a->ndim; ++i) {
    if (i) s += ", ";
    s += std::to_string(a->shape[i]);
  }
  return s + "]";
}

inline int64_t numel(const totri_array_t* a) {
  int64_t n = 1;
  for (int i = 0; i < a->ndim; ++i) n *= a->shape[i];
  return n;
}

inline bool is_contiguous(const totri_array_t* a) {
  int64_t expect = 1;
  for (int i = a->ndim - 1; i >= 0; --i) {
    if (a->shape[i] != 1 && a->strides[i] != expect) return false;
    expect *= a->shape[i];
  }
  return true;
}

// Checks presence, rank and dtype; returns TOTRI_OK or an error.
inline int check_array(const totri_array_t* a, const char* name, int ndim, int dtype) {
  if (!a) return fail(TOTRI_ERR_INVALID_ARGUMENT, std::string(name) + " is missing");
  if (a->ndim != ndim)
    return fail(TOTRI_ERR_INVALID_ARGUMENT, std::string(name) + " must have " +
                                                std::to_string(ndim) + " dimensions, got " +
                                                shape_str(a));
  if (dtype >= 0 && a->dtype != dtype)
    return fail(TOTRI_ERR_INVALID_ARGUMENT, std::string(name) + " must be " + dtype_name(dtype) +
                                                ", got " + dtype_name(a->dtype));
  if (!a->data && numel(a) > 0)
    return fail(TOTRI_ERR_INVALID_ARGUMENT, std::string(name) + " has a null data pointer");
  return TOTRI_OK;
}

inline int check_dim(const totri_array_t* a, const char* name, int dim, int64_t expect) {
  if (a->shape[dim] != expect)
    return fail(TOTRI_ERR_INVALID_ARGUMENT, std::string(name) + " has shape " + shape_str(a) +
                                                ", expected size " + std::to_string(expect) +
                                                " in dimension " + std::to_string(dim));
  return TOTRI_OK;
}

inline int check_contiguous(const totri_array_t* a, const char* name) {
  if (!is_contiguous(a))
    return fail(TOTRI_ERR_INVALID_ARGUMENT, std::string(name) + " must be C-contiguous");
  return TOTRI_OK;
}

inline View3f view3f(const totri_array_t* a) {
  return View3f{static_cast<const float*>(a->data), a->strides[0], a->strides[1],
                a->strides[2]};
}

#define TOTRI_TRY(expr)            \
  do {                             \
    int st__ = (expr);             \
    if (st__ != TOTRI_OK) return st__; \
  } while (0)

}  // namespace totri
