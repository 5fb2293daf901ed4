// CPU ORACLE — TEST INFRASTRUCTURE ONLY (see oracle_core.hpp).
//
// Declarations of the throughput form's entries (oracle_fast.cpp, one object
// per lane count W and scalar type: wWd for double, w4f for float).
#pragma once

#include "oracle_ops.hpp"

namespace orc
{
#define ORC_FAST_DECL(sfx, T)                                                                                    \
  int nh_vmult_fast_timed_##sfx(const Box &box, const Basis1D &b, const Material &mat, Caching caching,         \
                                const T *u, const T *src, T *dst, int warmup, int reps, double *seconds);       \
  int heat_vmult_fast_timed_##sfx(const Box &box, const Basis1D &b, double k_dt, const T *src, T *dst, int reps, \
                                  double *seconds);                                                             \
  FastLevel<T> make_fast_nh_##sfx(const Box &box, const Basis1D &b, const Material &mat, Caching caching,        \
                                  const T *u, bool &ok);                                                        \
  FastLevel<T> make_fast_heat_##sfx(const Box &box, const Basis1D &b, double k_dt);
  ORC_FAST_DECL(w2d, double)
  ORC_FAST_DECL(w4d, double)
  ORC_FAST_DECL(w8d, double)
  ORC_FAST_DECL(w4f, float)
#undef ORC_FAST_DECL

  // the level operators a driver uses: 2 lanes in FP64, 4 in FP32 (the
  // widths of a 128-bit vector)
  inline FastLevel<double>
  make_fast_nh(const Box &box, const Basis1D &b, const Material &mat, Caching caching, const double *u, bool &ok)
  {
    return make_fast_nh_w2d(box, b, mat, caching, u, ok);
  }
  inline FastLevel<float>
  make_fast_nh(const Box &box, const Basis1D &b, const Material &mat, Caching caching, const float *u, bool &ok)
  {
    return make_fast_nh_w4f(box, b, mat, caching, u, ok);
  }
  template <typename T>
  FastLevel<T> make_fast_heat(const Box &box, const Basis1D &b, double k_dt);
  template <>
  inline FastLevel<double>
  make_fast_heat<double>(const Box &box, const Basis1D &b, double k_dt)
  {
    return make_fast_heat_w2d(box, b, k_dt);
  }
  template <>
  inline FastLevel<float>
  make_fast_heat<float>(const Box &box, const Basis1D &b, double k_dt)
  {
    return make_fast_heat_w4f(box, b, k_dt);
  }
} // namespace orc
