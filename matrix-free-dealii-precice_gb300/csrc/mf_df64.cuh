// Double-float ("df64") arithmetic on the FP32 pipe.
//
// GB300 executes FP64 at 1.25 TFLOP/s but FP32 at ~73 TFLOP/s.  A df64
// number is an unevaluated sum hi + lo of two floats (|lo| <= ulp(hi)/2),
// carrying ~48 significant bits.  Products use the exact FMA residual
// (TwoProduct), sums use Knuth's TwoSum, both error-free transformations
// (Dekker 1971; Knuth TAOCP vol. 2; the compensated dot product follows
// Ogita, Rump, Oishi, "Accurate sum and dot product", SIAM J. Sci. Comput.
// 26 (2005)).  Relative rounding of a dot product is ~2^-48 times its
// condition number, well inside the 1e-12 operator tolerance.
//
// All float operations use the _rn intrinsics so that the compiler neither
// contracts nor reorders them.
#pragma once

#include <cuda_runtime.h>

namespace mfgpu
{
  struct __align__(8) df64
  {
    float hi, lo;
  };

  __host__ __device__ inline df64
  df_from_double_host(double x)
  {
    const float h = float(x);
    return {h, float(x - double(h))};
  }

  __device__ __forceinline__ df64
  df_from_double(double x)
  {
    const float h = __double2float_rn(x);
    return {h, __double2float_rn(x - double(h))};
  }

  __device__ __forceinline__ double
  df_to_double(df64 a)
  {
    return double(a.hi) + double(a.lo);
  }

  __device__ __forceinline__ void
  two_sum(float a, float b, float &s, float &e)
  {
    s              = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    e              = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  }

  __device__ __forceinline__ void
  quick_two_sum(float a, float b, float &s, float &e)
  {
    s = __fadd_rn(a, b);
    e = __fsub_rn(b, __fsub_rn(s, a));
  }

  // float -> double by exponent/mantissa re-encoding (integer pipe only);
  // zeros, float subnormals, infinities and NaN take the ordinary path
  __device__ __forceinline__ double
  f2d_bits(float f)
  {
    const unsigned u = __float_as_uint(f);
    const unsigned e = (u >> 23) & 0xffu;
    if (e == 0u || e == 255u)
      return double(f);
    const unsigned long long bits =
      (static_cast<unsigned long long>(u >> 31) << 63) |
      (static_cast<unsigned long long>(e + 896u) << 52) |
      (static_cast<unsigned long long>(u & 0x7fffffu) << 29);
    return __longlong_as_double(static_cast<long long>(bits));
  }

  // double -> df64 by splitting the mantissa: hi keeps the leading 24
  // significant bits (exact float), lo = x - hi rounded to 24 bits.  Uses
  // integer operations and one integer-to-float conversion; magnitudes
  // outside [2^-74, 2^127] take the FP64 path.
  __device__ __forceinline__ df64
  df_from_double_bits(double x)
  {
    const unsigned long long b = static_cast<unsigned long long>(__double_as_longlong(x));
    const unsigned           e = static_cast<unsigned>(b >> 52) & 0x7ffu;
    if (e < 949u || e > 1150u)
      return df_from_double(x);
    const unsigned sign = static_cast<unsigned>(b >> 63) << 31;
    const float    hi   = __uint_as_float(sign | ((e - 896u) << 23) |
                                          (static_cast<unsigned>(b >> 29) & 0x7fffffu));
    const unsigned r     = static_cast<unsigned>(b & 0x1fffffffu);
    const float    scale = __uint_as_float((e - 948u) << 23); // 2^(e - 1075)
    const float    lo    = __uint_as_float(sign | __float_as_uint(__fmul_rn(__uint2float_rn(r), scale)));
    float          s, t;
    quick_two_sum(hi, lo, s, t);
    return {s, t};
  }

  // df64 -> double: exact float->double re-encodings and one FP64 add
  __device__ __forceinline__ double
  df_to_double_bits(df64 a)
  {
    return f2d_bits(a.hi) + f2d_bits(a.lo);
  }

  __device__ __forceinline__ df64
  operator+(df64 a, df64 b)
  {
    float s, e, t, f;
    two_sum(a.hi, b.hi, s, e);
    two_sum(a.lo, b.lo, t, f);
    e = __fadd_rn(e, t);
    quick_two_sum(s, e, s, e);
    e = __fadd_rn(e, f);
    quick_two_sum(s, e, s, e);
    return {s, e};
  }

  __device__ __forceinline__ df64
  operator-(df64 a)
  {
    return {-a.hi, -a.lo};
  }

  __device__ __forceinline__ df64
  operator-(df64 a, df64 b)
  {
    return a + (-b);
  }

  __device__ __forceinline__ df64
  operator*(df64 a, df64 b)
  {
    const float p = __fmul_rn(a.hi, b.hi);
    float       e = __fmaf_rn(a.hi, b.hi, -p);
    e             = __fmaf_rn(a.hi, b.lo, e);
    e             = __fmaf_rn(a.lo, b.hi, e);
    float s;
    quick_two_sum(p, e, s, e);
    return {s, e};
  }

  __device__ __forceinline__ df64 &
  operator+=(df64 &a, df64 b)
  {
    a = a + b;
    return a;
  }

  __device__ __forceinline__ df64 &
  operator*=(df64 &a, df64 b)
  {
    a = a * b;
    return a;
  }

  // a*b + c with one TwoSum (accurate to ~2^-48 relative to |a b| + |c|)
  __device__ __forceinline__ df64
  fma_(df64 a, df64 b, df64 c)
  {
    const float p = __fmul_rn(a.hi, b.hi);
    float       e = __fmaf_rn(a.hi, b.hi, -p);
    e             = __fmaf_rn(a.hi, b.lo, e);
    e             = __fmaf_rn(a.lo, b.hi, e);
    float s, t;
    two_sum(p, c.hi, s, t);
    t = __fadd_rn(t, __fadd_rn(e, c.lo));
    quick_two_sum(s, t, s, t);
    return {s, t};
  }

  // compensated dot-product accumulator: terms are added with TwoSum on the
  // high parts and plain float sums of the low parts; normalised at the end
  struct DfAcc
  {
    float s, t;
    __device__ __forceinline__ void
    init(df64 a, df64 b)
    {
      s = __fmul_rn(a.hi, b.hi);
      t = __fmaf_rn(a.hi, b.hi, -s);
      t = __fmaf_rn(a.hi, b.lo, t);
      t = __fmaf_rn(a.lo, b.hi, t);
    }
    __device__ __forceinline__ void
    init_add(df64 c)
    {
      s = c.hi;
      t = c.lo;
    }
    __device__ __forceinline__ void
    add(df64 a, df64 b)
    {
      const float p = __fmul_rn(a.hi, b.hi);
      float       e = __fmaf_rn(a.hi, b.hi, -p);
      e             = __fmaf_rn(a.hi, b.lo, e);
      e             = __fmaf_rn(a.lo, b.hi, e);
      float q, r;
      two_sum(s, p, q, r);
      s = q;
      t = __fadd_rn(t, __fadd_rn(r, e));
    }
    __device__ __forceinline__ df64
    result() const
    {
      float a, b;
      quick_two_sum(s, t, a, b);
      return {a, b};
    }
  };

  // conversions between storage and compute types
  template <typename TC, typename TS>
  __device__ __forceinline__ TC
  to_compute(TS x)
  {
    return TC(x);
  }
  template <>
  __device__ __forceinline__ df64
  to_compute<df64, double>(double x)
  {
    return df_from_double_bits(x);
  }
  template <typename TS, typename TC>
  __device__ __forceinline__ TS
  to_storage(TC x)
  {
    return TS(x);
  }
  template <>
  __device__ __forceinline__ double
  to_storage<double, df64>(df64 x)
  {
    return df_to_double_bits(x);
  }

  // compile-time constant in the compute type
  template <typename T>
  __device__ __forceinline__ T
  cst(double v)
  {
    return T(v);
  }
  template <>
  __device__ __forceinline__ df64
  cst<df64>(double v)
  {
    return df_from_double(v);
  }

  template <typename T>
  struct is_df64
  {
    static constexpr bool value = false;
  };
  template <>
  struct is_df64<df64>
  {
    static constexpr bool value = true;
  };
} // namespace mfgpu
