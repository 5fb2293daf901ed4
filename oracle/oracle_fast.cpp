// CPU ORACLE — TEST INFRASTRUCTURE ONLY (see oracle_core.hpp).
//
// One lane count and scalar type of the throughput form of the tangent and
// heat operators (oracle_fast.hpp), compiled once per -DORC_FAST_W=2,4,8
// (double) and for the FP32 levels (-DORC_FAST_T=float -DORC_FAST_TS=f).
// The C entries in oracle_capi.cpp and the drivers in oracle_problems.hpp
// call the functions below by their suffixed names.
#include "oracle_fast.hpp"

#define ORC_FAST_FN(name) ORC_FAST_CAT3(name, ORC_FAST_W, ORC_FAST_TS)

namespace orc
{
  using ORC_FAST_NS::real;

  int ORC_FAST_FN(nh_vmult_fast_timed_w)(const Box &box, const Basis1D &b, const Material &mat, Caching caching,
                                         const real *u, const real *src, real *dst, int warmup, int reps,
                                         double *seconds)
  {
    using namespace ORC_FAST_NS;
    switch (box.p)
      {
        case 1: return nh_vmult_timed<2>(box, b, mat, caching, u, src, dst, warmup, reps, seconds);
        case 2: return nh_vmult_timed<3>(box, b, mat, caching, u, src, dst, warmup, reps, seconds);
        case 3: return nh_vmult_timed<4>(box, b, mat, caching, u, src, dst, warmup, reps, seconds);
        case 4: return nh_vmult_timed<5>(box, b, mat, caching, u, src, dst, warmup, reps, seconds);
        case 5: return nh_vmult_timed<6>(box, b, mat, caching, u, src, dst, warmup, reps, seconds);
        case 6: return nh_vmult_timed<7>(box, b, mat, caching, u, src, dst, warmup, reps, seconds);
        default: return -2;
      }
  }

  int ORC_FAST_FN(heat_vmult_fast_timed_w)(const Box &box, const Basis1D &b, double k_dt, const real *src,
                                           real *dst, int reps, double *seconds)
  {
    using namespace ORC_FAST_NS;
    switch (box.p)
      {
        case 1: return heat_vmult_timed<2>(box, b, k_dt, src, dst, reps, seconds);
        case 2: return heat_vmult_timed<3>(box, b, k_dt, src, dst, reps, seconds);
        case 3: return heat_vmult_timed<4>(box, b, k_dt, src, dst, reps, seconds);
        case 4: return heat_vmult_timed<5>(box, b, k_dt, src, dst, reps, seconds);
        case 5: return heat_vmult_timed<6>(box, b, k_dt, src, dst, reps, seconds);
        case 6: return heat_vmult_timed<7>(box, b, k_dt, src, dst, reps, seconds);
        default: return -2;
      }
  }

  FastLevel<real> ORC_FAST_FN(make_fast_nh_w)(const Box &box, const Basis1D &b, const Material &mat,
                                              Caching caching, const real *u, bool &ok)
  {
    using namespace ORC_FAST_NS;
    switch (box.p)
      {
        case 1: return make_nh_level<2>(box, b, mat, caching, u, ok);
        case 2: return make_nh_level<3>(box, b, mat, caching, u, ok);
        case 3: return make_nh_level<4>(box, b, mat, caching, u, ok);
        case 4: return make_nh_level<5>(box, b, mat, caching, u, ok);
        case 5: return make_nh_level<6>(box, b, mat, caching, u, ok);
        case 6: return make_nh_level<7>(box, b, mat, caching, u, ok);
        default: throw std::runtime_error("fast form: degree 1..6");
      }
  }

  FastLevel<real> ORC_FAST_FN(make_fast_heat_w)(const Box &box, const Basis1D &b, double k_dt)
  {
    using namespace ORC_FAST_NS;
    switch (box.p)
      {
        case 1: return make_heat_level<2>(box, b, k_dt);
        case 2: return make_heat_level<3>(box, b, k_dt);
        case 3: return make_heat_level<4>(box, b, k_dt);
        case 4: return make_heat_level<5>(box, b, k_dt);
        case 5: return make_heat_level<6>(box, b, k_dt);
        case 6: return make_heat_level<7>(box, b, k_dt);
        default: throw std::runtime_error("fast form: degree 1..6");
      }
  }
} // namespace orc
