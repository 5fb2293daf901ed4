// CPU ORACLE — TEST INFRASTRUCTURE ONLY (see oracle_core.hpp).
//
// One lane count of the throughput form of the tangent and heat vmults
// (oracle_fast.hpp), compiled once per -DORC_FAST_W=2,4,8; the C entry
// or_nh_vmult_fast_timed in oracle_capi.cpp dispatches on the lane count.
#include "oracle_fast.hpp"

namespace orc
{
  int ORC_FAST_CAT(nh_vmult_fast_timed_w, ORC_FAST_W)(const Box &box, const Basis1D &b, const Material &mat,
                                                       Caching caching, const double *u, const double *src,
                                                       double *dst, int reps, double *seconds)
  {
    using namespace ORC_FAST_NS;
    switch (box.p)
      {
        case 1: return nh_vmult_timed<2>(box, b, mat, caching, u, src, dst, reps, seconds);
        case 2: return nh_vmult_timed<3>(box, b, mat, caching, u, src, dst, reps, seconds);
        case 3: return nh_vmult_timed<4>(box, b, mat, caching, u, src, dst, reps, seconds);
        case 4: return nh_vmult_timed<5>(box, b, mat, caching, u, src, dst, reps, seconds);
        case 5: return nh_vmult_timed<6>(box, b, mat, caching, u, src, dst, reps, seconds);
        case 6: return nh_vmult_timed<7>(box, b, mat, caching, u, src, dst, reps, seconds);
        default: return -2;
      }
  }

  int ORC_FAST_CAT(heat_vmult_fast_timed_w, ORC_FAST_W)(const Box &box, const Basis1D &b, double k_dt,
                                                         const double *src, double *dst, int reps,
                                                         double *seconds)
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
} // namespace orc
