// fuelg_tc.cu -- tensor-core (tcgen05) tiers.
#include "fuelg_common.cuh"
#include "fuelg_internal.h"

namespace fuelg {

int lloyd_assign_tc(const LloydParams&, const float*, int32_t*, int32_t*, int64_t*, int*, cudaStream_t) {
  set_error("the tensor-core Lloyd tier is not available yet");
  return ST_ENOTSUP;
}

}  // namespace fuelg
