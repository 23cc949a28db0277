// AllPairs zip(x*y)/reduce(x+y) on the tcgen05 tensor cores (3xBF16).
// Placeholder until the contraction kernel lands: reports "not supported" so
// the launch falls back to the CUDA-core kernel.
#include <cstdint>

#include "internal.h"

namespace scl {

bool allpairs_tc_supported(uint32_t, uint32_t, uint32_t, const void*, const void*, const void*) {
  return false;
}

int allpairs_tc_launch(const float*, const float*, float*, uint32_t, uint32_t, uint32_t,
                       cudaStream_t, uint32_t, unsigned int*) {
  return fail(SCL_ERR_UNSUPPORTED, "tensor-core AllPairs is not built");
}

}  // namespace scl
