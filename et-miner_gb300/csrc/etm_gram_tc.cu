// Exact 0/1 Gram of prefix-group suffixes on the tcgen05 tensor cores.
#include "etm_count.cuh"

namespace etm {

int count_tiles_tensor(const uint64_t*, int64_t, int64_t, const int32_t*, int32_t, const int64_t*, const int32_t*,
                       const int64_t*, const int64_t*, const int64_t*, int64_t, int64_t, const uint8_t*, int32_t*,
                       cudaStream_t) {
    set_error("etm_count_tiles: the tensor-core method is not built in this library");
    return ETM_EINVAL;
}

}  // namespace etm
