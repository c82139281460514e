// Internal interfaces between the counting translation units.
#pragma once

#include "etm_common.cuh"

namespace etm {

int count_tiles_popcount(const uint64_t* fbv, int64_t ld, int64_t n_words, const int32_t* rows, int32_t width,
                         const int64_t* grp_first, const int32_t* grp_size, const int64_t* cand_off,
                         const int64_t* work_groups, const int64_t* work_off, int64_t n_work, int64_t chunk_base,
                         const uint8_t* cls, int32_t* out, int64_t n_tiles_hint, cudaStream_t s);

int count_tiles_proj_popcount(const uint64_t* cbuf, const int64_t* cbase, const int64_t* cwords, const int64_t* cld,
                              const int32_t* grp_size, const int64_t* cand_off, const int64_t* work_groups,
                              const int64_t* work_off, int64_t n_work, int64_t chunk_base, const uint8_t* cls,
                              int32_t* out, cudaStream_t s);

int proj_status_take(cudaStream_t s, int* out);

int gram_tc(const uint64_t* cbuf, const int64_t* cbase, const int64_t* cwords, const int64_t* cld,
            const int32_t* grp_size, const int64_t* cand_off, const int64_t* work_groups, const int64_t* work_off,
            int64_t n_work, int64_t n_tiles, int64_t chunk_base, const uint8_t* cls, int32_t elem, int32_t* out,
            int64_t* work_counter, cudaStream_t s);

int count_tiles_tensor(const uint64_t* fbv, int64_t ld, int64_t n_words, const int32_t* rows, int32_t width,
                       const int64_t* grp_first, const int32_t* grp_size, const int64_t* cand_off,
                       const int64_t* work_groups, const int64_t* work_off, int64_t n_work, int64_t chunk_base,
                       const uint8_t* cls, int32_t* out, cudaStream_t s);

}  // namespace etm
