// Internal interfaces between the counting translation units.
#pragma once

#include "etm_common.cuh"

namespace etm {

int count_tiles_popcount(const uint64_t* fbv, int64_t ld, int64_t n_words, const int32_t* rows, int32_t width,
                         const int64_t* grp_first, const int32_t* grp_size, const int64_t* cand_off,
                         const int64_t* work_groups, const int64_t* work_off, int64_t n_work, int64_t chunk_base,
                         const uint8_t* cls, int32_t* out, int64_t n_tiles_hint, cudaStream_t s, int32_t min_count,
                         uint32_t* surv);

int count_tiles_proj_popcount(const uint64_t* cbuf, const int64_t* cbase, const int64_t* cwords, const int64_t* cld,
                              const int32_t* grp_size, const int64_t* cand_off, const int64_t* work_groups,
                              const int64_t* work_off, int64_t n_work, int64_t chunk_base, const uint8_t* cls,
                              int32_t* out, cudaStream_t s, int32_t min_count, uint32_t* surv);

int proj_status_take(cudaStream_t s, int* out);
// The projection's first wait for a member's bulk copies, in ns (negative: the default; 0: give up at once).
void proj_set_first_wait(int64_t ns);

// Members per block of the Gram kernel for an element code (0 if the code is unknown).
int gram_block_members(int32_t elem);

// The Gram of projected member words: dense counts (surv == nullptr) or, with a survivor bitmask, only
// the counts reaching min_count and their bits.
int gram_tc(const uint64_t* cbuf, const int64_t* cbase, const int64_t* cwords, const int64_t* cld,
            const int32_t* grp_size, const int64_t* cand_off, const int64_t* work_groups, const int64_t* work_off,
            int64_t n_work, int64_t n_tiles, int64_t chunk_base, const uint8_t* cls, int32_t elem, int32_t min_count,
            int32_t* out, uint32_t* surv, int64_t* work_counter, cudaStream_t s);

int count_tiles_tensor(const uint64_t* fbv, int64_t ld, int64_t n_words, const int32_t* rows, int32_t width,
                       const int64_t* grp_first, const int32_t* grp_size, const int64_t* cand_off,
                       const int64_t* work_groups, const int64_t* work_off, int64_t n_work, int64_t chunk_base,
                       const uint8_t* cls, int32_t* out, cudaStream_t s);

}  // namespace etm
