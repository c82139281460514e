// The input layer's row order and tile occupancy: sort keys that gather the rows sharing their most
// frequent columns (the lex row order), the transaction CSR permuted into that order, and per column one
// bit per 32-word tile holding a row of it, which lets the prefix and per-candidate kernels skip tiles.
//
// HBM-bound integer work: warps over rows / occupancy words, grids a multiple of the SM count.
#include "etm_common.cuh"

namespace {

using namespace etm;

constexpr int IN_THREADS = 256;

__device__ inline uint64_t warp_or64(uint64_t x) {
    const unsigned lo = __reduce_or_sync(0xffffffffu, (unsigned)x);
    const unsigned hi = __reduce_or_sync(0xffffffffu, (unsigned)(x >> 32));
    return ((uint64_t)hi << 32) | lo;
}

// One warp per row. A row holding the column of rank r (ranks by descending support) sets bit 63 - r of its
// high key for r < 64 and bit 127 - r of its low key for 64 <= r < 128 (the key of
// gpu/kernels/_src/csr_to_bitvec.cu:75-104). Both keys are stored with their top bit flipped, so that an
// ascending signed sort orders them as unsigned values.
__global__ void __launch_bounds__(IN_THREADS) row_order_keys_kernel(const int64_t* __restrict__ row_ptr,
                                                                    const int32_t* __restrict__ cols, int64_t n_rows,
                                                                    const int32_t* __restrict__ rank_of_col,
                                                                    int64_t n_cols, int64_t* __restrict__ key_hi,
                                                                    int64_t* __restrict__ key_lo) {
    const int lane = threadIdx.x & 31;
    const int64_t n_warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < n_rows; r += n_warps) {
        const int64_t e1 = row_ptr[r + 1];
        uint64_t hi = 0, lo = 0;
        for (int64_t e = row_ptr[r] + lane; e < e1; e += 32) {
            const int32_t c = cols[e];
            if (c < 0 || c >= n_cols) continue;
            const int32_t k = rank_of_col[c];
            if (k >= 0 && k < 64) hi |= 1ULL << (63 - k);
            else if (k >= 64 && k < 128) lo |= 1ULL << (127 - k);
        }
        hi = warp_or64(hi);
        lo = warp_or64(lo);
        if (lane == 0) {
            key_hi[r] = (int64_t)(hi ^ (1ULL << 63));
            key_lo[r] = (int64_t)(lo ^ (1ULL << 63));
        }
    }
}

// One warp per output row p: input row order[p]'s entries copied to new_ptr[p] onwards. A row whose source
// index or destination range falls outside the arrays is skipped and reported in *bad.
__global__ void __launch_bounds__(IN_THREADS) permute_rows_kernel(const int64_t* __restrict__ row_ptr,
                                                                  const int32_t* __restrict__ cols, int64_t nnz,
                                                                  const int64_t* __restrict__ order, int64_t n_rows,
                                                                  const int64_t* __restrict__ new_ptr,
                                                                  int32_t* __restrict__ new_cols, int* bad) {
    const int lane = threadIdx.x & 31;
    const int64_t n_warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t p = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; p < n_rows; p += n_warps) {
        const int64_t src = order[p];
        if (src < 0 || src >= n_rows) {
            if (lane == 0) atomicExch(bad, 1);
            continue;
        }
        const int64_t e0 = row_ptr[src], n = row_ptr[src + 1] - e0, d0 = new_ptr[p];
        if (e0 < 0 || n < 0 || e0 + n > nnz || d0 < 0 || d0 + n > nnz) {
            if (lane == 0) atomicExch(bad, 1);
            continue;
        }
        for (int64_t i = lane; i < n; i += 32) new_cols[d0 + i] = cols[e0 + i];
    }
}

// occ[c][ow], bit b: tile t = 64 ow + b of column c (words [32 t, 32 t + 32) below n_words) holds a set bit
// (the occupancy of gpu/kernels/occupancy.py:37-58). One warp per occupancy word, 32 steps of 16-byte loads:
// lanes 0-15 read tile 2 i of step i, lanes 16-31 tile 2 i + 1.
__global__ void __launch_bounds__(IN_THREADS) tile_occupancy_kernel(const uint64_t* __restrict__ bv, int64_t n_cols,
                                                                    int64_t n_words, int64_t ld,
                                                                    uint64_t* __restrict__ occ, int64_t occ_ld) {
    const int lane = threadIdx.x & 31;
    const int64_t n_warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const int64_t total = n_cols * occ_ld;
    for (int64_t u = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; u < total; u += n_warps) {
        const int64_t c = u / occ_ld, ow = u - c * occ_ld;
        const uint64_t* col = bv + c * ld;
        const int64_t w0 = ow * (64 * ETM_OCC_TILE_WORDS) + 2 * lane;
        uint64_t bits = 0;
#pragma unroll 8
        for (int i = 0; i < 32; i++) {
            const int64_t w = w0 + 64 * i;
            uint64_t x = 0;
            if (w + 1 < n_words) {
                const ulonglong2 v = __ldg(reinterpret_cast<const ulonglong2*>(col + w));
                x = v.x | v.y;
            } else if (w < n_words) {
                x = __ldg(col + w);
            }
            const unsigned b = __ballot_sync(0xffffffffu, x != 0ULL);
            bits |= (uint64_t)((b & 0xFFFFu) != 0u) << (2 * i);
            bits |= (uint64_t)((b >> 16) != 0u) << (2 * i + 1);
        }
        if (lane == 0) occ[u] = bits;
    }
}

int in_grid(int64_t units_of_warps) {
    const int64_t cap = (int64_t)max(1, sm_count()) * 8;
    return (int)max64(1, min64(cap, ceil_div<int64_t>(units_of_warps, IN_THREADS / 32)));
}

}  // namespace

extern "C" int etm_row_order_keys(const int64_t* row_ptr, const int32_t* cols, int64_t n_rows,
                                  const int32_t* rank_of_col, int64_t n_cols, int64_t* key_hi, int64_t* key_lo,
                                  void* stream) {
    ETM_REQUIRE(n_rows >= 0 && n_cols >= 0, ETM_EINVAL, "etm_row_order_keys: negative size");
    if (n_rows == 0) return ETM_OK;
    row_order_keys_kernel<<<in_grid(n_rows), IN_THREADS, 0, as_stream(stream)>>>(row_ptr, cols, n_rows, rank_of_col,
                                                                                 n_cols, key_hi, key_lo);
    ETM_LAUNCHED("row_order_keys");
    return ETM_OK;
}

extern "C" int etm_permute_rows(const int64_t* row_ptr, const int32_t* cols, int64_t nnz, const int64_t* order,
                                int64_t n_rows, const int64_t* new_row_ptr, int32_t* new_cols, int32_t* status,
                                void* stream) {
    ETM_REQUIRE(n_rows >= 0 && nnz >= 0, ETM_EINVAL, "etm_permute_rows: negative size");
    ETM_REQUIRE(status != nullptr, ETM_EINVAL, "etm_permute_rows: status is required");
    cudaStream_t s = as_stream(stream);
    ETM_CUDA(cudaMemsetAsync(status, 0, sizeof(int32_t), s));
    if (n_rows == 0) return ETM_OK;
    permute_rows_kernel<<<in_grid(n_rows), IN_THREADS, 0, s>>>(row_ptr, cols, nnz, order, n_rows, new_row_ptr,
                                                               new_cols, reinterpret_cast<int*>(status));
    ETM_LAUNCHED("permute_rows");
    return ETM_OK;
}

extern "C" int etm_tile_occupancy(const uint64_t* bv, int64_t n_cols, int64_t n_words, int64_t ld, uint64_t* occ,
                                  int64_t occ_ld, void* stream) {
    ETM_REQUIRE(n_cols >= 0 && n_words >= 0 && ld >= n_words, ETM_EINVAL, "etm_tile_occupancy: bad sizes");
    ETM_REQUIRE(ld % 2 == 0 && (reinterpret_cast<uintptr_t>(bv) & 15) == 0, ETM_EINVAL,
                "etm_tile_occupancy: bv must be 16-byte aligned with an even ld");
    const int64_t tiles = ceil_div<int64_t>(n_words, ETM_OCC_TILE_WORDS);
    ETM_REQUIRE(occ_ld >= ceil_div<int64_t>(tiles, 64) && occ_ld >= 1, ETM_EINVAL,
                "etm_tile_occupancy: occ_ld %lld < ceil(tiles / 64)", (long long)occ_ld);
    if (n_cols == 0) return ETM_OK;
    tile_occupancy_kernel<<<in_grid(n_cols * occ_ld), IN_THREADS, 0, as_stream(stream)>>>(bv, n_cols, n_words, ld, occ,
                                                                                         occ_ld);
    ETM_LAUNCHED("tile_occupancy");
    return ETM_OK;
}
