// The device input layer: the item coding of a transaction CSR without sorting (a presence bitmap over the
// id span ranks every id; rows are checked to be canonical; a histogram of the ranks gives the supports),
// the lex row order (sort keys that gather the rows sharing their most frequent columns, and the CSR
// permuted into that order), and the tile occupancy (per column one bit per 32-word tile holding a row of
// it, which lets the prefix and per-candidate kernels skip tiles).
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
// (the occupancy of gpu/kernels/occupancy.py:37-58). One warp per occupancy word, 32 steps of two words per
// lane: lanes 0-15 read tile 2 i of step i, lanes 16-31 tile 2 i + 1; one 16-byte load per lane when every
// column starts 16-byte aligned (VEC), else two 8-byte loads.
template <bool VEC>
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
                if (VEC) {
                    const ulonglong2 v = __ldg(reinterpret_cast<const ulonglong2*>(col + w));
                    x = v.x | v.y;
                } else {
                    x = __ldg(col + w) | __ldg(col + w + 1);
                }
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

// ---- item coding of a transaction CSR: ids to ranks among the distinct ids, without sorting ----

// Bit (id - lo) of the bitmap for every entry with lo <= id < lo + span; an id outside sets *bad. A bit already
// set is not OR-ed again, so a frequent id costs a read, not an atomic.
__global__ void __launch_bounds__(IN_THREADS) id_presence_kernel(const int64_t* __restrict__ ids, int64_t nnz,
                                                                 int64_t lo, int64_t span, uint32_t* bitmap,
                                                                 int* bad) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < nnz; e += stride) {
        const uint64_t v = (uint64_t)ids[e] - (uint64_t)lo;
        if (v >= (uint64_t)span) {
            atomicExch(bad, 1);
            continue;
        }
        const unsigned bit = 1u << (v & 31);
        unsigned* w = bitmap + (v >> 5);
        if ((__ldcg(w) & bit) == 0u) atomicOr(w, bit);
    }
}

// One block: word_rank[w] = set bits in words [0, w) of the bitmap, word_rank[n] = the distinct ids.
__global__ void __launch_bounds__(1024) bitmap_rank_kernel(const uint32_t* __restrict__ bitmap, int64_t n,
                                                           int64_t* __restrict__ word_rank) {
    int64_t carry = 0;  // the same in every thread
    for (int64_t w0 = 0; w0 < n; w0 += blockDim.x) {
        const int64_t w = w0 + threadIdx.x;
        int64_t total;
        const int64_t ex = block_exclusive_scan(w < n ? __popc(bitmap[w]) : 0, &total);
        if (w < n) word_rank[w] = carry + ex;
        carry += total;
    }
    if (threadIdx.x == 0) word_rank[n] = carry;
}

// One warp per row: each entry's code, the rank of its id among the distinct ids (word_rank[w] plus the set
// bits below it in word w), and the canonical check: a row whose codes do not strictly ascend (an unsorted
// row, or a repeated id) sets *noncanonical.
__global__ void __launch_bounds__(IN_THREADS) code_rows_kernel(const int64_t* __restrict__ row_ptr,
                                                               const int64_t* __restrict__ ids, int64_t n_rows,
                                                               int64_t lo, int64_t span,
                                                               const uint32_t* __restrict__ bitmap,
                                                               const int64_t* __restrict__ word_rank,
                                                               int32_t* __restrict__ codes, int* noncanonical) {
    const int lane = threadIdx.x & 31;
    const int64_t n_warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < n_rows; r += n_warps) {
        const int64_t e0 = row_ptr[r], e1 = row_ptr[r + 1];
        int64_t carry = -1;  // the code of the previous (full) chunk's last entry
        bool bad = false;
        for (int64_t base = e0; base < e1; base += 32) {
            const int64_t e = base + lane;
            int64_t code = -1;
            if (e < e1) {
                const uint64_t v = (uint64_t)ids[e] - (uint64_t)lo;
                if (v < (uint64_t)span) {
                    const uint32_t word = bitmap[v >> 5];
                    code = word_rank[v >> 5] + __popc(word & ((1u << (v & 31)) - 1u));
                }
                codes[e] = (int32_t)code;
            }
            int64_t prev = __shfl_up_sync(0xffffffffu, code, 1);
            if (lane == 0) prev = carry;
            if (e < e1 && (code < 0 || (e > e0 && code <= prev))) bad = true;
            carry = __shfl_sync(0xffffffffu, code, 31);
        }
        if (__any_sync(0xffffffffu, bad) && lane == 0) atomicExch(noncanonical, 1);
    }
}

constexpr int HIST_SMEM_BINS = 12288;  // 48 KB of block-private counters

// Occurrences of each code in [0, n_bins) (others ignored): block-private shared counters when the bins fit,
// added to the global counts once per non-zero bin; global atomics otherwise.
template <bool SMEM>
__global__ void __launch_bounds__(IN_THREADS) code_histogram_kernel(const int32_t* __restrict__ codes, int64_t nnz,
                                                                    int64_t n_bins,
                                                                    unsigned long long* __restrict__ counts) {
    extern __shared__ uint32_t hist[];
    if (SMEM) {
        for (int64_t i = threadIdx.x; i < n_bins; i += blockDim.x) hist[i] = 0u;
        __syncthreads();
    }
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < nnz; e += stride) {
        const int32_t c = codes[e];
        if (c < 0 || c >= n_bins) continue;
        if (SMEM) atomicAdd(hist + c, 1u);
        else atomicAdd(counts + c, 1ULL);
    }
    if (SMEM) {
        __syncthreads();
        for (int64_t i = threadIdx.x; i < n_bins; i += blockDim.x)
            if (hist[i] != 0u) atomicAdd(counts + i, (unsigned long long)hist[i]);
    }
}

// The distinct ids in ascending order: lo + 32 w + b for every set bit b of word w, at out[word_rank[w]] on.
__global__ void __launch_bounds__(IN_THREADS) bitmap_values_kernel(const uint32_t* __restrict__ bitmap, int64_t n,
                                                                   const int64_t* __restrict__ word_rank, int64_t lo,
                                                                   int64_t* __restrict__ out) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t w = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; w < n; w += stride) {
        uint32_t x = bitmap[w];
        int64_t at = word_rank[w];
        while (x) {
            const int b = __ffs(x) - 1;
            out[at++] = lo + 32 * w + b;
            x &= x - 1u;
        }
    }
}

// One warp per row: its entries whose code maps to a column (0 <= code < lut_size and lut[code] >= 0).
__global__ void __launch_bounds__(IN_THREADS) kept_lengths_kernel(const int64_t* __restrict__ row_ptr,
                                                                  const int32_t* __restrict__ codes, int64_t n_rows,
                                                                  const int32_t* __restrict__ lut, int64_t lut_size,
                                                                  int64_t* __restrict__ out) {
    const int lane = threadIdx.x & 31;
    const int64_t n_warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < n_rows; r += n_warps) {
        unsigned n = 0;
        for (int64_t e = row_ptr[r] + lane; e < row_ptr[r + 1]; e += 32) {
            const int32_t c = codes[e];
            n += (c >= 0 && c < lut_size && lut[c] >= 0) ? 1u : 0u;
        }
        n = __reduce_add_sync(0xffffffffu, n);
        if (lane == 0) out[r] = n;
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
    ETM_REQUIRE((reinterpret_cast<uintptr_t>(bv) & 7) == 0, ETM_EINVAL, "etm_tile_occupancy: bv must be 8-byte aligned");
    const int64_t tiles = ceil_div<int64_t>(n_words, ETM_OCC_TILE_WORDS);
    ETM_REQUIRE(occ_ld >= ceil_div<int64_t>(tiles, 64) && occ_ld >= 1, ETM_EINVAL,
                "etm_tile_occupancy: occ_ld %lld < ceil(tiles / 64)", (long long)occ_ld);
    if (n_cols == 0) return ETM_OK;
    const int grid = in_grid(n_cols * occ_ld);
    if (ld % 2 == 0 && (reinterpret_cast<uintptr_t>(bv) & 15) == 0)
        tile_occupancy_kernel<true><<<grid, IN_THREADS, 0, as_stream(stream)>>>(bv, n_cols, n_words, ld, occ, occ_ld);
    else
        tile_occupancy_kernel<false><<<grid, IN_THREADS, 0, as_stream(stream)>>>(bv, n_cols, n_words, ld, occ, occ_ld);
    ETM_LAUNCHED("tile_occupancy");
    return ETM_OK;
}

extern "C" int etm_item_codes(const int64_t* row_ptr, const int64_t* ids, int64_t nnz, int64_t n_rows, int64_t lo,
                              int64_t span, uint32_t* bitmap, int64_t* word_rank, int32_t* codes, int32_t* status,
                              void* stream) {
    ETM_REQUIRE(nnz >= 0 && n_rows >= 0 && span >= 1 && span <= ETM_CODE_SPAN_MAX, ETM_EINVAL,
                "etm_item_codes: span %lld outside [1, 2^26] or negative size", (long long)span);
    ETM_REQUIRE(status != nullptr, ETM_EINVAL, "etm_item_codes: status is required");
    cudaStream_t s = as_stream(stream);
    const int64_t n_w = ceil_div<int64_t>(span, 32);
    ETM_CUDA(cudaMemsetAsync(status, 0, 2 * sizeof(int32_t), s));
    ETM_CUDA(cudaMemsetAsync(bitmap, 0, (size_t)n_w * 4, s));
    int* st = reinterpret_cast<int*>(status);
    if (nnz > 0) {
        id_presence_kernel<<<(int)max64(1, min64((int64_t)max(1, sm_count()) * 8, ceil_div<int64_t>(nnz, IN_THREADS))),
                             IN_THREADS, 0, s>>>(ids, nnz, lo, span, bitmap, st);
        ETM_LAUNCHED("id_presence");
    }
    bitmap_rank_kernel<<<1, 1024, 0, s>>>(bitmap, n_w, word_rank);
    ETM_LAUNCHED("bitmap_rank");
    if (n_rows > 0) {
        code_rows_kernel<<<in_grid(n_rows), IN_THREADS, 0, s>>>(row_ptr, ids, n_rows, lo, span, bitmap, word_rank,
                                                               codes, st + 1);
        ETM_LAUNCHED("code_rows");
    }
    return ETM_OK;
}

extern "C" int etm_code_histogram(const int32_t* codes, int64_t nnz, int64_t n_bins, int64_t* counts, void* stream) {
    ETM_REQUIRE(nnz >= 0 && n_bins >= 0, ETM_EINVAL, "etm_code_histogram: negative size");
    cudaStream_t s = as_stream(stream);
    if (n_bins == 0) return ETM_OK;
    ETM_CUDA(cudaMemsetAsync(counts, 0, (size_t)n_bins * 8, s));
    if (nnz == 0) return ETM_OK;
    auto* out = reinterpret_cast<unsigned long long*>(counts);
    const int grid = (int)max64(1, min64((int64_t)max(1, sm_count()) * 4, ceil_div<int64_t>(nnz, IN_THREADS)));
    if (n_bins <= HIST_SMEM_BINS) {
        code_histogram_kernel<true><<<grid, IN_THREADS, (size_t)n_bins * 4, s>>>(codes, nnz, n_bins, out);
    } else {
        code_histogram_kernel<false><<<grid, IN_THREADS, 0, s>>>(codes, nnz, n_bins, out);
    }
    ETM_LAUNCHED("code_histogram");
    return ETM_OK;
}

extern "C" int etm_bitmap_values(const uint32_t* bitmap, int64_t span, const int64_t* word_rank, int64_t lo,
                                 int64_t* out, void* stream) {
    ETM_REQUIRE(span >= 1 && span <= ETM_CODE_SPAN_MAX, ETM_EINVAL, "etm_bitmap_values: span out of range");
    const int64_t n_w = ceil_div<int64_t>(span, 32);
    bitmap_values_kernel<<<(int)min64((int64_t)max(1, sm_count()) * 8, ceil_div<int64_t>(n_w, IN_THREADS)), IN_THREADS,
                           0, as_stream(stream)>>>(bitmap, n_w, word_rank, lo, out);
    ETM_LAUNCHED("bitmap_values");
    return ETM_OK;
}

extern "C" int etm_kept_lengths(const int64_t* row_ptr, const int32_t* codes, int64_t n_rows, const int32_t* lut,
                                int64_t lut_size, int64_t* out_lengths, void* stream) {
    ETM_REQUIRE(n_rows >= 0 && lut_size >= 0, ETM_EINVAL, "etm_kept_lengths: negative size");
    if (n_rows == 0) return ETM_OK;
    kept_lengths_kernel<<<in_grid(n_rows), IN_THREADS, 0, as_stream(stream)>>>(row_ptr, codes, n_rows, lut, lut_size,
                                                                              out_lengths);
    ETM_LAUNCHED("kept_lengths");
    return ETM_OK;
}
