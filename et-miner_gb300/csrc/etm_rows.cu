// Row-wise K=2 counting: each transaction adds 1 to every pair of its
// frequent columns. The reference picks this kernel when its rows are short
// against the pair space (count_pairs_k2_rows, gpu/kernels/_src/pairs_k2_rows.cu:54;
// dispatch gpu/row_split_chunks.py:124-142): the work is sum over rows of
// C(len, 2) atomic increments instead of pairs x words AND+popcounts.
//
// One warp per row: the row's entries are mapped to generator indices (a
// lookup table, -1 for columns that do not generate), compacted in order into
// the warp's slice of shared memory with ballots, and the warp's lanes walk
// the row's C(L, 2) pairs, adding 1 at the pair's lexicographic slot in the
// dense K=2 count array (the slot etm_level_compact reads). Rows longer than
// the shared slice fall back to reading their entries from global memory.
#include "etm_common.cuh"

namespace {

using namespace etm;

constexpr int RT = 256;
constexpr int RW = RT / 32;
constexpr int ROW_SLICE = 512;  // generator ids per warp held in shared memory

__device__ __forceinline__ int32_t gen_of(const int32_t* __restrict__ cols, const int32_t* __restrict__ lut,
                                          int64_t lut_size, int64_t e) {
    const int32_t c = __ldg(cols + e);
    if (lut == nullptr) return c;
    return (c >= 0 && c < lut_size) ? __ldg(lut + c) : -1;
}

__global__ void __launch_bounds__(RT) pairs_rows_kernel(const int64_t* __restrict__ row_ptr,
                                                        const int32_t* __restrict__ cols, int64_t nnz,
                                                        const int32_t* __restrict__ lut, int64_t lut_size,
                                                        int64_t n_rows, int64_t n_gen, int32_t* __restrict__ out) {
    __shared__ int32_t slice[RW][ROW_SLICE];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int32_t* ids = slice[wid];
    const int64_t n_warps = ((int64_t)gridDim.x * RT) >> 5;
    for (int64_t r = ((int64_t)blockIdx.x * RT + threadIdx.x) >> 5; r < n_rows; r += n_warps) {
        const int64_t e0 = max64(0, row_ptr[r]), e1 = min64(row_ptr[r + 1], nnz);
        const int64_t len = e1 - e0;
        if (len < 2) continue;
        if (len <= ROW_SLICE) {
            // Compact the row's generator ids (ascending, as the row's columns are) into shared memory.
            int L = 0;
            for (int64_t b = 0; b < len; b += 32) {
                const int64_t e = e0 + b + lane;
                const int32_t g = e < e1 ? gen_of(cols, lut, lut_size, e) : -1;
                const unsigned keep = __ballot_sync(0xffffffffu, g >= 0);
                if (g >= 0) ids[L + __popc(keep & ((1u << lane) - 1u))] = g;
                L += __popc(keep);
            }
            __syncwarp();
            const int64_t P = pairs_of(L);
            for (int64_t p = lane; p < P; p += 32) {
                int64_t i, j;
                tri_decode(p, L, &i, &j);
                atomicAdd(out + tri_index(ids[i], ids[j], n_gen), 1);
            }
            __syncwarp();
        } else {
            // A long row: pairs straight from global memory (rare; rows above ROW_SLICE entries).
            for (int64_t a = e0 + lane; a < e1; a += 32) {
                const int32_t ga = gen_of(cols, lut, lut_size, a);
                if (ga < 0) continue;
                for (int64_t b = a + 1; b < e1; b++) {
                    const int32_t gb = gen_of(cols, lut, lut_size, b);
                    if (gb >= 0) atomicAdd(out + tri_index(ga, gb, n_gen), 1);
                }
            }
        }
    }
}

}  // namespace

extern "C" int etm_pair_counts_rows(const int64_t* row_ptr, const int32_t* cols, int64_t nnz, const int32_t* lut,
                                    int64_t lut_size, int64_t n_rows, int64_t n_gen, int32_t* out_counts,
                                    void* stream) {
    ETM_REQUIRE(n_rows >= 0 && n_gen >= 0 && nnz >= 0, ETM_EINVAL, "etm_pair_counts_rows: negative size");
    cudaStream_t s = as_stream(stream);
    const int64_t n_pairs = pairs_of(n_gen);
    if (n_pairs == 0) return ETM_OK;
    ETM_CUDA(cudaMemsetAsync(out_counts, 0, (size_t)n_pairs * sizeof(int32_t), s));
    if (n_rows == 0 || nnz == 0) return ETM_OK;
    const int64_t blocks = min64(ceil_div<int64_t>(n_rows, RW), (int64_t)max(1, sm_count()) * 16);
    pairs_rows_kernel<<<(unsigned)blocks, RT, 0, s>>>(row_ptr, cols, nnz, lut, lut_size, n_rows, n_gen, out_counts);
    ETM_LAUNCHED("pairs_rows");
    return ETM_OK;
}
