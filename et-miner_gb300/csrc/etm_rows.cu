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
//
// Row-wise K=3 (count_k3_rows, gpu/kernels/_src/k3_rows.cu:50-140; dispatch
// gpu/row_split_chunks.py:145-159): a row adds 1 to every K=3 candidate whose
// three items it holds. Here the candidates are laid out by prefix group (the
// engine's K=3 layout: group u, members v_0 < v_1 < ..., candidate (u, v_i,
// v_j) at cand_off[u] + tri_index(i, j, m_u)), so per row and per item u of
// the row that prefixes a group, the warp looks up which later items of the
// row are members of u's group (binary search in the group's sorted members),
// compacts their member indices, and adds 1 at each of their pairs' slots.
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

__device__ __forceinline__ int64_t member_index(const int32_t* __restrict__ gen_rows, int64_t first, int64_t m,
                                                int32_t v) {
    // gen_rows[(first + i) * 2 + 1], i < m, ascending: the index of v, or -1.
    int64_t lo = 0, hi = m;
    while (lo < hi) {
        const int64_t mid = (lo + hi) >> 1;
        const int32_t x = __ldg(gen_rows + (first + mid) * 2 + 1);
        if (x < v) lo = mid + 1;
        else hi = mid;
    }
    return (lo < m && __ldg(gen_rows + (first + lo) * 2 + 1) == v) ? lo : -1;
}

__device__ __forceinline__ void add_counted(int32_t* __restrict__ out, const uint8_t* __restrict__ cls, int64_t t,
                                            int64_t n_cands) {
    if (t >= 0 && t < n_cands && (cls == nullptr || cls[t] == ETM_CAND_COUNT)) atomicAdd(out + t, 1);
}

__global__ void zero_counted_kernel(int32_t* __restrict__ out, const uint8_t* __restrict__ cls, int64_t n) {
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x)
        if (cls == nullptr || cls[t] == ETM_CAND_COUNT) out[t] = 0;
}

__global__ void __launch_bounds__(RT) triples_rows_kernel(const int64_t* __restrict__ row_ptr,
                                                          const int32_t* __restrict__ cols, int64_t nnz,
                                                          const int32_t* __restrict__ lut, int64_t lut_size,
                                                          int64_t n_rows, const int32_t* __restrict__ gen_rows,
                                                          const int32_t* __restrict__ grp_of, int64_t n_gen1,
                                                          const int64_t* __restrict__ grp_first,
                                                          const int32_t* __restrict__ grp_size,
                                                          const int64_t* __restrict__ cand_off, int64_t base,
                                                          int64_t n_cands, const uint8_t* __restrict__ cls,
                                                          int32_t* __restrict__ out) {
    __shared__ int32_t slice[RW][ROW_SLICE];
    __shared__ int32_t mem[RW][ROW_SLICE];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int32_t* ids = slice[wid];
    int32_t* mi = mem[wid];
    const int64_t n_warps = ((int64_t)gridDim.x * RT) >> 5;
    for (int64_t r = ((int64_t)blockIdx.x * RT + threadIdx.x) >> 5; r < n_rows; r += n_warps) {
        const int64_t e0 = max64(0, row_ptr[r]), e1 = min64(row_ptr[r + 1], nnz);
        const int64_t len = e1 - e0;
        if (len < 3) continue;
        if (len <= ROW_SLICE) {
            int L = 0;
            for (int64_t b = 0; b < len; b += 32) {
                const int64_t e = e0 + b + lane;
                const int32_t g = e < e1 ? gen_of(cols, lut, lut_size, e) : -1;
                const unsigned keep = __ballot_sync(0xffffffffu, g >= 0);
                if (g >= 0) ids[L + __popc(keep & ((1u << lane) - 1u))] = g;
                L += __popc(keep);
            }
            __syncwarp();
            for (int a = 0; a + 2 < L; a++) {
                const int32_t u = ids[a];
                const int32_t grp = (u >= 0 && u < n_gen1) ? __ldg(grp_of + u) : -1;
                if (grp < 0) continue;
                const int64_t first = grp_first[grp], m = grp_size[grp];
                const int64_t cb = cand_off[grp] - base;
                if (cb >= n_cands || cb + m * (m - 1) / 2 <= 0) continue;  // the group lies outside this range
                // Member indices of the row's later items in u's group, ascending.
                int c = 0;
                for (int b0 = a + 1; b0 < L; b0 += 32) {
                    const int b = b0 + lane;
                    const int64_t x = b < L ? member_index(gen_rows, first, m, ids[b]) : -1;
                    const unsigned keep = __ballot_sync(0xffffffffu, x >= 0);
                    if (x >= 0) mi[c + __popc(keep & ((1u << lane) - 1u))] = (int32_t)x;
                    c += __popc(keep);
                }
                __syncwarp();
                const int64_t P = pairs_of(c);
                for (int64_t p = lane; p < P; p += 32) {
                    int64_t i, j;
                    tri_decode(p, c, &i, &j);
                    add_counted(out, cls, cb + tri_index(mi[i], mi[j], m), n_cands);
                }
                __syncwarp();
            }
            __syncwarp();
        } else {
            // A long row: triples straight from global memory (rare; rows above ROW_SLICE entries).
            for (int64_t a = e0 + lane; a < e1; a += 32) {
                const int32_t u = gen_of(cols, lut, lut_size, a);
                const int32_t grp = (u >= 0 && u < n_gen1) ? __ldg(grp_of + u) : -1;
                if (grp < 0) continue;
                const int64_t first = grp_first[grp], m = grp_size[grp];
                const int64_t cb = cand_off[grp] - base;
                for (int64_t b = a + 1; b < e1; b++) {
                    const int32_t gb = gen_of(cols, lut, lut_size, b);
                    const int64_t i = gb >= 0 ? member_index(gen_rows, first, m, gb) : -1;
                    if (i < 0) continue;
                    for (int64_t c2 = b + 1; c2 < e1; c2++) {
                        const int32_t gc = gen_of(cols, lut, lut_size, c2);
                        const int64_t j = gc >= 0 ? member_index(gen_rows, first, m, gc) : -1;
                        if (j >= 0) add_counted(out, cls, cb + tri_index(i, j, m), n_cands);
                    }
                }
            }
        }
    }
}

}  // namespace

extern "C" int etm_triple_counts_rows(const int64_t* row_ptr, const int32_t* cols, int64_t nnz, const int32_t* lut,
                                      int64_t lut_size, int64_t n_rows, const int32_t* gen_rows,
                                      const int32_t* grp_of, int64_t n_gen1, const int64_t* grp_first,
                                      const int32_t* grp_size, const int64_t* cand_off, int64_t chunk_base,
                                      int64_t n_cands, const uint8_t* cls, int32_t* out_counts, void* stream) {
    ETM_REQUIRE(n_rows >= 0 && nnz >= 0 && n_cands >= 0 && n_gen1 >= 0, ETM_EINVAL,
                "etm_triple_counts_rows: negative size");
    cudaStream_t s = as_stream(stream);
    if (n_cands == 0) return ETM_OK;
    const int grid0 = (int)min64(ceil_div<int64_t>(n_cands, 256), (int64_t)max(1, sm_count()) * 8);
    zero_counted_kernel<<<grid0, 256, 0, s>>>(out_counts, cls, n_cands);
    ETM_LAUNCHED("zero_counted");
    if (n_rows == 0 || nnz == 0) return ETM_OK;
    const int64_t blocks = min64(ceil_div<int64_t>(n_rows, RW), (int64_t)max(1, sm_count()) * 8);
    triples_rows_kernel<<<(unsigned)blocks, RT, 0, s>>>(row_ptr, cols, nnz, lut, lut_size, n_rows, gen_rows, grp_of,
                                                        n_gen1, grp_first, grp_size, cand_off, chunk_base, n_cands,
                                                        cls, out_counts);
    ETM_LAUNCHED("triples_rows");
    return ETM_OK;
}

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
