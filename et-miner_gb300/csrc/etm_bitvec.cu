// Column bitvectors: the CSR -> bitvector build, K=1 popcounts, the padded
// copy of the frequent columns, and the hash-defined Bernoulli generator.
//
// These kernels are HBM-bound integer work: coalesced 16-byte accesses,
// grids sized to fill all SMs, no per-bit host work.
#include "etm_common.cuh"

namespace {

using namespace etm;

constexpr int BUILD_THREADS = 256;
constexpr int BUILD_ROWS = 256;  // rows per block: 4 bitvector words per column

// One block per BUILD_ROWS consecutive rows. Their entries are contiguous in
// the CSR, so the id reads are coalesced; each entry finds its row by binary
// search over the block's row_ptr slice in shared memory and ORs its bit into
// the column's word. Different rows of a block meet in a word only when they
// hold the same column, so the atomics rarely contend.
__global__ void __launch_bounds__(BUILD_THREADS) build_bitvecs_kernel(
    const int64_t* __restrict__ row_ptr, const int32_t* __restrict__ ids, int64_t nnz, const int32_t* __restrict__ lut,
    int64_t lut_size, int64_t n_rows, int64_t n_cols, int64_t ld, unsigned long long* __restrict__ out) {
    __shared__ int64_t ptr[BUILD_ROWS + 1];
    const int64_t r0 = (int64_t)blockIdx.x * BUILD_ROWS;
    const int nr = (int)min64(BUILD_ROWS, n_rows - r0);
    for (int t = threadIdx.x; t <= nr; t += blockDim.x) ptr[t] = row_ptr[r0 + t];
    __syncthreads();
    // Entries outside [0, nnz) are never read, whatever row_ptr holds.
    const int64_t e0 = max64(ptr[0], 0), e1 = min64(ptr[nr], nnz);
    for (int64_t e = e0 + threadIdx.x; e < e1; e += blockDim.x) {
        int lo = 0, hi = nr;  // ptr[lo] <= e < ptr[hi] when row_ptr is non-decreasing
        while (hi - lo > 1) {
            int mid = (lo + hi) >> 1;
            if (ptr[mid] <= e) lo = mid;
            else hi = mid;
        }
        if (e < ptr[lo] || e >= ptr[lo + 1]) continue;  // malformed row_ptr: skip the entry
        int64_t col = ids[e];
        if (lut) col = (col >= 0 && col < lut_size) ? (int64_t)lut[col] : -1;
        if (col < 0 || col >= n_cols) continue;
        const int64_t row = r0 + lo;
        atomicOr(out + col * ld + (row >> 6), 1ULL << (row & 63));
    }
}

// Shared-memory form for up to SMEM_BUILD_COLS columns: the block's 256 rows are 4 words of every column,
// held in shared memory as [word][column] (n_cols x 32 bytes); each warp takes whole rows (a row's entries are
// distinct columns, so a warp's ORs hit distinct words, spread over the banks), then the block writes each of
// its words once, 32 contiguous bytes per column. Every output word is written by exactly one block, so the
// output needs no zeroing first and no global atomics run.
constexpr int SMEM_BUILD_COLS = 3072;  // 96 KB of shared memory
__global__ void __launch_bounds__(BUILD_THREADS) build_bitvecs_smem_kernel(
    const int64_t* __restrict__ row_ptr, const int32_t* __restrict__ ids, int64_t nnz, const int32_t* __restrict__ lut,
    int64_t lut_size, int64_t n_rows, int64_t n_cols, int64_t ld, uint64_t* __restrict__ out) {
    extern __shared__ unsigned long long words[];  // [4][n_cols]
    __shared__ int64_t ptr[BUILD_ROWS + 1];
    const int64_t r0 = (int64_t)blockIdx.x * BUILD_ROWS;
    const int nr = (int)min64(BUILD_ROWS, n_rows - r0);
    for (int t = threadIdx.x; t <= nr; t += blockDim.x) ptr[t] = row_ptr[r0 + t];
    for (int64_t t = threadIdx.x; t < n_cols * 4; t += blockDim.x) words[t] = 0ULL;
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, n_warps = blockDim.x >> 5;
    for (int r = warp; r < nr; r += n_warps) {
        const int64_t b = max64(ptr[r], 0), e = min64(ptr[r + 1], nnz);
        unsigned long long* wq = words + (int64_t)(r >> 6) * n_cols;
        const unsigned long long bit = 1ULL << (r & 63);
        for (int64_t i = b + lane; i < e; i += 32) {
            int64_t col = ids[i];
            if (lut) col = (col >= 0 && col < lut_size) ? (int64_t)lut[col] : -1;
            if (col < 0 || col >= n_cols) continue;
            atomicOr(wq + col, bit);
        }
    }
    __syncthreads();
    const int64_t w0 = r0 >> 6;
    for (int64_t t = threadIdx.x; t < n_cols * 4; t += blockDim.x) {
        const int64_t col = t >> 2, q = t & 3;
        if (w0 + q < ld) out[col * ld + w0 + q] = words[q * n_cols + col];
    }
}

constexpr int POP_THREADS = 256;
constexpr int64_t POP_SEG_WORDS = 1 << 16;  // words per block: a column is split over several blocks

__global__ void __launch_bounds__(POP_THREADS) popcount_cols_kernel(const uint64_t* __restrict__ bv, int64_t n_cols,
                                                                    int64_t n_words, int64_t ld, int64_t n_seg,
                                                                    unsigned long long* __restrict__ out) {
    const int64_t col = blockIdx.x / n_seg;
    const int64_t seg = blockIdx.x % n_seg;
    const int64_t w0 = seg * POP_SEG_WORDS;
    const int64_t w1 = min(n_words, w0 + POP_SEG_WORDS);
    const uint64_t* p = bv + col * ld;
    unsigned s = 0;
    // 16-byte loads when the column start and w0 are 2-word aligned (ld even); else words.
    if ((ld & 1) == 0 && ((reinterpret_cast<uintptr_t>(bv) & 15) == 0)) {
        const int64_t v0 = w0 >> 1, v1 = w1 >> 1;
        const ulonglong2* q = reinterpret_cast<const ulonglong2*>(p);
        for (int64_t v = v0 + threadIdx.x; v < v1; v += blockDim.x) {
            ulonglong2 x = __ldg(q + v);
            s += __popcll(x.x) + __popcll(x.y);
        }
        if ((w1 & 1) && threadIdx.x == 0 && w1 - 1 >= w0) s += __popcll(__ldg(p + w1 - 1));
    } else {
        for (int64_t w = w0 + threadIdx.x; w < w1; w += blockDim.x) s += __popcll(__ldg(p + w));
    }
    s = __reduce_add_sync(0xffffffffu, s);
    __shared__ unsigned part[POP_THREADS / 32];
    if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
        unsigned v = threadIdx.x < POP_THREADS / 32 ? part[threadIdx.x] : 0;
        v = __reduce_add_sync(0xffffffffu, v);
        if (threadIdx.x == 0 && v) atomicAdd(out + col, (unsigned long long)v);
    }
}

constexpr int GATHER_THREADS = 256;

// One block per (column, 4096-word slab): 16-byte copies, zero fill past n_words.
__global__ void __launch_bounds__(GATHER_THREADS) gather_cols_kernel(const uint64_t* __restrict__ bv, int64_t ld,
                                                                     const int32_t* __restrict__ cols, int64_t n_words,
                                                                     uint64_t* __restrict__ out, int64_t out_ld,
                                                                     int64_t n_slab) {
    const int64_t f = blockIdx.x / n_slab;
    const int64_t slab = blockIdx.x % n_slab;
    const int64_t c = cols[f];
    const uint64_t* src = bv + c * ld;
    uint64_t* dst = out + f * out_ld;
    const int64_t w0 = slab * 4096, w1 = min(out_ld, w0 + 4096);
    const bool vec = ((ld & 1) == 0) && ((reinterpret_cast<uintptr_t>(bv) & 15) == 0);
    for (int64_t w = w0 + 2 * threadIdx.x; w < w1; w += 2 * blockDim.x) {
        ulonglong2 x;
        if (vec && w + 1 < n_words) {
            x = __ldg(reinterpret_cast<const ulonglong2*>(src + w));
        } else {
            x.x = w < n_words ? __ldg(src + w) : 0ULL;
            x.y = (w + 1) < n_words ? __ldg(src + w + 1) : 0ULL;
        }
        *reinterpret_cast<ulonglong2*>(dst + w) = x;
    }
}

__device__ __forceinline__ uint64_t bit_hash(uint64_t seed, uint64_t item, uint64_t row) {
    uint64_t x = seed ^ (item * 0x9E3779B97F4A7C15ULL) ^ (row * 0xD1B54A32D192ED03ULL);
    x ^= x >> 30;
    x *= 0xBF58476D1CE4E5B9ULL;
    x ^= x >> 27;
    x *= 0x94D049BB133111EBULL;
    x ^= x >> 31;
    return x;
}

// One thread per output word: 64 hashes, one coalesced store.
__global__ void synth_bernoulli_kernel(const uint64_t* __restrict__ thr, int32_t n_items, int64_t n_rows,
                                       uint64_t seed, uint64_t* __restrict__ out, int64_t ld) {
    const int64_t words = (n_rows + 63) >> 6;
    const int64_t total = (int64_t)n_items * ld;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t item = t / ld, w = t % ld;
        uint64_t word = 0;
        if (w < words) {
            const uint64_t th = thr[item];
            const int64_t r0 = w << 6;
            const int nb = (int)min64(64, n_rows - r0);
            for (int b = 0; b < nb; b++) word |= (uint64_t)(bit_hash(seed, item, r0 + b) < th) << b;
        }
        out[t] = word;
    }
}

// Rows built from planted patterns, one thread per row (the deep sparse workload's generator, defined by
// bit_hash so the host restates it exactly). Stream ids of the draws: 1 the length, 2 + p the p-th
// pattern, 64 + 16 p + q the keep draw of item q of pattern p, 4096 + t the t-th noise draw.
constexpr int SYN_MAX_LEN = 64;
__global__ void synth_patterns_kernel(const uint64_t* __restrict__ len_thr, int32_t n_len,
                                      const uint64_t* __restrict__ pat_thr, int32_t n_pat,
                                      const int64_t* __restrict__ pat_ptr, const int32_t* __restrict__ pat_items,
                                      int32_t per_row, uint64_t keep_thr, int32_t n_items, int64_t n_rows,
                                      uint64_t seed, unsigned long long* __restrict__ out, int64_t ld) {
    for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n_rows; r += (int64_t)gridDim.x * blockDim.x) {
        // Length: 1 + the number of cdf thresholds the draw reaches, at most n_len (<= SYN_MAX_LEN).
        const uint64_t hl = bit_hash(seed, 1, r);
        int len = 1;
        while (len - 1 < n_len && hl >= len_thr[len - 1]) ++len;
        int32_t items[SYN_MAX_LEN];
        int n = 0;
        for (int p = 0; p < per_row && n < len; p++) {
            const uint64_t hp = bit_hash(seed, 2 + p, r);
            int j = 0;
            while (j < n_pat - 1 && hp >= pat_thr[j]) ++j;
            for (int64_t q = pat_ptr[j]; q < pat_ptr[j + 1] && n < len; q++) {
                if (bit_hash(seed, 64 + 16 * p + (q - pat_ptr[j]), r) >= keep_thr) continue;
                const int32_t x = pat_items[q];
                bool dup = false;
                for (int e = 0; e < n; e++) dup |= items[e] == x;
                if (!dup) items[n++] = x;
            }
        }
        for (int t = 0; n < len && t < 65536; t++) {
            const int32_t x = (int32_t)(bit_hash(seed, 4096 + t, r) % (uint64_t)n_items);
            bool dup = false;
            for (int e = 0; e < n; e++) dup |= items[e] == x;
            if (!dup) items[n++] = x;
        }
        const unsigned long long bit = 1ULL << (r & 63);
        for (int e = 0; e < n; e++) atomicOr(out + (int64_t)items[e] * ld + (r >> 6), bit);
    }
}

}  // namespace

extern "C" int etm_synth_patterns(const uint64_t* len_thr, int32_t n_len, const uint64_t* pat_thr, int32_t n_pat,
                                  const int64_t* pat_ptr, const int32_t* pat_items, int32_t per_row,
                                  uint64_t keep_thr, int32_t n_items, int64_t n_rows, uint64_t seed, uint64_t* out_bv,
                                  int64_t ld, void* stream) {
    ETM_REQUIRE(ld >= (n_rows + 63) / 64 && n_items > 0 && n_rows >= 0, ETM_EINVAL, "etm_synth_patterns: bad sizes");
    ETM_REQUIRE(n_len >= 0 && n_len < SYN_MAX_LEN && n_pat >= 1 && per_row >= 0 && per_row <= 60, ETM_EINVAL,
                "etm_synth_patterns: n_len must be < %d, n_pat >= 1, per_row in 0..60", SYN_MAX_LEN);
    cudaStream_t s = as_stream(stream);
    ETM_CUDA(cudaMemsetAsync(out_bv, 0, (size_t)n_items * ld * 8, s));
    if (n_rows == 0) return ETM_OK;
    const int blocks = (int)min64(ceil_div<int64_t>(n_rows, 256), (int64_t)max(1, sm_count()) * 32);
    synth_patterns_kernel<<<blocks, 256, 0, s>>>(len_thr, n_len, pat_thr, n_pat, pat_ptr, pat_items, per_row, keep_thr,
                                                 n_items, n_rows, seed, reinterpret_cast<unsigned long long*>(out_bv),
                                                 ld);
    ETM_LAUNCHED("synth_patterns");
    return ETM_OK;
}

extern "C" int etm_build_bitvecs(const int64_t* row_ptr, const int32_t* ids, int64_t nnz, const int32_t* lut,
                                 int64_t lut_size, int64_t n_rows, int64_t n_cols, int64_t ld, uint64_t* out_bv,
                                 void* stream) {
    ETM_REQUIRE(n_rows >= 0 && n_cols >= 0, ETM_EINVAL, "etm_build_bitvecs: negative size");
    ETM_REQUIRE(ld >= (n_rows + 63) / 64, ETM_EINVAL, "etm_build_bitvecs: ld %lld < ceil(n_rows/64)", (long long)ld);
    ETM_REQUIRE(n_rows < (1LL << 31), ETM_EINVAL, "etm_build_bitvecs: n_rows must be < 2^31");
    cudaStream_t s = as_stream(stream);
    if (n_cols == 0 || ld == 0) return ETM_OK;
    const int64_t blocks = ceil_div<int64_t>(n_rows, BUILD_ROWS);
    if (n_cols <= SMEM_BUILD_COLS && n_rows > 0) {
        // The blocks write words [0, 4 blocks) of every column; words past that (a wider ld) are zeroed.
        if (ld > 4 * blocks)
            ETM_CUDA(cudaMemset2DAsync(out_bv + 4 * blocks, ld * 8, 0, (size_t)(ld - 4 * blocks) * 8, (size_t)n_cols, s));
        const size_t smem = (size_t)n_cols * 32;
        static bool configured = false;
        if (!configured) {
            ETM_CUDA(cudaFuncSetAttribute(build_bitvecs_smem_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          SMEM_BUILD_COLS * 32));
            configured = true;
        }
        build_bitvecs_smem_kernel<<<(unsigned)blocks, BUILD_THREADS, smem, s>>>(row_ptr, ids, nnz, lut, lut_size, n_rows,
                                                                               n_cols, ld, out_bv);
        ETM_LAUNCHED("build_bitvecs");
        return ETM_OK;
    }
    ETM_CUDA(cudaMemsetAsync(out_bv, 0, (size_t)n_cols * ld * 8, s));
    if (n_rows == 0) return ETM_OK;
    build_bitvecs_kernel<<<(unsigned)blocks, BUILD_THREADS, 0, s>>>(row_ptr, ids, nnz, lut, lut_size, n_rows, n_cols, ld,
                                                                    reinterpret_cast<unsigned long long*>(out_bv));
    ETM_LAUNCHED("build_bitvecs");
    return ETM_OK;
}

extern "C" int etm_popcount_cols(const uint64_t* bv, int64_t n_cols, int64_t n_words, int64_t ld,
                                 int64_t* out_counts, void* stream) {
    ETM_REQUIRE(n_cols >= 0 && n_words >= 0 && ld >= n_words, ETM_EINVAL, "etm_popcount_cols: bad sizes");
    cudaStream_t s = as_stream(stream);
    if (n_cols == 0) return ETM_OK;
    ETM_CUDA(cudaMemsetAsync(out_counts, 0, (size_t)n_cols * 8, s));
    if (n_words == 0) return ETM_OK;
    const int64_t n_seg = ceil_div<int64_t>(n_words, POP_SEG_WORDS);
    ETM_REQUIRE(n_cols * n_seg < (1LL << 31), ETM_EINVAL, "etm_popcount_cols: too many blocks");
    popcount_cols_kernel<<<(unsigned)(n_cols * n_seg), POP_THREADS, 0, s>>>(
        bv, n_cols, n_words, ld, n_seg, reinterpret_cast<unsigned long long*>(out_counts));
    ETM_LAUNCHED("popcount_cols");
    return ETM_OK;
}

extern "C" int etm_gather_cols(const uint64_t* bv, int64_t ld, const int32_t* cols, int32_t n_f, int64_t n_words,
                               uint64_t* out, int64_t out_ld, void* stream) {
    ETM_REQUIRE(out_ld % 32 == 0 && out_ld >= n_words, ETM_EINVAL, "etm_gather_cols: out_ld must be a multiple of 32 >= n_words");
    ETM_REQUIRE((reinterpret_cast<uintptr_t>(out) & 15) == 0, ETM_EINVAL, "etm_gather_cols: out must be 16-byte aligned");
    if (n_f <= 0 || out_ld == 0) return ETM_OK;
    const int64_t n_slab = ceil_div<int64_t>(out_ld, 4096);
    ETM_REQUIRE((int64_t)n_f * n_slab < (1LL << 31), ETM_EINVAL, "etm_gather_cols: too many blocks");
    gather_cols_kernel<<<(unsigned)(n_f * n_slab), GATHER_THREADS, 0, as_stream(stream)>>>(bv, ld, cols, n_words, out,
                                                                                         out_ld, n_slab);
    ETM_LAUNCHED("gather_cols");
    return ETM_OK;
}

extern "C" int etm_synth_bernoulli(const uint64_t* thresholds, int32_t n_items, int64_t n_rows, uint64_t seed,
                                   uint64_t* out_bv, int64_t ld, void* stream) {
    ETM_REQUIRE(ld >= (n_rows + 63) / 64 && n_items >= 0, ETM_EINVAL, "etm_synth_bernoulli: bad sizes");
    if (n_items == 0 || ld == 0) return ETM_OK;
    const int blocks = 4 * max(1, sm_count()) * 8;
    synth_bernoulli_kernel<<<blocks, 256, 0, as_stream(stream)>>>(thresholds, n_items, n_rows, seed, out_bv, ld);
    ETM_LAUNCHED("synth_bernoulli");
    return ETM_OK;
}
