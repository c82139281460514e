// Device-wide ordered scan-and-apply, the building block of every stream
// compaction here (survivors of a candidate chunk, prefix-group runs, kept
// rows). Three launches, no atomics, so the output order is the input order:
//
//   1. each block sums val(i) over its SCAN_TILE elements -> partial[b]
//   2. one block turns partial[] into exclusive block offsets, adds the base
//      *acc (if given) and writes the new running total back to *acc
//   3. each block rescans its elements and calls act(i, offset) for every
//      element with val(i) > 0 (offset = base + elements before it)
//
// The element count `n` is a host upper bound; val() returns 0 beyond the
// live range. Workspace: scan_workspace_words(n) int64 words.
#pragma once

#include "etm_common.cuh"

namespace etm {

constexpr int SCAN_THREADS = 512;
constexpr int SCAN_ITEMS = 8;
constexpr int64_t SCAN_TILE = (int64_t)SCAN_THREADS * SCAN_ITEMS;

inline int64_t scan_blocks(int64_t n) { return n <= 0 ? 1 : ceil_div<int64_t>(n, SCAN_TILE); }
inline int64_t scan_workspace_words(int64_t n) { return scan_blocks(n) + 2; }

template <class Val>
__global__ void __launch_bounds__(SCAN_THREADS) scan_partials_kernel(int64_t n, Val val, int64_t* partial) {
    const int64_t base = (int64_t)blockIdx.x * SCAN_TILE;
    int64_t s = 0;
#pragma unroll
    for (int t = 0; t < SCAN_ITEMS; t++) {
        int64_t i = base + (int64_t)t * SCAN_THREADS + threadIdx.x;
        if (i < n) s += val(i);
    }
    int64_t total;
    block_exclusive_scan(s, &total);
    if (threadIdx.x == 0) partial[blockIdx.x] = total;
}

// One block: exclusive scan of partial[0..nb) in place; base = *acc (or 0);
// partial[nb] = base (kept for phase 3), *acc = base + sum.
static __global__ void __launch_bounds__(1024) scan_offsets_kernel(int64_t nb, int64_t* partial, int64_t* acc) {
    __shared__ int64_t carry;
    if (threadIdx.x == 0) carry = acc ? *acc : 0;
    __syncthreads();
    const int64_t base = carry;
    for (int64_t c0 = 0; c0 < nb; c0 += blockDim.x) {
        int64_t i = c0 + threadIdx.x;
        int64_t v = i < nb ? partial[i] : 0;
        int64_t total;
        int64_t ex = block_exclusive_scan(v, &total);
        if (i < nb) partial[i] = carry + ex;
        __syncthreads();
        if (threadIdx.x == 0) carry += total;
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        partial[nb] = base;
        if (acc) *acc = carry;
    }
}

template <class Val, class Act>
__global__ void __launch_bounds__(SCAN_THREADS) scan_apply_kernel(int64_t n, Val val, Act act, const int64_t* partial) {
    const int64_t base = (int64_t)blockIdx.x * SCAN_TILE;
    // Each thread owns SCAN_ITEMS consecutive elements so that offsets follow element order.
    const int64_t first = base + (int64_t)threadIdx.x * SCAN_ITEMS;
    int64_t v[SCAN_ITEMS];
    int64_t s = 0;
#pragma unroll
    for (int t = 0; t < SCAN_ITEMS; t++) {
        int64_t i = first + t;
        v[t] = i < n ? val(i) : 0;
        s += v[t];
    }
    int64_t total;
    int64_t off = partial[blockIdx.x] + block_exclusive_scan(s, &total);
#pragma unroll
    for (int t = 0; t < SCAN_ITEMS; t++) {
        if (v[t] > 0) act(first + t, off);
        off += v[t];
    }
}

// Runs the three phases on `stream`. `acc` (device, nullable) is the running base/total.
template <class Val, class Act>
int scan_apply(int64_t n, Val val, Act act, int64_t* ws, int64_t ws_words, int64_t* acc, cudaStream_t stream) {
    const int64_t nb = scan_blocks(n);
    ETM_REQUIRE(ws_words >= nb + 2, ETM_ENOSPACE, "scan workspace too small: %lld words, need %lld",
                (long long)ws_words, (long long)(nb + 2));
    ETM_REQUIRE(nb < (1LL << 31), ETM_EINVAL, "scan over %lld elements is too large", (long long)n);
    scan_partials_kernel<<<(unsigned)nb, SCAN_THREADS, 0, stream>>>(n, val, ws);
    ETM_LAUNCHED("scan_partials");
    scan_offsets_kernel<<<1, 1024, 0, stream>>>(nb, ws, acc);
    ETM_LAUNCHED("scan_offsets");
    scan_apply_kernel<<<(unsigned)nb, SCAN_THREADS, 0, stream>>>(n, val, act, ws);
    ETM_LAUNCHED("scan_apply");
    return ETM_OK;
}

}  // namespace etm
