// Shared device/host helpers of libetm_gb300: status codes, the last-error
// message, launch checks, warp/block scans and the bitvector conventions.
//
// Conventions (the reference's bitvecs= contract, core/apriori.py:409-413):
//   column c of a bitvector array is a row of `ld` uint64 words; bit r % 64 of
//   word r / 64 is set when transaction r holds column c; bits past N are 0.
//   Level rows are int32 column indices, ascending within a row, rows in
//   strictly ascending lexicographic order; counts are int32 (N < 2^31).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>

#include <string>

#include "etm.h"

namespace etm {

void set_error(const char* fmt, ...);
const char* last_error();

#define ETM_REQUIRE(cond, code, ...)        \
    do {                                    \
        if (!(cond)) {                      \
            ::etm::set_error(__VA_ARGS__);  \
            return (code);                  \
        }                                   \
    } while (0)

#define ETM_CUDA(call)                                                                       \
    do {                                                                                     \
        cudaError_t e_ = (call);                                                             \
        if (e_ != cudaSuccess) {                                                             \
            ::etm::set_error("%s:%d %s: %s", __FILE__, __LINE__, #call, cudaGetErrorString(e_)); \
            return ETM_ECUDA;                                                                \
        }                                                                                    \
    } while (0)

#define ETM_LAUNCHED(name)                                                                   \
    do {                                                                                     \
        cudaError_t e_ = cudaGetLastError();                                                 \
        if (e_ != cudaSuccess) {                                                             \
            ::etm::set_error("launch of %s failed: %s", name, cudaGetErrorString(e_));       \
            return ETM_ECUDA;                                                                \
        }                                                                                    \
    } while (0)

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

int sm_count();

template <typename T>
__host__ __device__ inline T ceil_div(T a, T b) { return (a + b - 1) / b; }

__host__ __device__ inline int64_t min64(int64_t a, int64_t b) { return a < b ? a : b; }
__host__ __device__ inline int64_t max64(int64_t a, int64_t b) { return a > b ? a : b; }

// Number of candidates of a prefix group with m members: C(m, 2).
__host__ __device__ inline int64_t pairs_of(int64_t m) { return m * (m - 1) / 2; }

// Lexicographic (i-major) index of pair (i, j), i < j < m, among C(m, 2).
__host__ __device__ inline int64_t tri_index(int64_t i, int64_t j, int64_t m) {
    return i * (2 * m - i - 1) / 2 + (j - i - 1);
}

// Inverse of tri_index: the pair (i, j) at lexicographic position t of C(m, 2).
__device__ inline void tri_decode(int64_t t, int64_t m, int64_t* pi, int64_t* pj) {
    // Row i starts at S(i) = i*(2m-i-1)/2. Solve with doubles, then correct.
    double b = 2.0 * (double)m - 1.0;
    double disc = b * b - 8.0 * (double)t;
    int64_t i = (int64_t)((b - sqrt(disc > 0 ? disc : 0.0)) * 0.5);
    if (i < 0) i = 0;
    if (i > m - 2) i = m - 2;
    while (i > 0 && i * (2 * m - i - 1) / 2 > t) --i;
    while (i < m - 2 && (i + 1) * (2 * m - i - 2) / 2 <= t) ++i;
    int64_t start = i * (2 * m - i - 1) / 2;
    *pi = i;
    *pj = i + 1 + (t - start);
}

// Largest g with off[g] <= t in a non-decreasing array off[0..n] (off[0] <= t < off[n]).
__device__ inline int64_t upper_find(const int64_t* __restrict__ off, int64_t n, int64_t t) {
    int64_t lo = 0, hi = n;  // invariant: off[lo] <= t < off[hi]
    while (hi - lo > 1) {
        int64_t mid = lo + ((hi - lo) >> 1);
        if (off[mid] <= t) lo = mid;
        else hi = mid;
    }
    return lo;
}

// Inclusive warp scan of a 64-bit value.
__device__ inline int64_t warp_inclusive_scan(int64_t v) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        int64_t y = __shfl_up_sync(0xffffffffu, v, d);
        if (lane >= d) v += y;
    }
    return v;
}

// Exclusive block scan of one 64-bit value per thread (blockDim.x a multiple of 32, <= 1024).
// Returns the thread's exclusive prefix; *total receives the block sum.
__device__ inline int64_t block_exclusive_scan(int64_t v, int64_t* total) {
    __shared__ int64_t warp_sums[33];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    int64_t inc = warp_inclusive_scan(v);
    if (lane == 31) warp_sums[warp] = inc;
    __syncthreads();
    if (warp == 0) {
        int64_t s = lane < nwarps ? warp_sums[lane] : 0;
        int64_t si = warp_inclusive_scan(s);
        if (lane < nwarps) warp_sums[lane] = si - s;
        if (lane == nwarps - 1) warp_sums[32] = si;
    }
    __syncthreads();
    int64_t out = warp_sums[warp] + inc - v;
    int64_t tot = warp_sums[32];
    __syncthreads();
    *total = tot;
    return out;
}

}  // namespace etm
