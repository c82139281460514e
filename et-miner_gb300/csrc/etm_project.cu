// Prefix projection: count a prefix group over only the transactions its
// prefix holds. The reference's CPU route does this for wide groups
// (_count_group_proj, core/cpu_miner.py:720-791: a Gram over the prefix's
// tidset); here it is three device passes per chunk of groups:
//
//   1. prefix counts:  popcount of the AND of the group's prefix columns
//                      (sizes the row lists; coalesced 16-byte reads)
//   2. prefix rows:    the ascending transaction ids of that AND (block scan
//                      of per-word popcounts, then each word's bit positions)
//   3. projection:     for every member, the bits of its column at those rows,
//                      packed 64 per word by two warp ballots per 64 rows
//
// after which the tile-pair kernel counts the group on words that hold only
// the prefix's rows: a group whose prefix holds a fraction d of the rows
// costs d of the AND+popcount work it would cost on the full bitvectors.
#include "etm_count.cuh"
#include "etm_scan.cuh"

namespace {

using namespace etm;

constexpr int PT = 256;

__device__ inline uint64_t prefix_word(const uint64_t* __restrict__ fbv, int64_t ld, const int32_t* __restrict__ pref,
                                       int plen, int64_t w) {
    uint64_t p = ~0ULL;
    for (int q = 0; q < plen; q++) p &= __ldg(fbv + (int64_t)pref[q] * ld + w);
    return p;
}

__global__ void __launch_bounds__(PT) prefix_counts_kernel(const uint64_t* __restrict__ fbv, int64_t ld,
                                                           int64_t n_words, const int32_t* __restrict__ rows,
                                                           int width, const int64_t* __restrict__ grp_first,
                                                           const int64_t* __restrict__ work_groups,
                                                           int64_t* __restrict__ out) {
    __shared__ int32_t pref[64];
    __shared__ unsigned part[PT / 32];
    const int64_t wi = blockIdx.x;
    const int64_t first = grp_first[work_groups[wi]];
    const int plen = width - 1;
    if (threadIdx.x < plen) pref[threadIdx.x] = rows[first * width + threadIdx.x];
    __syncthreads();
    unsigned s = 0;
    for (int64_t w = threadIdx.x; w < n_words; w += PT) s += __popcll(prefix_word(fbv, ld, pref, plen, w));
    s = __reduce_add_sync(0xffffffffu, s);
    if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
        unsigned v = threadIdx.x < PT / 32 ? part[threadIdx.x] : 0;
        v = __reduce_add_sync(0xffffffffu, v);
        if (threadIdx.x == 0) out[wi] = v;
    }
}

__global__ void __launch_bounds__(PT) prefix_rows_kernel(const uint64_t* __restrict__ fbv, int64_t ld, int64_t n_words,
                                                         const int32_t* __restrict__ rows, int width,
                                                         const int64_t* __restrict__ grp_first,
                                                         const int64_t* __restrict__ work_groups,
                                                         const int64_t* __restrict__ row_off,
                                                         int32_t* __restrict__ out) {
    __shared__ int32_t pref[64];
    const int64_t wi = blockIdx.x;
    const int64_t first = grp_first[work_groups[wi]];
    const int plen = width - 1;
    if (threadIdx.x < plen) pref[threadIdx.x] = rows[first * width + threadIdx.x];
    __syncthreads();
    int64_t base = row_off[wi];
    const int64_t end = row_off[wi + 1];
    for (int64_t w0 = 0; w0 < n_words; w0 += PT) {
        const int64_t w = w0 + threadIdx.x;
        uint64_t p = w < n_words ? prefix_word(fbv, ld, pref, plen, w) : 0ULL;
        int64_t total;
        int64_t at = base + block_exclusive_scan(__popcll(p), &total);
        while (p) {
            const int b = __ffsll((long long)p) - 1;
            if (at < end) out[at] = (int32_t)(w * 64 + b);
            ++at;
            p &= p - 1;
        }
        base += total;
    }
}

constexpr int MB = 8;  // members per warp: the row-list loads are shared and 2 * MB gathers are in flight

// One warp per (work entry, block of MB members): the members' column bits at the prefix's rows.
// mblk_off is the exclusive prefix of ceil(m / MB) over the work entries.
__global__ void __launch_bounds__(PT) project_kernel(const uint64_t* __restrict__ fbv, int64_t ld,
                                                     const int32_t* __restrict__ rows, int width,
                                                     const int64_t* __restrict__ grp_first,
                                                     const int32_t* __restrict__ grp_size,
                                                     const int64_t* __restrict__ work_groups,
                                                     const int64_t* __restrict__ mblk_off, int64_t n_work,
                                                     const int64_t* __restrict__ row_off,
                                                     const int32_t* __restrict__ rowidx,
                                                     const int64_t* __restrict__ cbase, const int64_t* __restrict__ cld,
                                                     uint64_t* __restrict__ cbuf) {
    const int lane = threadIdx.x & 31;
    const int64_t total = mblk_off[n_work];
    const int64_t n_warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t q = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; q < total; q += n_warps) {
        const int64_t wi = upper_find(mblk_off, n_work, q);
        const int64_t g = work_groups[wi];
        const int64_t m = grp_size[g];
        const int64_t i0 = (q - mblk_off[wi]) * MB;
        const int nm = (int)min64(MB, m - i0);
        const int32_t* R = rowidx + row_off[wi];
        const int64_t n = row_off[wi + 1] - row_off[wi];
        const int64_t stride = cld[wi];
        const int64_t first = grp_first[g];
        const uint64_t* src[MB];
#pragma unroll
        for (int j = 0; j < MB; j++) {
            const int64_t col = rows[(first + i0 + (j < nm ? j : 0)) * width + width - 1];
            src[j] = fbv + col * ld;
        }
        uint64_t* dst = cbuf + cbase[wi] + i0 * stride;
        const int64_t nw = (n + 63) >> 6;
        for (int64_t t = 0; t < nw; t++) {
            const int64_t e0 = t * 64 + lane, e1 = e0 + 32;
            const int32_t r0 = e0 < n ? __ldg(R + e0) : -1;
            const int32_t r1 = e1 < n ? __ldg(R + e1) : -1;
            uint64_t x0[MB], x1[MB];
#pragma unroll
            for (int j = 0; j < MB; j++) {
                x0[j] = r0 >= 0 ? __ldg(src[j] + (r0 >> 6)) : 0ULL;
                x1[j] = r1 >= 0 ? __ldg(src[j] + (r1 >> 6)) : 0ULL;
            }
#pragma unroll
            for (int j = 0; j < MB; j++) {
                const unsigned lo = __ballot_sync(0xffffffffu, (unsigned)(x0[j] >> (r0 & 63)) & 1u);
                const unsigned hi = __ballot_sync(0xffffffffu, (unsigned)(x1[j] >> (r1 & 63)) & 1u);
                if (lane == j && j < nm) dst[j * stride + t] = (uint64_t)lo | ((uint64_t)hi << 32);
            }
        }
        for (int j = 0; j < nm; j++)
            for (int64_t w = nw + lane; w < stride; w += 32) dst[j * stride + w] = 0ULL;
    }
}

}  // namespace

extern "C" int etm_prefix_counts(const uint64_t* fbv, int64_t ld, int64_t n_words, const int32_t* rows, int32_t width,
                                 const int64_t* grp_first, const int64_t* work_groups, int64_t n_work,
                                 int64_t* out_counts, void* stream) {
    ETM_REQUIRE(width >= 2 && width <= 64, ETM_EINVAL, "etm_prefix_counts: width %d out of range (2..64)", width);
    ETM_REQUIRE(ld >= n_words, ETM_EINVAL, "etm_prefix_counts: ld < n_words");
    ETM_REQUIRE(n_work < (1LL << 31), ETM_EINVAL, "etm_prefix_counts: too many groups");
    if (n_work <= 0) return ETM_OK;
    prefix_counts_kernel<<<(unsigned)n_work, PT, 0, as_stream(stream)>>>(fbv, ld, n_words, rows, width, grp_first,
                                                                         work_groups, out_counts);
    ETM_LAUNCHED("prefix_counts");
    return ETM_OK;
}

extern "C" int etm_prefix_rows(const uint64_t* fbv, int64_t ld, int64_t n_words, const int32_t* rows, int32_t width,
                               const int64_t* grp_first, const int64_t* work_groups, int64_t n_work,
                               const int64_t* row_off, int32_t* out_rows, void* stream) {
    ETM_REQUIRE(width >= 2 && width <= 64, ETM_EINVAL, "etm_prefix_rows: width %d out of range (2..64)", width);
    ETM_REQUIRE(ld >= n_words && n_words < (1LL << 25), ETM_EINVAL, "etm_prefix_rows: bad n_words");
    ETM_REQUIRE(n_work < (1LL << 31), ETM_EINVAL, "etm_prefix_rows: too many groups");
    if (n_work <= 0) return ETM_OK;
    prefix_rows_kernel<<<(unsigned)n_work, PT, 0, as_stream(stream)>>>(fbv, ld, n_words, rows, width, grp_first,
                                                                       work_groups, row_off, out_rows);
    ETM_LAUNCHED("prefix_rows");
    return ETM_OK;
}

extern "C" int etm_project(const uint64_t* fbv, int64_t ld, const int32_t* rows, int32_t width,
                           const int64_t* grp_first, const int32_t* grp_size, const int64_t* work_groups,
                           const int64_t* mblk_off, int64_t n_work, const int64_t* row_off, const int32_t* row_idx,
                           const int64_t* cbase, const int64_t* cld, uint64_t* cbuf, void* stream) {
    ETM_REQUIRE(width >= 2 && width <= 64, ETM_EINVAL, "etm_project: width %d out of range (2..64)", width);
    if (n_work <= 0) return ETM_OK;
    const int grid = max(1, sm_count()) * 8;
    project_kernel<<<grid, PT, 0, as_stream(stream)>>>(fbv, ld, rows, width, grp_first, grp_size, work_groups,
                                                       mblk_off, n_work, row_off, row_idx, cbase, cld, cbuf);
    ETM_LAUNCHED("project");
    return ETM_OK;
}

extern "C" int etm_count_tiles_proj(const uint64_t* cbuf, const int64_t* cbase, const int64_t* cwords,
                                    const int64_t* cld, const int32_t* grp_size, const int64_t* cand_off,
                                    const int64_t* work_groups, const int64_t* work_off, int64_t n_work,
                                    int64_t chunk_base, const uint8_t* cls, int32_t method, int32_t* out_counts,
                                    void* stream) {
    ETM_REQUIRE((reinterpret_cast<uintptr_t>(cbuf) & 15) == 0, ETM_EINVAL, "etm_count_tiles_proj: cbuf must be 16-byte aligned");
    if (n_work <= 0) return ETM_OK;
    ETM_REQUIRE(method == ETM_METHOD_POPCOUNT, ETM_EINVAL, "etm_count_tiles_proj: method %d not available", method);
    return etm::count_tiles_proj_popcount(cbuf, cbase, cwords, cld, grp_size, cand_off, work_groups, work_off, n_work,
                                          chunk_base, cls, out_counts, as_stream(stream));
}
