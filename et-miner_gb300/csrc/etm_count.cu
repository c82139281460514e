// Support counting on CUDA cores: the tile-pair AND+popcount kernel (prefix
// groups with many members, and K=2 as the one group of every frequent
// column) and the warp-per-candidate kernel (small groups).
//
// Tile kernel: a persistent grid walks a list of tile-pairs (ti <= tj) of
// 64 x 64 suffixes. Per 32-word slab it stages in shared memory the AND of
// the group's prefix columns, the 64 "A" suffix rows ANDed with it and the 64
// "B" suffix rows, all with 16-byte coalesced loads; each of the 256 threads
// then accumulates a 4 x 4 block of pair counts from registers. A slab whose
// prefix AND is zero is skipped. The A-row reads are (near) broadcasts and the
// B rows are read at a padded 33-word stride, so the shared-memory reads are
// free of bank conflicts.
#include "etm_common.cuh"
#include "etm_count.cuh"

namespace {

using namespace etm;

// A candidate's count: every count (surv == nullptr), or only a count reaching min_count, with bit t of
// the survivor bitmask set (the fused threshold of count_shared_tiled_fused, shared_tiled.cu:246-280).
__device__ __forceinline__ void emit_count(int32_t* out, uint32_t* surv, int64_t t, int32_t v, int32_t min_count) {
    if (surv == nullptr) {
        out[t] = v;
    } else if (v >= min_count) {
        out[t] = v;
        atomicOr(surv + (t >> 5), 1u << (t & 31));
    }
}

constexpr int TT = 64;                 // suffixes per tile side
constexpr int WCH = 32;                // words per shared-memory slab
constexpr int TILE_THREADS = 256;      // 16 x 16 threads, 4 x 4 pairs each
constexpr int MAXP = 63;               // prefix columns handled
constexpr int STRIDE = WCH + 1;        // padded row stride (words)

struct TileShared {
    uint64_t a[TT * STRIDE];
    uint64_t b[TT * STRIDE];
    uint64_t pre[WCH];
    int64_t oa[TT];  // word offset of each A / B suffix row in `src`, -1 past the group
    int64_t ob[TT];
    int32_t pref[MAXP + 1];
};

// Tile-pair counting over one of two sources:
//   PROJ = false: the padded frequent columns fbv [n_f][ld]; a group's suffix i is
//                 column rows[first+i][width-1]; the prefix columns are ANDed in per word.
//   PROJ = true:  compacted suffix bitvectors: work entry wi's member i is at
//                 src + cbase[wi] + i * cld[wi], cwords[wi] words long, prefix already applied.
template <bool PROJ>
__global__ void __launch_bounds__(TILE_THREADS) count_tiles_popc_kernel(
    const uint64_t* __restrict__ src, int64_t ld, int64_t n_words, const int64_t* __restrict__ cbase,
    const int64_t* __restrict__ cwords, const int64_t* __restrict__ cld, const int32_t* __restrict__ rows, int width,
    const int64_t* __restrict__ grp_first, const int32_t* __restrict__ grp_size, const int64_t* __restrict__ cand_off,
    const int64_t* __restrict__ work_groups, const int64_t* __restrict__ work_off, int64_t n_work, int64_t chunk_base,
    const uint8_t* __restrict__ cls, int32_t* __restrict__ out, int32_t min_count, uint32_t* __restrict__ surv,
    int n_split) {
    __shared__ TileShared sh;
    const int tid = threadIdx.x;
    const int ty = tid >> 4, tx = tid & 15;
    // With n_split > 1 every tile-pair's word range is cut into n_split parts counted by different CTAs, which
    // add their partial counts into `out` (zeroed by the caller): few tile-pairs over many rows still fill the GPU.
    const int64_t total = work_off[n_work] * n_split;
    const int plen = PROJ ? 0 : width - 1;

    for (int64_t unit = blockIdx.x; unit < total; unit += gridDim.x) {
        const int64_t tp = unit / n_split;
        const int part = (int)(unit - tp * n_split);
        const int64_t wi = upper_find(work_off, n_work, tp);
        const int64_t g = work_groups[wi];
        const int64_t m = grp_size[g];
        const int64_t nt = ceil_div<int64_t>(m, TT);
        int64_t ti, tj1;
        tri_decode(tp - work_off[wi], nt + 1, &ti, &tj1);
        const int64_t tj = tj1 - 1;
        const int64_t first = PROJ ? 0 : grp_first[g];  // the projected source needs no rows
        const int64_t cb = cand_off[g] - chunk_base;
        const int64_t words = PROJ ? cwords[wi] : n_words;
        const int64_t n_slabs_all = ceil_div<int64_t>(words, WCH);
        const int64_t per = ceil_div<int64_t>(n_slabs_all, n_split);
        const int64_t s_first = part * per;
        const int64_t n_slabs = min64(n_slabs_all, s_first + per);

        if (tid < TT) {
            const int64_t ia = ti * TT + tid, ib = tj * TT + tid;
            if (PROJ) {
                const int64_t b0 = cbase[wi], st = cld[wi];
                sh.oa[tid] = ia < m ? b0 + ia * st : -1;
                sh.ob[tid] = ib < m ? b0 + ib * st : -1;
            } else {
                sh.oa[tid] = ia < m ? (int64_t)rows[(first + ia) * width + width - 1] * ld : -1;
                sh.ob[tid] = ib < m ? (int64_t)rows[(first + ib) * width + width - 1] * ld : -1;
            }
        }
        if (tid < plen) sh.pref[tid] = rows[first * width + tid];

        // Candidates of this tile-pair that still need a count.
        int any = cls == nullptr;
        if (!any) {
            for (int r = 0; r < 4 && !any; r++) {
                const int64_t i = ti * TT + ty * 4 + r;
                for (int c = 0; c < 4; c++) {
                    const int64_t j = tj * TT + tx + 16 * c;
                    if (i < j && j < m && cls[cb + tri_index(i, j, m)] == ETM_CAND_COUNT) {
                        any = 1;
                        break;
                    }
                }
            }
        }
        if (!__syncthreads_or(any)) continue;

        unsigned acc[4][4];
#pragma unroll
        for (int r = 0; r < 4; r++)
#pragma unroll
            for (int c = 0; c < 4; c++) acc[r][c] = 0;

        for (int64_t s = s_first; s < n_slabs; s++) {
            const int64_t w0 = s * WCH;
            if (!PROJ) {
                if (tid < WCH) {
                    uint64_t p = ~0ULL;
                    for (int q = 0; q < plen; q++) p &= __ldg(src + (int64_t)sh.pref[q] * ld + w0 + tid);
                    sh.pre[tid] = p;
                }
                __syncthreads();
                const int live = tid < WCH ? (sh.pre[tid] != 0ULL) : 0;
                if (!__syncthreads_or(live)) continue;
            }
            // Stage A (masked by the prefix) and B: 64 rows x 16 vectors each.
#pragma unroll
            for (int q = 0; q < (TT * WCH / 2) / TILE_THREADS; q++) {
                const int idx = q * TILE_THREADS + tid;
                const int r = idx >> 4, v = idx & 15;
                const int64_t oa = sh.oa[r], ob = sh.ob[r];
                ulonglong2 xa = make_ulonglong2(0, 0), xb = make_ulonglong2(0, 0);
                if (oa >= 0) xa = __ldg(reinterpret_cast<const ulonglong2*>(src + oa + w0) + v);
                if (ob >= 0) xb = __ldg(reinterpret_cast<const ulonglong2*>(src + ob + w0) + v);
                if (!PROJ) {
                    xa.x &= sh.pre[2 * v];
                    xa.y &= sh.pre[2 * v + 1];
                }
                sh.a[r * STRIDE + 2 * v] = xa.x;
                sh.a[r * STRIDE + 2 * v + 1] = xa.y;
                sh.b[r * STRIDE + 2 * v] = xb.x;
                sh.b[r * STRIDE + 2 * v + 1] = xb.y;
            }
            __syncthreads();
#pragma unroll 4
            for (int w = 0; w < WCH; w++) {
                uint64_t av[4], bv[4];
#pragma unroll
                for (int r = 0; r < 4; r++) av[r] = sh.a[(ty * 4 + r) * STRIDE + w];
#pragma unroll
                for (int c = 0; c < 4; c++) bv[c] = sh.b[(tx + 16 * c) * STRIDE + w];
#pragma unroll
                for (int r = 0; r < 4; r++)
#pragma unroll
                    for (int c = 0; c < 4; c++) acc[r][c] += __popcll(av[r] & bv[c]);
            }
            __syncthreads();
        }
#pragma unroll
        for (int r = 0; r < 4; r++) {
            const int64_t i = ti * TT + ty * 4 + r;
#pragma unroll
            for (int c = 0; c < 4; c++) {
                const int64_t j = tj * TT + tx + 16 * c;
                if (i < j && j < m) {
                    const int64_t t = cb + tri_index(i, j, m);
                    if (cls == nullptr || cls[t] == ETM_CAND_COUNT) {
                        if (n_split > 1) {
                            if (acc[r][c]) atomicAdd(out + t, (int32_t)acc[r][c]);
                        } else {
                            emit_count(out, surv, t, (int32_t)acc[r][c], min_count);
                        }
                    }
                }
            }
        }
        __syncthreads();
    }
}

constexpr int CAND_THREADS = 256;
constexpr int MAXK = 64;

// One warp per candidate: AND of its k columns, 16 bytes per lane per step.
// The candidate's columns sit in the warp's slice of shared memory, so the
// word loop (whose trip count differs between lanes) holds no warp collective.
__global__ void __launch_bounds__(CAND_THREADS) count_cands_kernel(
    const uint64_t* __restrict__ fbv, int64_t ld, int64_t n_words, const int32_t* __restrict__ rows, int width,
    const int64_t* __restrict__ grp_first, const int32_t* __restrict__ grp_size, const int64_t* __restrict__ cand_off,
    const int64_t* __restrict__ work_groups, const int64_t* __restrict__ work_off, int64_t n_work, int64_t chunk_base,
    const uint8_t* __restrict__ cls, int32_t* __restrict__ out, int32_t min_count, uint32_t* __restrict__ surv,
    const uint64_t* __restrict__ occ, int64_t occ_ld) {
    __shared__ int32_t cols_sh[CAND_THREADS / 32][MAXK];
    const int lane = threadIdx.x & 31;
    int32_t* cols = cols_sh[threadIdx.x >> 5];
    const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t n_warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const int64_t total = work_off[n_work];
    const int64_t n_vec = (n_words + 1) >> 1;
    const int k = width + 1;
    for (int64_t c = warp; c < total; c += n_warps) {
        const int64_t wi = upper_find(work_off, n_work, c);
        const int64_t g = work_groups[wi];
        const int64_t local = c - work_off[wi];
        const int64_t t = cand_off[g] - chunk_base + local;
        if (cls && cls[t] != ETM_CAND_COUNT) continue;  // warp-uniform: every lane has the same c
        int64_t i, j;
        tri_decode(local, grp_size[g], &i, &j);
        const int64_t first = grp_first[g];
        __syncwarp();
        for (int q = lane; q < k; q += 32)
            cols[q] = q < width ? rows[(first + i) * width + q] : rows[(first + j) * width + width - 1];
        __syncwarp();
        unsigned s = 0;
        // Blocks of 64 occupancy tiles (1,024 pairs of words): with the occupancy, a tile where one of the
        // columns holds no row is not read (pair v lies in tile v / 16), and a block with none is skipped by
        // the whole warp.
        for (int64_t v0 = 0; v0 < n_vec; v0 += 32 * ETM_OCC_TILE_WORDS) {
            uint64_t live = ~0ULL;
            if (occ != nullptr) {
                const int64_t ow = v0 / (32 * ETM_OCC_TILE_WORDS);
                for (int q = 0; q < k; q++) live &= __ldg(occ + (int64_t)cols[q] * occ_ld + ow);
                if (live == 0ULL) continue;
            }
            const int64_t v1 = min64(n_vec, v0 + 32 * ETM_OCC_TILE_WORDS);
            for (int64_t v = v0 + lane; v < v1; v += 32) {
                if (((live >> ((v - v0) >> 4)) & 1ULL) == 0ULL) continue;
                ulonglong2 x = __ldg(reinterpret_cast<const ulonglong2*>(fbv + (int64_t)cols[0] * ld) + v);
                for (int q = 1; q < k; q++) {
                    const ulonglong2 y = __ldg(reinterpret_cast<const ulonglong2*>(fbv + (int64_t)cols[q] * ld) + v);
                    x.x &= y.x;
                    x.y &= y.y;
                }
                s += __popcll(x.x) + __popcll(x.y);
            }
        }
        s = __reduce_add_sync(0xffffffffu, s);
        if (lane == 0) emit_count(out, surv, t, (int32_t)s, min_count);
    }
}

}  // namespace

namespace etm {

int count_tiles_popcount(const uint64_t* fbv, int64_t ld, int64_t n_words, const int32_t* rows, int32_t width,
                         const int64_t* grp_first, const int32_t* grp_size, const int64_t* cand_off,
                         const int64_t* work_groups, const int64_t* work_off, int64_t n_work, int64_t chunk_base,
                         const uint8_t* cls, int32_t* out, int64_t n_tiles_hint, cudaStream_t s, int32_t min_count,
                         uint32_t* surv) {
    const int64_t cap = (int64_t)max(1, sm_count()) * 6;
    const int grid = (int)max64(1, min64(cap, n_tiles_hint > 0 ? n_tiles_hint : cap));
    count_tiles_popc_kernel<false><<<grid, TILE_THREADS, 0, s>>>(fbv, ld, n_words, nullptr, nullptr, nullptr, rows,
                                                                 width, grp_first, grp_size, cand_off, work_groups,
                                                                 work_off, n_work, chunk_base, cls, out, min_count,
                                                                 surv, 1);
    ETM_LAUNCHED("count_tiles_popc");
    return ETM_OK;
}

int count_tiles_proj_popcount(const uint64_t* cbuf, const int64_t* cbase, const int64_t* cwords, const int64_t* cld,
                              const int32_t* grp_size, const int64_t* cand_off, const int64_t* work_groups,
                              const int64_t* work_off, int64_t n_work, int64_t chunk_base, const uint8_t* cls,
                              int32_t* out, cudaStream_t s, int32_t min_count, uint32_t* surv) {
    const int grid = max(1, sm_count()) * 6;
    count_tiles_popc_kernel<true><<<grid, TILE_THREADS, 0, s>>>(cbuf, 0, 0, cbase, cwords, cld, nullptr, 1, nullptr,
                                                                grp_size, cand_off, work_groups, work_off, n_work,
                                                                chunk_base, cls, out, min_count, surv, 1);
    ETM_LAUNCHED("count_tiles_proj_popc");
    return ETM_OK;
}

}  // namespace etm

extern "C" int etm_count_tiles(const uint64_t* fbv, int64_t ld, int64_t n_words, const int32_t* rows, int32_t width,
                               const int64_t* grp_first, const int32_t* grp_size, const int64_t* cand_off,
                               const int64_t* work_groups, const int64_t* work_off, int64_t n_work,
                               int64_t chunk_base, const uint8_t* cls, int32_t method, int32_t* out_counts,
                               void* stream) {
    ETM_REQUIRE(width >= 1 && width <= MAXP, ETM_EINVAL, "etm_count_tiles: width %d out of range", width);
    ETM_REQUIRE(ld % WCH == 0 && ld >= n_words, ETM_EINVAL, "etm_count_tiles: ld must be a multiple of %d >= n_words", WCH);
    ETM_REQUIRE((reinterpret_cast<uintptr_t>(fbv) & 15) == 0, ETM_EINVAL, "etm_count_tiles: fbv must be 16-byte aligned");
    if (n_work <= 0) return ETM_OK;
    cudaStream_t s = as_stream(stream);
    if (method == ETM_METHOD_TENSOR)
        return etm::count_tiles_tensor(fbv, ld, n_words, rows, width, grp_first, grp_size, cand_off, work_groups,
                                       work_off, n_work, chunk_base, cls, out_counts, s);
    ETM_REQUIRE(method == ETM_METHOD_POPCOUNT, ETM_EINVAL, "etm_count_tiles: unknown method %d", method);
    return etm::count_tiles_popcount(fbv, ld, n_words, rows, width, grp_first, grp_size, cand_off, work_groups,
                                     work_off, n_work, chunk_base, cls, out_counts, -1, s, 0, nullptr);
}

extern "C" int etm_count_tiles_split(const uint64_t* fbv, int64_t ld, int64_t n_words, const int32_t* rows,
                                     int32_t width, const int64_t* grp_first, const int32_t* grp_size,
                                     const int64_t* cand_off, const int64_t* work_groups, const int64_t* work_off,
                                     int64_t n_work, int64_t n_tiles, int64_t chunk_base, const uint8_t* cls,
                                     int32_t n_split, int32_t* out_counts, void* stream) {
    ETM_REQUIRE(width >= 1 && width <= MAXP, ETM_EINVAL, "etm_count_tiles_split: width %d out of range", width);
    ETM_REQUIRE(ld % WCH == 0 && ld >= n_words, ETM_EINVAL,
                "etm_count_tiles_split: ld must be a multiple of %d >= n_words", WCH);
    ETM_REQUIRE((reinterpret_cast<uintptr_t>(fbv) & 15) == 0, ETM_EINVAL,
                "etm_count_tiles_split: fbv must be 16-byte aligned");
    ETM_REQUIRE(n_split >= 1 && n_split <= 65536, ETM_EINVAL, "etm_count_tiles_split: n_split %d out of range", n_split);
    if (n_work <= 0) return ETM_OK;
    const int64_t cap = (int64_t)max(1, sm_count()) * 6;
    const int64_t units = (n_tiles > 0 ? n_tiles : cap) * n_split;
    const int grid = (int)max64(1, min64(cap, units));
    count_tiles_popc_kernel<false><<<grid, TILE_THREADS, 0, as_stream(stream)>>>(
        fbv, ld, n_words, nullptr, nullptr, nullptr, rows, width, grp_first, grp_size, cand_off, work_groups, work_off,
        n_work, chunk_base, cls, out_counts, 0, nullptr, n_split);
    ETM_LAUNCHED("count_tiles_popc");
    return ETM_OK;
}

extern "C" int etm_count_tiles_sel(const uint64_t* fbv, int64_t ld, int64_t n_words, const int32_t* rows,
                                   int32_t width, const int64_t* grp_first, const int32_t* grp_size,
                                   const int64_t* cand_off, const int64_t* work_groups, const int64_t* work_off,
                                   int64_t n_work, int64_t chunk_base, const uint8_t* cls, int32_t min_count,
                                   int32_t* out_counts, uint32_t* surv_bits, void* stream) {
    ETM_REQUIRE(width >= 1 && width <= MAXP, ETM_EINVAL, "etm_count_tiles_sel: width %d out of range", width);
    ETM_REQUIRE(ld % WCH == 0 && ld >= n_words, ETM_EINVAL, "etm_count_tiles_sel: ld must be a multiple of %d >= n_words",
                WCH);
    ETM_REQUIRE((reinterpret_cast<uintptr_t>(fbv) & 15) == 0, ETM_EINVAL, "etm_count_tiles_sel: fbv must be 16-byte aligned");
    ETM_REQUIRE(surv_bits != nullptr, ETM_EINVAL, "etm_count_tiles_sel: surv_bits is required");
    if (n_work <= 0) return ETM_OK;
    return etm::count_tiles_popcount(fbv, ld, n_words, rows, width, grp_first, grp_size, cand_off, work_groups,
                                     work_off, n_work, chunk_base, cls, out_counts, -1, as_stream(stream), min_count,
                                     surv_bits);
}

extern "C" int etm_count_cands(const uint64_t* fbv, int64_t ld, int64_t n_words, const int32_t* rows, int32_t width,
                               const int64_t* grp_first, const int32_t* grp_size, const int64_t* cand_off,
                               const int64_t* work_groups, const int64_t* work_off, int64_t n_work,
                               int64_t chunk_base, const uint8_t* cls, int32_t* out_counts, void* stream) {
    ETM_REQUIRE(width >= 1 && width < MAXK, ETM_EINVAL, "etm_count_cands: width %d out of range", width);
    ETM_REQUIRE(ld % 2 == 0 && ld >= n_words, ETM_EINVAL, "etm_count_cands: ld must be even and >= n_words");
    ETM_REQUIRE((reinterpret_cast<uintptr_t>(fbv) & 15) == 0, ETM_EINVAL, "etm_count_cands: fbv must be 16-byte aligned");
    if (n_work <= 0) return ETM_OK;
    const int grid = max(1, sm_count()) * 8;
    count_cands_kernel<<<grid, CAND_THREADS, 0, as_stream(stream)>>>(fbv, ld, n_words, rows, width, grp_first, grp_size,
                                                                     cand_off, work_groups, work_off, n_work,
                                                                     chunk_base, cls, out_counts, 0, nullptr, nullptr,
                                                                     0);
    ETM_LAUNCHED("count_cands");
    return ETM_OK;
}

extern "C" int etm_count_cands_sel(const uint64_t* fbv, int64_t ld, int64_t n_words, const int32_t* rows,
                                   int32_t width, const int64_t* grp_first, const int32_t* grp_size,
                                   const int64_t* cand_off, const int64_t* work_groups, const int64_t* work_off,
                                   int64_t n_work, int64_t chunk_base, const uint8_t* cls, int32_t min_count,
                                   int32_t* out_counts, uint32_t* surv_bits, const uint64_t* occ, int64_t occ_ld,
                                   void* stream) {
    ETM_REQUIRE(width >= 1 && width < MAXK, ETM_EINVAL, "etm_count_cands_sel: width %d out of range", width);
    ETM_REQUIRE(occ == nullptr || occ_ld >= ceil_div<int64_t>(ceil_div<int64_t>(n_words, ETM_OCC_TILE_WORDS), 64),
                ETM_EINVAL, "etm_count_cands_sel: occ_ld too small for n_words");
    ETM_REQUIRE(ld % 2 == 0 && ld >= n_words, ETM_EINVAL, "etm_count_cands_sel: ld must be even and >= n_words");
    ETM_REQUIRE((reinterpret_cast<uintptr_t>(fbv) & 15) == 0, ETM_EINVAL, "etm_count_cands_sel: fbv must be 16-byte aligned");
    ETM_REQUIRE(surv_bits != nullptr, ETM_EINVAL, "etm_count_cands_sel: surv_bits is required");
    if (n_work <= 0) return ETM_OK;
    const int grid = max(1, sm_count()) * 8;
    count_cands_kernel<<<grid, CAND_THREADS, 0, as_stream(stream)>>>(fbv, ld, n_words, rows, width, grp_first, grp_size,
                                                                     cand_off, work_groups, work_off, n_work,
                                                                     chunk_base, cls, out_counts, min_count, surv_bits,
                                                                     occ, occ_ld);
    ETM_LAUNCHED("count_cands");
    return ETM_OK;
}

namespace {

// The AND+popcount issue rate of the tile kernel's inner loop with nothing else in the way: every thread
// keeps a 4 x 4 block of counters over 4 + 4 words in registers and adds popc(a_r & b_c) per pair, the
// operands rotating every step so no product can be hoisted. The rate is the CUDA-core roofline of the
// tile kernels (their pair counts per second), which are bound by the popcount pipe, not by HBM.
constexpr int RATE_THREADS = 256;
__device__ unsigned g_popc_sink;

__global__ void __launch_bounds__(RATE_THREADS) popc_rate_kernel(int64_t iters, unsigned* __restrict__ sink) {
    const uint64_t seed = 0x9E3779B97F4A7C15ULL * (uint64_t)(blockIdx.x * RATE_THREADS + threadIdx.x + 1);
    uint64_t a[4], b[4];
#pragma unroll
    for (int r = 0; r < 4; r++) {
        a[r] = seed ^ (0xD6E8FEB86659FD93ULL * (uint64_t)(r + 1));
        b[r] = seed + (0xA0761D6478BD642FULL * (uint64_t)(r + 5));
    }
    unsigned acc[4][4];
#pragma unroll
    for (int r = 0; r < 4; r++)
#pragma unroll
        for (int c = 0; c < 4; c++) acc[r][c] = 0;
    for (int64_t it = 0; it < iters; it++) {
#pragma unroll
        for (int r = 0; r < 4; r++)
#pragma unroll
            for (int c = 0; c < 4; c++) acc[r][c] += __popcll(a[r] & b[c]);
#pragma unroll
        for (int r = 0; r < 4; r++) {
            a[r] = (a[r] << 1) | (a[r] >> 63);
            b[r] += 0x9E3779B97F4A7C15ULL;
        }
    }
    unsigned total = 0;
#pragma unroll
    for (int r = 0; r < 4; r++)
#pragma unroll
        for (int c = 0; c < 4; c++) total += acc[r][c];
    if (total == 0xFFFFFFFFu) sink[0] = total;  // never true in practice; keeps the loop alive
}

}  // namespace

extern "C" int etm_popc_rate(int64_t iters, double* out_gops, void* stream) {
    ETM_REQUIRE(iters > 0 && iters < (1LL << 32) && out_gops != nullptr, ETM_EINVAL, "etm_popc_rate: bad iters");
    cudaStream_t s = as_stream(stream);
    unsigned* sink = nullptr;
    ETM_CUDA(cudaGetSymbolAddress(reinterpret_cast<void**>(&sink), g_popc_sink));
    const int grid = max(1, sm_count()) * 8;
    cudaEvent_t e0, e1;
    ETM_CUDA(cudaEventCreate(&e0));
    ETM_CUDA(cudaEventCreate(&e1));
    popc_rate_kernel<<<grid, RATE_THREADS, 0, s>>>(iters / 8 + 1, sink);  // warm-up
    cudaEventRecord(e0, s);
    popc_rate_kernel<<<grid, RATE_THREADS, 0, s>>>(iters, sink);
    cudaEventRecord(e1, s);
    cudaError_t err = cudaGetLastError();
    if (err == cudaSuccess) err = cudaEventSynchronize(e1);
    float ms = 0.f;
    if (err == cudaSuccess) cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (err != cudaSuccess) {
        etm::set_error("etm_popc_rate: %s", cudaGetErrorString(err));
        return ETM_ECUDA;
    }
    const double ops = 16.0 * (double)iters * (double)grid * RATE_THREADS;
    *out_gops = ms > 0.f ? ops / (ms * 1e-3) / 1e9 : 0.0;
    return ETM_OK;
}
