// Exact 0/1 Gram of prefix-group suffixes on the tcgen05 tensor cores.
//
// For a group whose members are bit rows x_0..x_{m-1} (projected suffix
// words, or for K=2 the frequent columns themselves), the pair counts are
// C[i][j] = popcount(x_i & x_j) = sum_r x_i[r] * x_j[r]: the Gram matrix X X^T
// of a 0/1 matrix. Three kernels compute it, all persistent (one CTA per SM)
// and all with the same pipeline:
//
//   producers  one thread per operand row: per stage (K = 64 transactions for
//              f16, 128 for e4m3) it expands its row's words (prefetched a
//              batch of 4 stages ahead into registers) into elements in the
//              128-byte swizzled K-major shared-memory layout the MMA reads
//              (SWIZZLE_128B), then fence.proxy.async and an mbarrier arrive.
//   MMA        one thread issues tcgen05.mma per 32-byte K step into f32
//              accumulators in tensor memory; tcgen05.commit frees each stage
//              and finally signals the epilogue.
//   epilogue   the producer warps read their TMEM lanes back with tcgen05.ld
//              and write the i < j counts at their lexicographic slots.
//
//   gram_tc_kernel    128 x 256 items (A: 128 members, B: 256), 12 producer
//                     warps, 4 stages; optionally A from tensor memory
//                     (tcgen05.st; exact but slower on GB300).
//   gram_wide_kernel  256 x 256 block pairs, 16 producer warps, 3 stages of
//                     64 KB, two M = 128 MMAs per K step sharing the B tile
//                     (accumulators in TMEM columns 0-255 and 256-511): a
//                     third fewer shared-memory stores per unit of work. The
//                     engine's default.
//   gram_pair_kernel  256 x 256 block pairs over a cluster of two CTAs
//                     (cta_group::2, M = 256); see its own comment.
//
// On a diagonal item the A rows are rows of B and are read from B's tile.
//
// Exactness: a set bit is stored as the format's smallest subnormal s
// (f16 2^-24, e4m3 2^-9), so every product is 0 or s^2 and every partial sum
// is c * s^2 with an integer c below 2^24 (the caller sends only groups of at
// most 2^24 rows here): exact in f32, and scaled back exactly to c.
//
// Every mbarrier wait is bounded: after WAIT_LIMIT polls the block raises an
// abort flag, every thread leaves its loop, the MMA thread waits (bounded) for
// its issued MMAs, TMEM is freed, and the kernel records ETM_ETIMEOUT in its
// status word instead of hanging.
#include "etm_count.cuh"

namespace {

using namespace etm;

constexpr int TC_M = 128;  // A rows per work item
constexpr int TC_N = 256;  // B rows per work item (a super-tile of two A tiles)
constexpr int TC_STAGES = 4;
constexpr int TC_PRODUCERS = TC_M + TC_N;  // one operand row per thread: 0-127 the A rows, 128-383 the B rows
constexpr int TC_THREADS = TC_PRODUCERS + 32;
constexpr int MMA_WARP = TC_PRODUCERS / 32;
constexpr int EPI_WARPS = 8;                // warps 0-7 read the accumulator: lanes (w % 4), columns (w / 4)
constexpr uint32_t TC_TMEM_COLS = 512;      // columns 0-255: the f32 accumulator; 256-383: A operand stages
constexpr uint32_t A_TMEM_COL = 256;
constexpr uint32_t A_STAGE_COLS = 32;       // one 128-byte operand row = 32 32-bit TMEM columns
constexpr int A_BYTES = TC_M * 128;         // 128 rows x 128 bytes, one SWIZZLE_128B K block
constexpr int B_BYTES = TC_N * 128;
// Shared-memory bytes per pipeline stage: the B tile, plus the A tile unless A lives in TMEM.
template <bool A_TMEM>
__host__ __device__ constexpr int slot_bytes() { return A_TMEM ? B_BYTES : A_BYTES + B_BYTES; }
template <bool A_TMEM>
__host__ __device__ constexpr int smem_bytes() { return TC_STAGES * slot_bytes<A_TMEM>() + 1024; }
constexpr long long WAIT_LIMIT = 1LL << 25;

__device__ int g_tc_status;

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ bool mbar_test(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// try_wait suspends the thread in hardware until the phase completes or a short time-out passes.
__device__ __forceinline__ bool mbar_try(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Waits for the phase of `parity` to complete; false if the block aborts or the wait runs out.
__device__ bool mbar_wait(uint64_t* bar, uint32_t parity, volatile int* abort_flag) {
    long long n = 0;
    while (!mbar_try(bar, parity)) {
        if (*abort_flag) return false;
        if (++n > WAIT_LIMIT) {
            *abort_flag = 1;
            return false;
        }
    }
    return true;
}

__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// Shared-memory matrix descriptor: K-major, SWIZZLE_128B, 8-row groups 1024 bytes apart.
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr) {
    uint64_t d = 0;
    d |= (uint64_t)((addr >> 4) & 0x3FFF);
    d |= (uint64_t)1 << 16;                  // leading byte offset (unused for swizzled K-major)
    d |= (uint64_t)(1024 >> 4) << 32;        // stride byte offset: 8 rows x 128 B
    d |= (uint64_t)1 << 46;                  // descriptor version for tcgen05
    d |= (uint64_t)2 << 61;                  // SWIZZLE_128B
    return d;
}

// Instruction descriptor: D f32, A/B format code 0 (f16 for kind::f16, e4m3 for kind::f8f6f4),
// both K-major, N = 256, M = 128.
__host__ __device__ constexpr uint32_t instr_desc() {
    return (1u << 4) | ((uint32_t)(TC_N >> 3) << 17) | ((uint32_t)(TC_M >> 4) << 24);
}

// D (TMEM) += A x B, both from shared-memory descriptors.
template <int ELEM>
__device__ __forceinline__ void mma_ss(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t acc) {
    if constexpr (ELEM == 2) {
        asm volatile(
            "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
            " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
            "l"(a), "l"(b), "r"(instr_desc()), "r"(acc));
    } else {
        asm volatile(
            "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
            " tcgen05.mma.cta_group::1.kind::f8f6f4 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
            "l"(a), "l"(b), "r"(instr_desc()), "r"(acc));
    }
}

// D (TMEM) += A (TMEM, row i in lane i, K packed along columns) x B (shared memory descriptor).
template <int ELEM>
__device__ __forceinline__ void mma(uint32_t tmem_d, uint32_t tmem_a, uint64_t b, uint32_t acc) {
    if constexpr (ELEM == 2) {
        asm volatile(
            "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
            " tcgen05.mma.cta_group::1.kind::f16 [%0], [%1], %2, %3, p;\n}\n" ::"r"(tmem_d),
            "r"(tmem_a), "l"(b), "r"(instr_desc()), "r"(acc));
    } else {
        asm volatile(
            "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
            " tcgen05.mma.cta_group::1.kind::f8f6f4 [%0], [%1], %2, %3, p;\n}\n" ::"r"(tmem_d),
            "r"(tmem_a), "l"(b), "r"(instr_desc()), "r"(acc));
    }
}

// A set bit becomes the format's smallest positive subnormal (f16 0x0001 = 2^-24, e4m3 0x01 = 2^-9): the
// expansion is then the bare bit spread, with no multiply. Every product is one power of two (2^-48 or
// 2^-18), a count c accumulates to exactly c * 2^-48 or c * 2^-18 in f32 (c < 2^24), and the epilogue
// scales back exactly.
template <int ELEM>
__device__ __forceinline__ constexpr float count_scale() { return ELEM == 2 ? 281474976710656.0f : 262144.0f; }

// One operand row as 32 32-bit words: bits of x0 (and x1 for e4m3) expanded to elements.
template <int ELEM>
__device__ __forceinline__ void expand_row(uint64_t x0, uint64_t x1, uint32_t* w) {
#pragma unroll
    for (int c = 0; c < 32; c++) {
        if constexpr (ELEM == 2) {
            const uint32_t t = (uint32_t)(x0 >> (2 * c)) & 3u;
            w[c] = (t & 1u) | ((t >> 1) << 16);  // f16 0x0001 = 2^-24 per set bit
        } else {
            const uint32_t nib = (uint32_t)((c < 16 ? x0 : x1) >> (4 * (c & 15))) & 0xFu;
            w[c] = (nib * 0x00204081u) & 0x01010101u;  // e4m3 0x01 = 2^-9 per set bit
        }
    }
}

__device__ __forceinline__ void tmem_store_row(uint32_t taddr, const uint32_t* w) {
    asm volatile(
        "tcgen05.st.sync.aligned.32x32b.x32.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,"
        "%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31,%32};" ::"r"(taddr),
        "r"(w[0]), "r"(w[1]), "r"(w[2]), "r"(w[3]), "r"(w[4]), "r"(w[5]), "r"(w[6]), "r"(w[7]), "r"(w[8]),
        "r"(w[9]), "r"(w[10]), "r"(w[11]), "r"(w[12]), "r"(w[13]), "r"(w[14]), "r"(w[15]), "r"(w[16]),
        "r"(w[17]), "r"(w[18]), "r"(w[19]), "r"(w[20]), "r"(w[21]), "r"(w[22]), "r"(w[23]), "r"(w[24]),
        "r"(w[25]), "r"(w[26]), "r"(w[27]), "r"(w[28]), "r"(w[29]), "r"(w[30]), "r"(w[31])
        : "memory");
    asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}

// 16 bytes of operand elements from bits [0, 16/ELEM) of v: the smallest subnormal (f16 0x0001, e4m3 0x01) or 0.
template <int ELEM>
__device__ __forceinline__ uint4 expand_chunk(uint32_t v) {
    uint4 o;
    if constexpr (ELEM == 2) {
        // 8 bits -> 8 halves: two bits per 32-bit word.
        uint32_t w[4];
#pragma unroll
        for (int q = 0; q < 4; q++) {
            const uint32_t t = (v >> (2 * q)) & 3u;
            w[q] = (t & 1u) | ((t >> 1) << 16);
        }
        o = make_uint4(w[0], w[1], w[2], w[3]);
    } else {
        // 16 bits -> 16 bytes: four bits per 32-bit word, spread to one bit per byte.
        uint32_t w[4];
#pragma unroll
        for (int q = 0; q < 4; q++) {
            const uint32_t nib = (v >> (4 * q)) & 0xFu;
            w[q] = (nib * 0x00204081u) & 0x01010101u;
        }
        o = make_uint4(w[0], w[1], w[2], w[3]);
    }
    return o;
}

// Row r of a 128 x 128-byte SWIZZLE_128B atom: logical 16-byte chunk c lives at chunk c ^ (r % 8).
template <int ELEM>
__device__ __forceinline__ void store_row(uint8_t* atom, int r, uint64_t x0, uint64_t x1) {
    uint8_t* row = atom + (r >> 3) * 1024 + (r & 7) * 128;
#pragma unroll
    for (int c = 0; c < 8; c++) {
        uint32_t bits;
        if constexpr (ELEM == 2) bits = (uint32_t)(x0 >> (8 * c)) & 0xFFu;
        else bits = (uint32_t)((c < 4 ? x0 : x1) >> (16 * (c & 3))) & 0xFFFFu;
        *reinterpret_cast<uint4*>(row + ((c ^ (r & 7)) << 4)) = expand_chunk<ELEM>(bits);
    }
}

template <int ELEM, bool A_TMEM>
__global__ void __launch_bounds__(TC_THREADS, 1) gram_tc_kernel(
    const uint64_t* __restrict__ src, const int64_t* __restrict__ cbase, const int64_t* __restrict__ cwords,
    const int64_t* __restrict__ cld, const int32_t* __restrict__ grp_size, const int64_t* __restrict__ cand_off,
    const int64_t* __restrict__ work_groups, const int64_t* __restrict__ work_off, int64_t n_work, int64_t chunk_base,
    const uint8_t* __restrict__ cls, int32_t* __restrict__ out) {
    constexpr int WORDS_PER_STAGE = ELEM == 2 ? 1 : 2;  // a 128-byte row holds 64 halves or 128 bytes
    constexpr int SLOT_BYTES = slot_bytes<A_TMEM>();
    extern __shared__ uint8_t dsmem[];
    __shared__ __align__(8) uint64_t full_bar[TC_STAGES];
    __shared__ __align__(8) uint64_t empty_bar[TC_STAGES];
    __shared__ __align__(8) uint64_t acc_bar;
    __shared__ __align__(8) uint64_t drain_bar;
    __shared__ uint32_t tmem_sh;
    __shared__ int abort_sh;
    __shared__ int64_t off_a[TC_M];
    __shared__ int64_t off_b[TC_N];

    uint8_t* slots = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(dsmem) + 1023) & ~uintptr_t(1023));
    const int tid = threadIdx.x;
    const int warp = tid >> 5, lane = tid & 31;

    if (tid == 0) {
        for (int s = 0; s < TC_STAGES; s++) {
            mbar_init(&full_bar[s], TC_PRODUCERS);
            mbar_init(&empty_bar[s], 1);
        }
        mbar_init(&acc_bar, 1);
        mbar_init(&drain_bar, 1);
        abort_sh = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == MMA_WARP) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_sh)),
                     "r"(TC_TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
        tc_fence_before();
    }
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_sh;
    volatile int* abort_flag = &abort_sh;

    const int64_t total = work_off[n_work];
    int64_t gstage = 0;      // stages issued so far (barrier phases)
    uint32_t tile_iter = 0;  // tiles whose accumulator was committed

    for (int64_t tp = blockIdx.x; tp < total; tp += gridDim.x) {
        // Work item: half h of super-tile ua (A: 128 members) against super-tile ub (B: 256 members),
        // ua <= ub; two items per super-tile pair.
        const int64_t wi = upper_find(work_off, n_work, tp);
        const int64_t g = work_groups[wi];
        const int64_t m = grp_size[g];
        const int64_t nb = ceil_div<int64_t>(m, TC_N);
        const int64_t local = tp - work_off[wi];
        int64_t ua, ub1;
        tri_decode(local >> 1, nb + 1, &ua, &ub1);
        const int64_t ub = ub1 - 1;
        const int64_t a0 = ua * TC_N + (local & 1) * TC_M;  // first A member
        const int64_t b0 = ub * TC_N;                       // first B member
        if (a0 >= m) continue;                              // empty half (uniform across the block)
        const bool diag = ua == ub;                         // A rows lie inside B's rows
        const int a_in_b = (int)(local & 1);                // which half of B they are
        const int64_t cb = cand_off[g] - chunk_base;
        const int64_t words = cwords[wi];
        const int64_t n_stages = ceil_div<int64_t>(words, WORDS_PER_STAGE);
        if (tid < TC_M) {
            const int64_t ia = a0 + tid;
            off_a[tid] = ia < m ? cbase[wi] + ia * cld[wi] : -1;
        }
        if (tid < TC_N) {
            const int64_t ib = b0 + tid;
            off_b[tid] = ib < m ? cbase[wi] + ib * cld[wi] : -1;
        }
        int any = cls == nullptr;
        if (!any && tid < TC_M) {
            const int64_t i = a0 + tid;
            for (int c = 0; c < TC_N && !any; c++) {
                const int64_t j = b0 + c;
                any = i < j && j < m && cls[cb + tri_index(i, j, m)] == ETM_CAND_COUNT;
            }
        }
        if (!__syncthreads_or(any)) continue;

        if (warp < MMA_WARP) {
            // ---- producers: thread t expands row t % 128 of A (t < 128) or of B ----
            // Words for PF stages are loaded one batch ahead into registers, so the global
            // latency of batch b+1 overlaps the expansion and MMAs of batch b.
            constexpr int PF = 4;
            constexpr int BW = PF * WORDS_PER_STAGE;  // words per row per batch (16-byte aligned)
            const bool is_b = tid >= TC_M;
            const int prow = is_b ? tid - TC_M : tid;
            // On a diagonal item the A rows are rows of B: the MMA reads them from B's tile.
            const bool idle = !is_b && diag;
            const int64_t off = idle ? -1 : (is_b ? off_b[prow] : off_a[prow]);
            uint64_t cur[BW], nxt[BW];
            auto load_batch = [&](int64_t s0, uint64_t* x) {
#pragma unroll
                for (int q = 0; q < BW; q += 2) {
                    ulonglong2 v = make_ulonglong2(0, 0);
                    if (off >= 0) v = __ldg(reinterpret_cast<const ulonglong2*>(src + off + s0 * WORDS_PER_STAGE + q));
                    x[q] = v.x;
                    x[q + 1] = v.y;
                }
            };
            if (n_stages > 0) load_batch(0, cur);
            for (int64_t s0 = 0; s0 < n_stages && !*abort_flag; s0 += PF) {
                if (s0 + PF < n_stages) load_batch(s0 + PF, nxt);
#pragma unroll
                for (int j = 0; j < PF; j++) {
                    const int64_t s = s0 + j;
                    if (s >= n_stages) break;
                    const int64_t G = gstage + s;
                    const int slot = (int)(G % TC_STAGES);
                    const uint32_t use = (uint32_t)(G / TC_STAGES);
                    if (!mbar_wait(&empty_bar[slot], (use & 1u) ^ 1u, abort_flag)) break;
                    const uint64_t x0 = cur[j * WORDS_PER_STAGE];
                    const uint64_t x1 = WORDS_PER_STAGE == 2 ? cur[j * WORDS_PER_STAGE + 1] : 0ULL;
                    if (idle) {
                        // nothing to stage
                    } else if (A_TMEM && !is_b) {
                        // A rows go straight from registers into this warp's TMEM lanes, after the
                        // MMAs that read this slot (their commit completed the barrier just waited on).
                        tc_fence_after();
                        uint32_t w[32];
                        expand_row<ELEM>(x0, x1, w);
                        tmem_store_row(tmem + ((uint32_t)(warp * 32) << 16) + A_TMEM_COL + slot * A_STAGE_COLS, w);
                        tc_fence_before();
                    } else {
                        // Rows of the swizzled shared tiles: B (the A rows again on a diagonal
                        // tile-pair), and A too when it does not live in TMEM.
                        const int atom = (!A_TMEM && is_b) ? A_BYTES : 0;
                        store_row<ELEM>(slots + slot * SLOT_BYTES + atom, prow, x0, x1);
                        fence_proxy_async();
                    }
                    mbar_arrive(&full_bar[slot]);
                }
#pragma unroll
                for (int q = 0; q < BW; q++) cur[q] = nxt[q];
            }
            // ---- epilogue: warp w < 8 reads TMEM lanes 32 (w % 4) .. +31, columns 128 (w / 4) .. +127 ----
            const bool ok = n_stages == 0 || mbar_wait(&acc_bar, tile_iter & 1u, abort_flag);
            if (ok && warp < EPI_WARPS) {
                tc_fence_after();
                const int lane_base = (warp & 3) * 32;
                const int64_t i = a0 + lane_base + lane;
                for (int q = 0; q < 4; q++) {
                    const int col0 = (warp >> 2) * 128 + q * 32;
                    uint32_t v[32];
                    if (n_stages > 0) {
                        const uint32_t taddr = tmem + ((uint32_t)lane_base << 16) + (uint32_t)col0;
                        asm volatile(
                            "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,"
                            "%14,%15,%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
                            : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]),
                              "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]),
                              "=r"(v[14]), "=r"(v[15]), "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]),
                              "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]), "=r"(v[24]), "=r"(v[25]),
                              "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
                            : "r"(taddr));
                        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
                    } else {
#pragma unroll
                        for (int c = 0; c < 32; c++) v[c] = 0u;
                    }
                    if (i < m) {
#pragma unroll
                        for (int c = 0; c < 32; c++) {
                            const int64_t j = b0 + col0 + c;
                            if (i < j && j < m) {
                                const int64_t t = cb + tri_index(i, j, m);
                                if (cls == nullptr || cls[t] == ETM_CAND_COUNT)
                                    out[t] = n_stages > 0 ? __float2int_rn(__uint_as_float(v[c]) * count_scale<ELEM>()) : 0;
                            }
                        }
                    }
                }
            }
            tc_fence_before();
        } else if (lane == 0) {
            // ---- MMA issuer ----
            tc_fence_after();
            for (int64_t s = 0; s < n_stages; s++) {
                const int64_t G = gstage + s;
                const int slot = (int)(G % TC_STAGES);
                const uint32_t use = (uint32_t)(G / TC_STAGES);
                if (!mbar_wait(&full_bar[slot], use & 1u, abort_flag)) break;
                tc_fence_after();
                const uint32_t base = smem_u32(slots + slot * SLOT_BYTES);
                const uint32_t b_addr = A_TMEM ? base : base + A_BYTES;
                // A: its own tile, or on a diagonal item rows 128 h.. of B's tile (16 KB per 128 rows).
                const uint32_t a_addr = diag ? b_addr + a_in_b * A_BYTES : base;
                const uint32_t a_tmem = tmem + A_TMEM_COL + slot * A_STAGE_COLS;
#pragma unroll
                for (int k = 0; k < 4; k++) {  // 4 x 32 bytes of K per 128-byte row (8 TMEM columns of A)
                    const uint32_t acc = (s > 0 || k > 0) ? 1u : 0u;
                    if (A_TMEM && !diag) mma<ELEM>(tmem, a_tmem + 8 * k, smem_desc(b_addr + 32 * k), acc);
                    else mma_ss<ELEM>(tmem, smem_desc(a_addr + 32 * k), smem_desc(b_addr + 32 * k), acc);
                }
                mma_commit(&empty_bar[slot]);
            }
            mma_commit(&acc_bar);
        }
        gstage += n_stages;
        tile_iter += 1;
        __syncthreads();
        if (*abort_flag) break;
    }

    // Teardown: make sure no MMA is still writing TMEM, then free it.
    if (warp == MMA_WARP) {
        if (lane == 0 && *abort_flag) {
            mma_commit(&drain_bar);
            long long n = 0;
            while (!mbar_test(&drain_bar, 0) && ++n < WAIT_LIMIT) __nanosleep(64);
        }
        __syncwarp();
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TC_TMEM_COLS) : "memory");
    }
    if (tid == 0 && *abort_flag) atomicExch(&g_tc_status, ETM_ETIMEOUT);
}

template <int ELEM, bool A_TMEM>
int launch_gram(const uint64_t* cbuf, const int64_t* cbase, const int64_t* cwords, const int64_t* cld,
                const int32_t* grp_size, const int64_t* cand_off, const int64_t* work_groups, const int64_t* work_off,
                int64_t n_work, int64_t n_tiles, int64_t chunk_base, const uint8_t* cls, int32_t* out,
                int64_t* /*work_counter: items go round-robin*/, cudaStream_t s) {
    static bool configured = false;
    if (!configured) {
        ETM_CUDA(cudaFuncSetAttribute(gram_tc_kernel<ELEM, A_TMEM>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      smem_bytes<A_TMEM>()));
        configured = true;
    }
    const int64_t sms = max(1, sm_count());
    const int grid = (int)max64(1, min64(sms, n_tiles > 0 ? n_tiles : sms));
    gram_tc_kernel<ELEM, A_TMEM><<<grid, TC_THREADS, smem_bytes<A_TMEM>(), s>>>(
        cbuf, cbase, cwords, cld, grp_size, cand_off, work_groups, work_off, n_work, chunk_base, cls, out);
    ETM_LAUNCHED("gram_tc");
    return ETM_OK;
}

// ---------------------------------------------------------------------------------------------
// Wide form: one CTA computes a whole 256 x 256 block pair with two M = 128 MMAs per K step that
// share the B tile (accumulators in TMEM columns 0-255 and 256-511). Per stage it stages 512
// operand rows (256 on a diagonal block pair) for twice the MMA work of a 128 x 256 item: a third
// fewer shared-memory stores per unit of work than gram_tc_kernel.
constexpr int WD_TILE = 256;                     // A rows and B rows per block pair
constexpr int WD_STAGES = 3;
constexpr int WD_PRODUCERS = 2 * WD_TILE;        // thread t < 256: A row t; else B row t - 256
constexpr int WD_THREADS = WD_PRODUCERS + 32;
constexpr int WD_MMA_WARP = WD_PRODUCERS / 32;
constexpr int WD_HALF = 128 * 128;               // bytes of one 128-row operand tile
constexpr int WD_SLOT = 4 * WD_HALF;             // A (two halves), then B (two halves)
constexpr int WD_SMEM = WD_STAGES * WD_SLOT + 1024;

template <int ELEM>
__global__ void __launch_bounds__(WD_THREADS, 1) gram_wide_kernel(
    const uint64_t* __restrict__ src, const int64_t* __restrict__ cbase, const int64_t* __restrict__ cwords,
    const int64_t* __restrict__ cld, const int32_t* __restrict__ grp_size, const int64_t* __restrict__ cand_off,
    const int64_t* __restrict__ work_groups, const int64_t* __restrict__ work_off, int64_t n_work, int64_t chunk_base,
    const uint8_t* __restrict__ cls, int32_t* __restrict__ out,
    unsigned long long* __restrict__ work_counter) {
    constexpr int WORDS_PER_STAGE = ELEM == 2 ? 1 : 2;
    extern __shared__ uint8_t dsmem[];
    __shared__ __align__(8) uint64_t full_bar[WD_STAGES];
    __shared__ __align__(8) uint64_t empty_bar[WD_STAGES];
    __shared__ __align__(8) uint64_t acc_bar;
    __shared__ __align__(8) uint64_t drain_bar;
    __shared__ uint32_t tmem_sh;
    __shared__ int abort_sh;
    __shared__ int64_t off_a[WD_TILE];
    __shared__ int64_t off_b[WD_TILE];
    __shared__ int64_t next_sh;

    uint8_t* slots = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(dsmem) + 1023) & ~uintptr_t(1023));
    const int tid = threadIdx.x;
    const int warp = tid >> 5, lane = tid & 31;

    if (tid == 0) {
        for (int s = 0; s < WD_STAGES; s++) {
            mbar_init(&full_bar[s], WD_PRODUCERS);
            mbar_init(&empty_bar[s], 1);
        }
        mbar_init(&acc_bar, 1);
        mbar_init(&drain_bar, 1);
        abort_sh = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == WD_MMA_WARP) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_sh)),
                     "r"(TC_TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
        tc_fence_before();
    }
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_sh;
    volatile int* abort_flag = &abort_sh;

    const int64_t total = work_off[n_work];
    int64_t gstage = 0;
    uint32_t tile_iter = 0;
    // Block pairs in work-list order; with a work counter each CTA takes the next unclaimed one
    // (dynamic balance across groups of different lengths), else every gridDim.x-th.
    auto next_item = [&](int64_t tp) -> int64_t {
        if (tid == 0)
            next_sh = work_counter != nullptr ? (int64_t)gridDim.x + (int64_t)atomicAdd(work_counter, 1ULL)
                                               : tp + gridDim.x;
        __syncthreads();
        return next_sh;
    };
    for (int64_t tp = blockIdx.x; tp < total; tp = next_item(tp)) {
        const int64_t wi = upper_find(work_off, n_work, tp);
        const int64_t g = work_groups[wi];
        const int64_t m = grp_size[g];
        const int64_t nb = ceil_div<int64_t>(m, WD_TILE);
        int64_t ua, ub1;
        tri_decode(tp - work_off[wi], nb + 1, &ua, &ub1);
        const int64_t ub = ub1 - 1;
        const bool diag = ua == ub;
        const int64_t a0 = ua * WD_TILE, b0 = ub * WD_TILE;
        const int64_t cb = cand_off[g] - chunk_base;
        const int64_t words = cwords[wi];
        const int64_t n_stages = ceil_div<int64_t>(words, WORDS_PER_STAGE);
        if (tid < WD_TILE) {
            const int64_t ia = a0 + tid, ib = b0 + tid;
            off_a[tid] = ia < m ? cbase[wi] + ia * cld[wi] : -1;
            off_b[tid] = ib < m ? cbase[wi] + ib * cld[wi] : -1;
        }
        int any = cls == nullptr;
        if (!any && tid < WD_TILE) {
            const int64_t i = a0 + tid;
            for (int c = 0; c < WD_TILE && !any; c++) {
                const int64_t j = b0 + c;
                any = i < j && j < m && cls[cb + tri_index(i, j, m)] == ETM_CAND_COUNT;
            }
        }
        if (!__syncthreads_or(any)) continue;

        if (warp < WD_MMA_WARP) {
            // ---- producers: thread t expands A row t (t < 256) or B row t - 256 ----
            constexpr int PF = 4;
            constexpr int BW = PF * WORDS_PER_STAGE;
            const bool is_b = tid >= WD_TILE;
            const int prow = is_b ? tid - WD_TILE : tid;
            const bool idle = !is_b && diag;  // on a diagonal block pair the A rows are the B rows
            const int64_t off = idle ? -1 : (is_b ? off_b[prow] : off_a[prow]);
            // Row r of a 256-row operand: half r / 128 (16 KB apart), row r % 128 of the half.
            const int dst = (is_b ? 2 * WD_HALF : 0) + (prow >> 7) * WD_HALF;
            const int hrow = prow & 127;
            uint64_t cur[BW], nxt[BW];
            auto load_batch = [&](int64_t s0, uint64_t* x) {
#pragma unroll
                for (int q = 0; q < BW; q += 2) {
                    ulonglong2 v = make_ulonglong2(0, 0);
                    if (off >= 0) v = __ldg(reinterpret_cast<const ulonglong2*>(src + off + s0 * WORDS_PER_STAGE + q));
                    x[q] = v.x;
                    x[q + 1] = v.y;
                }
            };
            if (n_stages > 0) load_batch(0, cur);
            for (int64_t s0 = 0; s0 < n_stages && !*abort_flag; s0 += PF) {
                if (s0 + PF < n_stages) load_batch(s0 + PF, nxt);
#pragma unroll
                for (int j = 0; j < PF; j++) {
                    const int64_t s = s0 + j;
                    if (s >= n_stages) break;
                    const int64_t G = gstage + s;
                    const int slot = (int)(G % WD_STAGES);
                    const uint32_t use = (uint32_t)(G / WD_STAGES);
                    if (!mbar_wait(&empty_bar[slot], (use & 1u) ^ 1u, abort_flag)) break;
                    if (!idle) {
                        const uint64_t x0 = cur[j * WORDS_PER_STAGE];
                        const uint64_t x1 = WORDS_PER_STAGE == 2 ? cur[j * WORDS_PER_STAGE + 1] : 0ULL;
                        store_row<ELEM>(slots + slot * WD_SLOT + dst, hrow, x0, x1);
                        fence_proxy_async();
                    }
                    mbar_arrive(&full_bar[slot]);
                }
#pragma unroll
                for (int q = 0; q < BW; q++) cur[q] = nxt[q];
            }
            // ---- epilogue: warp w reads lanes 32 (w % 4) .. of accumulator (w / 8), columns 128 ((w / 4) % 2) .. ----
            const bool ok = n_stages == 0 || mbar_wait(&acc_bar, tile_iter & 1u, abort_flag);
            if (ok) {
                tc_fence_after();
                const int lane_base = (warp & 3) * 32;
                const int accn = warp >> 3;
                const int64_t i = a0 + accn * 128 + lane_base + lane;
                for (int q = 0; q < 4; q++) {
                    const int col0 = ((warp >> 2) & 1) * 128 + q * 32;
                    uint32_t v[32];
                    if (n_stages > 0) {
                        const uint32_t taddr = tmem + ((uint32_t)lane_base << 16) + (uint32_t)(accn * 256 + col0);
                        asm volatile(
                            "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,"
                            "%14,%15,%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
                            : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]),
                              "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]),
                              "=r"(v[14]), "=r"(v[15]), "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]),
                              "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]), "=r"(v[24]), "=r"(v[25]),
                              "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
                            : "r"(taddr));
                        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
                    } else {
#pragma unroll
                        for (int c = 0; c < 32; c++) v[c] = 0u;
                    }
                    if (i < m) {
#pragma unroll
                        for (int c = 0; c < 32; c++) {
                            const int64_t j = b0 + col0 + c;
                            if (i < j && j < m) {
                                const int64_t t = cb + tri_index(i, j, m);
                                if (cls == nullptr || cls[t] == ETM_CAND_COUNT)
                                    out[t] = n_stages > 0 ? __float2int_rn(__uint_as_float(v[c]) * count_scale<ELEM>()) : 0;
                            }
                        }
                    }
                }
            }
            tc_fence_before();
        } else if (lane == 0) {
            // ---- MMA issuer: two M = 128 MMAs per K step, sharing the B tile ----
            tc_fence_after();
            for (int64_t s = 0; s < n_stages; s++) {
                const int64_t G = gstage + s;
                const int slot = (int)(G % WD_STAGES);
                const uint32_t use = (uint32_t)(G / WD_STAGES);
                if (!mbar_wait(&full_bar[slot], use & 1u, abort_flag)) break;
                tc_fence_after();
                const uint32_t base = smem_u32(slots + slot * WD_SLOT);
                const uint32_t b_addr = base + 2 * WD_HALF;
                const uint32_t a_addr = diag ? b_addr : base;
#pragma unroll
                for (int k = 0; k < 4; k++) {
                    const uint32_t acc = (s > 0 || k > 0) ? 1u : 0u;
                    const uint64_t bd = smem_desc(b_addr + 32 * k);
                    mma_ss<ELEM>(tmem, smem_desc(a_addr + 32 * k), bd, acc);
                    mma_ss<ELEM>(tmem + 256, smem_desc(a_addr + WD_HALF + 32 * k), bd, acc);
                }
                mma_commit(&empty_bar[slot]);
            }
            mma_commit(&acc_bar);
        }
        gstage += n_stages;
        tile_iter += 1;
        __syncthreads();
        if (*abort_flag) break;
    }

    if (warp == WD_MMA_WARP) {
        if (lane == 0 && *abort_flag) {
            mma_commit(&drain_bar);
            long long n = 0;
            while (!mbar_test(&drain_bar, 0) && ++n < WAIT_LIMIT) __nanosleep(64);
        }
        __syncwarp();
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TC_TMEM_COLS) : "memory");
    }
    if (tid == 0 && *abort_flag) atomicExch(&g_tc_status, ETM_ETIMEOUT);
}

template <int ELEM>
int launch_gram_wide(const uint64_t* cbuf, const int64_t* cbase, const int64_t* cwords, const int64_t* cld,
                     const int32_t* grp_size, const int64_t* cand_off, const int64_t* work_groups,
                     const int64_t* work_off, int64_t n_work, int64_t n_tiles, int64_t chunk_base, const uint8_t* cls,
                     int32_t* out, int64_t* work_counter, cudaStream_t s) {
    static bool configured = false;
    if (!configured) {
        ETM_CUDA(cudaFuncSetAttribute(gram_wide_kernel<ELEM>, cudaFuncAttributeMaxDynamicSharedMemorySize, WD_SMEM));
        configured = true;
    }
    const int64_t sms = max(1, sm_count());
    const int grid = (int)max64(1, min64(sms, n_tiles > 0 ? n_tiles : sms));
    if (work_counter != nullptr) ETM_CUDA(cudaMemsetAsync(work_counter, 0, sizeof(int64_t), s));
    gram_wide_kernel<ELEM><<<grid, WD_THREADS, WD_SMEM, s>>>(cbuf, cbase, cwords, cld, grp_size, cand_off, work_groups,
                                                             work_off, n_work, chunk_base, cls, out,
                                                             reinterpret_cast<unsigned long long*>(work_counter));
    ETM_LAUNCHED("gram_tc");
    return ETM_OK;
}

// ---------------------------------------------------------------------------------------------
// CTA-pair form (cta_group::2). A cluster of two CTAs on two SMs computes a 256 x 256 block pair
// with one M = 256, N = 256 MMA per K step: CTA r holds A rows 128 r .. 128 r + 127 and B rows
// 128 r .. 128 r + 127 of the blocks, the leader (rank 0) issues the MMAs and each CTA's tensor
// memory receives its 128 A rows against all 256 B rows. Per SM and unit of MMA work this stages
// 256 operand rows instead of 384 (128 on a diagonal block pair, where a CTA's A rows are its own
// B rows) and the tensor cores read a third less shared memory.
//
// Hand-over: every producer warp of both CTAs arrives (one elected lane, cluster-scope release)
// on the leader's full barrier of the stage; the leader's commits arrive on the empty and
// accumulator barriers of both CTAs (multicast). Per block pair the two CTAs take the same
// decisions (skip, abort) from values exchanged through distributed shared memory between
// cluster barriers, so both always execute the same sequence of cluster barriers.
//
// Tensor memory: each CTA allocates PR_TMEM_COLS columns with cta_group::2 and the MMAs and both
// epilogues use the leader's columns.
//
// Measured on GB300 (16 groups of 1,280 members over 131,072 projected rows): exact, but 3.3 ms
// against 2.6 ms for gram_tc_kernel; without the operand stores it still takes 2.4 ms, so the pair's
// cross-SM hand-over (remote arrivals, multicast commits) costs more than the shared-memory traffic it
// saves. The engine keeps the single-CTA kernel by default; ETM_TC_PAIR selects this one.
constexpr int PR_ROWS = 128;                     // A rows and B rows per CTA
constexpr int PR_TILE = 256;                     // members per block
constexpr int PR_STAGES = 6;
constexpr int PR_PRODUCERS = 2 * PR_ROWS;        // thread t < 128: A row t; else B row t - 128
constexpr int PR_PWARPS = PR_PRODUCERS / 32;
constexpr int PR_THREADS = PR_PRODUCERS + 32;
constexpr int PR_MMA_WARP = PR_PRODUCERS / 32;
constexpr uint32_t PR_TMEM_COLS = 256;
constexpr int PR_HALF = PR_ROWS * 128;           // bytes of one 128-row operand tile
constexpr int PR_SLOT = 2 * PR_HALF;             // A tile, then B tile
// + 1024 for the alignment of the slots, + one spare half tile after the last slot.
constexpr int PR_SMEM = PR_STAGES * PR_SLOT + 1024 + PR_HALF;

__device__ __forceinline__ uint32_t cluster_rank() {
    uint32_t r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
}
__device__ __forceinline__ void cluster_sync() {
    asm volatile("barrier.cluster.arrive.release.aligned;\nbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}
__device__ __forceinline__ uint32_t map_to(uint32_t saddr, uint32_t rank) {
    uint32_t r;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(saddr), "r"(rank));
    return r;
}
__device__ __forceinline__ uint32_t ld_cluster_u32(uint32_t caddr) {
    uint32_t v;
    asm volatile("ld.shared::cluster.u32 %0, [%1];" : "=r"(v) : "r"(caddr) : "memory");
    return v;
}
__device__ __forceinline__ void arrive_cluster(uint32_t caddr) {
    asm volatile("mbarrier.arrive.release.cluster.shared::cluster.b64 _, [%0];" ::"r"(caddr) : "memory");
}
__device__ __forceinline__ bool mbar_try_cluster(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.acquire.cluster.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
__device__ bool mbar_wait_cluster(uint64_t* bar, uint32_t parity, volatile int* abort_flag) {
    long long n = 0;
    while (!mbar_try_cluster(bar, parity)) {
        if (*abort_flag) return false;
        if (++n > WAIT_LIMIT) {
            *abort_flag = 1;
            return false;
        }
    }
    return true;
}
__device__ __forceinline__ void commit_pair(uint64_t* bar) {
    asm volatile(
        "{\n .reg .b16 msk;\n mov.b16 msk, 3;\n"
        " tcgen05.commit.cta_group::2.mbarrier::arrive::one.shared::cluster.multicast::cluster.b64 [%0], msk;\n}\n"
        ::"r"(smem_u32(bar))
        : "memory");
}
__device__ __forceinline__ void commit_pair_local(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::2.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}
// Instruction descriptor of the pair MMA: D f32, A/B format code 0, K-major, N = 256, M = 256.
__host__ __device__ constexpr uint32_t pair_desc() { return (1u << 4) | (256u >> 3) << 17 | (256u >> 4) << 24; }

template <int ELEM>
__device__ __forceinline__ void mma_pair(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t acc) {
    if constexpr (ELEM == 2) {
        asm volatile(
            "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
            " tcgen05.mma.cta_group::2.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
            "l"(a), "l"(b), "r"(pair_desc()), "r"(acc));
    } else {
        asm volatile(
            "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
            " tcgen05.mma.cta_group::2.kind::f8f6f4 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
            "l"(a), "l"(b), "r"(pair_desc()), "r"(acc));
    }
}

template <int ELEM>
__global__ void __cluster_dims__(2, 1, 1) __launch_bounds__(PR_THREADS, 1) gram_pair_kernel(
    const uint64_t* __restrict__ src, const int64_t* __restrict__ cbase, const int64_t* __restrict__ cwords,
    const int64_t* __restrict__ cld, const int32_t* __restrict__ grp_size, const int64_t* __restrict__ cand_off,
    const int64_t* __restrict__ work_groups, const int64_t* __restrict__ work_off, int64_t n_work, int64_t chunk_base,
    const uint8_t* __restrict__ cls, int32_t* __restrict__ out) {
    constexpr int WORDS_PER_STAGE = ELEM == 2 ? 1 : 2;
    extern __shared__ uint8_t dsmem[];
    __shared__ __align__(8) uint64_t full_bar[PR_STAGES];   // the leader's: 2 x PR_PWARPS warp arrivals
    __shared__ __align__(8) uint64_t empty_bar[PR_STAGES];  // each CTA's: the leader's commit
    __shared__ __align__(8) uint64_t acc_bar;
    __shared__ __align__(8) uint64_t drain_bar;
    __shared__ uint32_t tmem_sh;
    __shared__ int abort_sh;
    __shared__ int any_sh[2];    // per block-pair parity: this CTA has a candidate to count
    __shared__ int stop_sh[2];   // per block-pair parity: this CTA aborted
    __shared__ int64_t off_a[PR_ROWS];
    __shared__ int64_t off_b[PR_ROWS];

    uint8_t* slots = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(dsmem) + 1023) & ~uintptr_t(1023));
    const int tid = threadIdx.x;
    const int warp = tid >> 5, lane = tid & 31;
    const uint32_t rank = cluster_rank();
    const uint32_t peer = rank ^ 1u;

    if (tid == 0) {
        for (int s = 0; s < PR_STAGES; s++) {
            mbar_init(&full_bar[s], 2 * PR_PWARPS);
            mbar_init(&empty_bar[s], 1);
        }
        mbar_init(&acc_bar, 1);
        mbar_init(&drain_bar, 1);
        abort_sh = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == PR_MMA_WARP) {
        asm volatile("tcgen05.alloc.cta_group::2.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_sh)),
                     "r"(PR_TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::2.sync.aligned;" ::: "memory");
        tc_fence_before();
    }
    cluster_sync();
    tc_fence_after();
    const uint32_t tmem_own = tmem_sh;
    const uint32_t tmem = rank == 0 ? tmem_own : ld_cluster_u32(map_to(smem_u32(&tmem_sh), 0));
    volatile int* abort_flag = &abort_sh;

    const int64_t total = work_off[n_work];
    const int64_t pair = blockIdx.x >> 1, n_pairs = gridDim.x >> 1;
    int64_t gstage = 0;
    uint32_t tile_iter = 0;
    int par = 0;
    for (int64_t tp = pair; tp < total; tp += n_pairs, par ^= 1) {
        const int64_t wi = upper_find(work_off, n_work, tp);
        const int64_t g = work_groups[wi];
        const int64_t m = grp_size[g];
        const int64_t nb = ceil_div<int64_t>(m, PR_TILE);
        int64_t ua, ub1;
        tri_decode(tp - work_off[wi], nb + 1, &ua, &ub1);
        const int64_t ub = ub1 - 1;
        const bool diag = ua == ub;
        const int64_t a0 = ua * PR_TILE + rank * PR_ROWS;  // this CTA's A rows
        const int64_t b0 = ub * PR_TILE + rank * PR_ROWS;  // this CTA's B rows
        const int64_t bcol0 = ub * PR_TILE;                // the accumulator's 256 columns
        const int64_t cb = cand_off[g] - chunk_base;
        const int64_t words = cwords[wi];
        const int64_t n_stages = ceil_div<int64_t>(words, WORDS_PER_STAGE);
        if (tid < PR_ROWS) {
            const int64_t ia = a0 + tid, ib = b0 + tid;
            off_a[tid] = ia < m ? cbase[wi] + ia * cld[wi] : -1;
            off_b[tid] = ib < m ? cbase[wi] + ib * cld[wi] : -1;
        }
        int any = cls == nullptr;
        if (!any && tid < PR_ROWS) {
            const int64_t i = a0 + tid;
            for (int c = 0; c < PR_TILE && !any; c++) {
                const int64_t j = bcol0 + c;
                any = i < j && j < m && cls[cb + tri_index(i, j, m)] == ETM_CAND_COUNT;
            }
        }
        any = __syncthreads_or(any);
        if (tid == 0) any_sh[par] = any;
        cluster_sync();
        const int pair_any = any | (int)ld_cluster_u32(map_to(smem_u32(&any_sh[par]), peer));
        if (!pair_any) continue;  // both CTAs skip the block pair

        if (warp < PR_MMA_WARP) {
            // ---- producers: thread t expands A row t (t < 128) or B row t - 128 of this CTA ----
            constexpr int PF = 4;
            constexpr int BW = PF * WORDS_PER_STAGE;
            const bool is_b = tid >= PR_ROWS;
            const int prow = is_b ? tid - PR_ROWS : tid;
            const bool idle = !is_b && diag;  // on a diagonal pair the A rows are this CTA's B rows
            const int64_t off = idle ? -1 : (is_b ? off_b[prow] : off_a[prow]);
            uint64_t cur[BW], nxt[BW];
            auto load_batch = [&](int64_t s0, uint64_t* x) {
#pragma unroll
                for (int q = 0; q < BW; q += 2) {
                    ulonglong2 v = make_ulonglong2(0, 0);
                    if (off >= 0) v = __ldg(reinterpret_cast<const ulonglong2*>(src + off + s0 * WORDS_PER_STAGE + q));
                    x[q] = v.x;
                    x[q + 1] = v.y;
                }
            };
            if (n_stages > 0) load_batch(0, cur);
            for (int64_t s0 = 0; s0 < n_stages && !*abort_flag; s0 += PF) {
                if (s0 + PF < n_stages) load_batch(s0 + PF, nxt);
#pragma unroll
                for (int j = 0; j < PF; j++) {
                    const int64_t s = s0 + j;
                    if (s >= n_stages) break;
                    const int64_t G = gstage + s;
                    const int slot = (int)(G % PR_STAGES);
                    const uint32_t use = (uint32_t)(G / PR_STAGES);
                    if (!mbar_wait(&empty_bar[slot], (use & 1u) ^ 1u, abort_flag)) break;
                    if (!idle) {
                        const uint64_t x0 = cur[j * WORDS_PER_STAGE];
                        const uint64_t x1 = WORDS_PER_STAGE == 2 ? cur[j * WORDS_PER_STAGE + 1] : 0ULL;
                        store_row<ELEM>(slots + slot * PR_SLOT + (is_b ? PR_HALF : 0), prow, x0, x1);
                        fence_proxy_async();  // this CTA's tile, read by the pair's MMA through its own SM
                    }
                    __syncwarp();
                    if (lane == 0) arrive_cluster(map_to(smem_u32(&full_bar[slot]), 0));
                }
#pragma unroll
                for (int q = 0; q < BW; q++) cur[q] = nxt[q];
            }
            // ---- epilogue: warp w reads TMEM lanes 32 (w % 4) .., columns 128 (w / 4) .. +127 ----
            const bool ok = n_stages == 0 || mbar_wait(&acc_bar, tile_iter & 1u, abort_flag);
            if (ok) {
                tc_fence_after();
                const int lane_base = (warp & 3) * 32;
                const int64_t i = a0 + lane_base + lane;
                for (int q = 0; q < 4; q++) {
                    const int col0 = (warp >> 2) * 128 + q * 32;
                    uint32_t v[32];
                    if (n_stages > 0) {
                        const uint32_t taddr = tmem + ((uint32_t)lane_base << 16) + (uint32_t)col0;
                        asm volatile(
                            "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,"
                            "%14,%15,%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
                            : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]),
                              "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]),
                              "=r"(v[14]), "=r"(v[15]), "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]),
                              "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]), "=r"(v[24]), "=r"(v[25]),
                              "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
                            : "r"(taddr));
                        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
                    } else {
#pragma unroll
                        for (int c = 0; c < 32; c++) v[c] = 0u;
                    }
                    if (i < m) {
#pragma unroll
                        for (int c = 0; c < 32; c++) {
                            const int64_t j = bcol0 + col0 + c;
                            if (i < j && j < m) {
                                const int64_t t = cb + tri_index(i, j, m);
                                if (cls == nullptr || cls[t] == ETM_CAND_COUNT)
                                    out[t] = n_stages > 0 ? __float2int_rn(__uint_as_float(v[c]) * count_scale<ELEM>()) : 0;
                            }
                        }
                    }
                }
            }
            tc_fence_before();
        } else if (rank == 0 && lane == 0) {
            // ---- MMA issuer (the leader) ----
            tc_fence_after();
            for (int64_t s = 0; s < n_stages; s++) {
                const int64_t G = gstage + s;
                const int slot = (int)(G % PR_STAGES);
                const uint32_t use = (uint32_t)(G / PR_STAGES);
                if (!mbar_wait_cluster(&full_bar[slot], use & 1u, abort_flag)) break;
                tc_fence_after();
                const uint32_t base = smem_u32(slots + slot * PR_SLOT);
                const uint32_t b_addr = base + PR_HALF;
                const uint32_t a_addr = diag ? b_addr : base;
#pragma unroll
                for (int k = 0; k < 4; k++) {
                    const uint32_t acc = (s > 0 || k > 0) ? 1u : 0u;
                    mma_pair<ELEM>(tmem, smem_desc(a_addr + 32 * k), smem_desc(b_addr + 32 * k), acc);
                }
                commit_pair(&empty_bar[slot]);
            }
            commit_pair(&acc_bar);
        }
        gstage += n_stages;
        tile_iter += 1;
        __syncthreads();
        if (tid == 0) stop_sh[par] = *abort_flag;
        cluster_sync();  // the accumulator is read in both CTAs; both stop flags are set
        const int stop = *abort_flag | (int)ld_cluster_u32(map_to(smem_u32(&stop_sh[par]), peer));
        if (stop) {
            *abort_flag = 1;
            break;
        }
    }

    // Teardown: the leader waits (bounded) for any MMA still in flight, then both CTAs free tensor memory.
    if (rank == 0 && warp == PR_MMA_WARP && lane == 0 && *abort_flag) {
        commit_pair_local(&drain_bar);
        long long n = 0;
        while (!mbar_test(&drain_bar, 0) && ++n < WAIT_LIMIT) __nanosleep(64);
    }
    __syncthreads();
    cluster_sync();
    if (warp == PR_MMA_WARP) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::2.sync.aligned.b32 %0, %1;" ::"r"(tmem_own), "r"(PR_TMEM_COLS)
                     : "memory");
    }
    if (tid == 0 && *abort_flag) atomicExch(&g_tc_status, ETM_ETIMEOUT);
}

template <int ELEM>
int launch_gram_pair(const uint64_t* cbuf, const int64_t* cbase, const int64_t* cwords, const int64_t* cld,
                     const int32_t* grp_size, const int64_t* cand_off, const int64_t* work_groups,
                     const int64_t* work_off, int64_t n_work, int64_t n_tiles, int64_t chunk_base, const uint8_t* cls,
                     int32_t* out, int64_t* /*work_counter: items go round-robin*/, cudaStream_t s) {
    static bool configured = false;
    static int max_clusters = 0;
    if (!configured) {
        ETM_CUDA(cudaFuncSetAttribute(gram_pair_kernel<ELEM>, cudaFuncAttributeMaxDynamicSharedMemorySize, PR_SMEM));
        // Persistent clusters: as many as can be resident at once (SM pairs within a GPC).
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(2 * max(1, sm_count() / 2));
        cfg.blockDim = dim3(PR_THREADS);
        cfg.dynamicSmemBytes = PR_SMEM;
        cudaLaunchAttribute attr;
        attr.id = cudaLaunchAttributeClusterDimension;
        attr.val.clusterDim.x = 2;
        attr.val.clusterDim.y = 1;
        attr.val.clusterDim.z = 1;
        cfg.attrs = &attr;
        cfg.numAttrs = 1;
        ETM_CUDA(cudaOccupancyMaxActiveClusters(&max_clusters, gram_pair_kernel<ELEM>, &cfg));
        configured = true;
    }
    const int64_t pairs = max(1, min(max_clusters, sm_count() / 2));
    const int grid = 2 * (int)max64(1, min64(pairs, n_tiles > 0 ? n_tiles : pairs));
    gram_pair_kernel<ELEM><<<grid, PR_THREADS, PR_SMEM, s>>>(cbuf, cbase, cwords, cld, grp_size, cand_off,
                                                             work_groups, work_off, n_work, chunk_base, cls, out);
    ETM_LAUNCHED("gram_tc");
    return ETM_OK;
}

}  // namespace

namespace etm {

int gram_tc(const uint64_t* cbuf, const int64_t* cbase, const int64_t* cwords, const int64_t* cld,
            const int32_t* grp_size, const int64_t* cand_off, const int64_t* work_groups, const int64_t* work_off,
            int64_t n_work, int64_t n_tiles, int64_t chunk_base, const uint8_t* cls, int32_t elem, int32_t* out,
            int64_t* work_counter, cudaStream_t s) {
    // elem: 1 = e4m3, 2 = f16; + ETM_TC_A_TMEM: the A operand is staged in tensor memory
    // (tcgen05.st) instead of shared memory; + ETM_TC_PAIR: the CTA-pair kernel (cta_group::2).
    const bool a_tmem = (elem & ETM_TC_A_TMEM) != 0;
    const bool pair = (elem & ETM_TC_PAIR) != 0;
    const bool wide = (elem & ETM_TC_WIDE) != 0;
    const int e = elem & ~(ETM_TC_A_TMEM | ETM_TC_PAIR | ETM_TC_WIDE);
    ETM_REQUIRE(e == 1 || e == 2, ETM_EINVAL, "gram_tc: element code %d (1 = e4m3, 2 = f16)", e);
    ETM_REQUIRE(!(pair && a_tmem), ETM_EINVAL, "gram_tc: the CTA-pair form stages both operands in shared memory");
#define ETM_GRAM_ARGS cbuf, cbase, cwords, cld, grp_size, cand_off, work_groups, work_off, n_work, n_tiles, chunk_base, cls, out, work_counter, s
    ETM_REQUIRE(!(wide && (pair || a_tmem)), ETM_EINVAL, "gram_tc: ETM_TC_WIDE combines with no other flag");
    if (pair) return e == 2 ? launch_gram_pair<2>(ETM_GRAM_ARGS) : launch_gram_pair<1>(ETM_GRAM_ARGS);
    if (wide) return e == 2 ? launch_gram_wide<2>(ETM_GRAM_ARGS) : launch_gram_wide<1>(ETM_GRAM_ARGS);
    if (e == 2) return a_tmem ? launch_gram<2, true>(ETM_GRAM_ARGS) : launch_gram<2, false>(ETM_GRAM_ARGS);
    return a_tmem ? launch_gram<1, true>(ETM_GRAM_ARGS) : launch_gram<1, false>(ETM_GRAM_ARGS);
#undef ETM_GRAM_ARGS
}

int count_tiles_tensor(const uint64_t*, int64_t, int64_t, const int32_t*, int32_t, const int64_t*, const int32_t*,
                       const int64_t*, const int64_t*, const int64_t*, int64_t, int64_t, const uint8_t*, int32_t*,
                       cudaStream_t) {
    set_error("etm_count_tiles: the tensor method counts projected groups; use etm_count_tiles_tc");
    return ETM_EINVAL;
}

}  // namespace etm

extern "C" int etm_count_tiles_tc(const uint64_t* cbuf, const int64_t* cbase, const int64_t* cwords,
                                  const int64_t* cld, const int32_t* grp_size, const int64_t* cand_off,
                                  const int64_t* work_groups, const int64_t* work_off, int64_t n_work,
                                  int64_t n_tiles, int64_t chunk_base, const uint8_t* cls, int32_t elem,
                                  int32_t* out_counts, int64_t* work_counter, void* stream) {
    ETM_REQUIRE((reinterpret_cast<uintptr_t>(cbuf) & 15) == 0, ETM_EINVAL, "etm_count_tiles_tc: cbuf must be 16-byte aligned");
    if (n_work <= 0) return ETM_OK;
    return etm::gram_tc(cbuf, cbase, cwords, cld, grp_size, cand_off, work_groups, work_off, n_work, n_tiles,
                        chunk_base, cls, elem, out_counts, work_counter, as_stream(stream));
}

extern "C" int etm_device_status(void* stream) {
    int v = 0;
    ETM_CUDA(cudaMemcpyFromSymbolAsync(&v, g_tc_status, sizeof(int), 0, cudaMemcpyDeviceToHost, as_stream(stream)));
    ETM_CUDA(cudaStreamSynchronize(as_stream(stream)));
    if (v != 0) {
        const int zero = 0;
        ETM_CUDA(cudaMemcpyToSymbolAsync(g_tc_status, &zero, sizeof(int), 0, cudaMemcpyHostToDevice, as_stream(stream)));
        ETM_CUDA(cudaStreamSynchronize(as_stream(stream)));
        etm::set_error("a tensor-core counting kernel gave up a bounded wait (status %d)", v);
        return v;
    }
    int p = 0;
    const int st = etm::proj_status_take(as_stream(stream), &p);
    if (st != ETM_OK) return st;
    if (p != 0) etm::set_error("the projection gave up a bounded wait for its bulk copies (status %d)", p);
    return p;
}
