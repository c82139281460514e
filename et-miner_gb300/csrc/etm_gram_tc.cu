// Exact 0/1 Gram of prefix-group suffixes on the tcgen05 tensor cores.
//
// For a group whose members are bit rows x_0..x_{m-1} (projected suffix
// words, or for K=2 the frequent columns themselves), the pair counts are
// C[i][j] = popcount(x_i & x_j) = sum_r x_i[r] * x_j[r]: the Gram matrix X X^T
// of a 0/1 matrix. One persistent kernel (one CTA per SM) computes it by
// block pairs: the members are cut into blocks of T, and a CTA takes a whole
// block pair (ua <= ub) at a time.
//
//   producers  512 threads, one operand row each (thread t < 256: row t of
//              block ua, else row t - 256 of block ub): per stage they load
//              the row's next bits (prefetched PF stages ahead into
//              registers), expand them into 128 bytes of operand elements
//              in the 128-byte swizzled K-major layout the MMA reads
//              (SWIZZLE_128B), then fence.proxy.async and an mbarrier
//              arrive. A diagonal block pair stages only the B rows and
//              reads A from them.
//   MMA        one thread issues, per 32-byte K step, two M = 128 MMAs that
//              share the B tile (A halves: the first and last T/2 rows of
//              block ua) into two f32 accumulators in tensor memory;
//              tcgen05.commit frees each stage and finally signals the
//              epilogue.
//   epilogue   the producer warps read the accumulators back with
//              tcgen05.ld and emit the i < j pair counts at their
//              lexicographic candidate slots: every count (dense), or only
//              the counts reaching min_count plus a survivor bit each
//              (fused threshold).
//
// Operand formats (the element a set bit becomes, and what a product is):
//
//   FMT 1  e4m3 under kind::f8f6f4, T = 256, 128 bits per stage row:
//          0x01 = 2^-9, products 2^-18.
//   FMT 2  f16 under kind::f16, T = 256, 64 bits per stage row:
//          0x0001 = 2^-24, products 2^-48.
//   FMT 4  packed e2m1 under kind::mxf4 (block scale 2X, every ue8m0 scale
//          factor 127 = 1.0), T = 240, 256 bits per stage row: 0b0001 =
//          0.5, products 0.25. The two 240-column accumulators take TMEM
//          columns 0-479 and the scale factors 480-511, so a block holds
//          240 members (each A half 120 rows of a 128-row MMA; rows 120-127
//          are not read back).
//
// Exactness: every product is one power of two s and every partial sum is
// c * s with an integer c below 2^24 (the caller sends only groups of at
// most 2^24 rows here): exact in f32, and scaled back exactly to c.
//
// Bit expansion: the order of the transactions along K does not change a
// Gram entry, as long as every row uses the same order. So a 32-bit piece v
// of a row is spread by shifts: word q of an output chunk is (v >> q) & M
// with M = 0x11111111 (e2m1 nibbles), 0x01010101 (e4m3 bytes) or
// 0x00010001 (f16 halves); two operations per output word, the same
// permutation in every row.
//
// Every mbarrier wait is bounded in time (%globaltimer): after the limit the
// block raises an abort flag, every thread leaves its loop, the MMA thread
// waits (bounded) for its issued MMAs, TMEM is freed, and the kernel records
// ETM_ETIMEOUT in its status word instead of hanging.
#include <cstdlib>
#include <mutex>

#include "etm_count.cuh"

namespace {

using namespace etm;

constexpr int PRODUCERS = 512;                 // thread t < 256: A row t; else B row t - 256
constexpr int THREADS = PRODUCERS + 32;
constexpr int MMA_WARP = PRODUCERS / 32;
constexpr int STAGES = 3;
constexpr int HALF_BYTES = 128 * 128;          // one 128-row operand tile of 128-byte rows
constexpr int SLOT_BYTES = 4 * HALF_BYTES;     // A (two 128-row halves), then B (256 rows)
constexpr int SMEM_BYTES = STAGES * SLOT_BYTES + 1024;
// Staged form (packed e2m1 over blocked rows): a loader warp copies each stage's raw bits (the block's
// 32-byte chunk of every member: T x 32 bytes per block, one contiguous run in the blocked layout) into a
// ring of RAW_STAGES shared-memory slots with bulk copies; the producers expand from there. Two operand
// stages leave room for the ring.
constexpr int ST_OPS = 2;
constexpr int RAW_STAGES = 5;
constexpr int RAW_BLOCK = 240 * 32;             // one block's raw chunk: 240 members x 32 bytes
constexpr int RAW_SLOT = 2 * RAW_BLOCK;         // A block, then B block
constexpr int ST_THREADS = PRODUCERS + 64;      // producers, the MMA warp, the loader warp
constexpr int LOAD_WARP = MMA_WARP + 1;
constexpr int ST_SMEM = ST_OPS * SLOT_BYTES + RAW_STAGES * RAW_SLOT + 1024;
static_assert(ST_SMEM <= 227 * 1024 - 8192, "staged shared memory");
constexpr uint32_t TMEM_COLS = 512;
constexpr uint32_t SF_COL = 480;               // FMT 4: scale factors in TMEM columns 480-511
constexpr uint64_t WAIT_NS = 2000000000ull;    // every bounded wait: 2 s

template <int FMT>
struct Fmt;
template <>
struct Fmt<1> {  // e4m3
    static constexpr int T = 256, WORDS = 2, PF = 4;
    static constexpr float SCALE = 262144.0f;  // 2^18
};
template <>
struct Fmt<2> {  // f16
    static constexpr int T = 256, WORDS = 1, PF = 4;
    static constexpr float SCALE = 281474976710656.0f;  // 2^48
};
template <>
struct Fmt<4> {  // e2m1, block-scaled with unit scales
    static constexpr int T = 240, WORDS = 4, PF = 2;
    static constexpr float SCALE = 4.0f;
};

__device__ int g_tc_status;

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ uint64_t now_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

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

// Waits for the phase of `parity` to complete; false if the block aborts or `limit_ns` passes first
// (then the abort flag is raised). A limit of 0 gives up at once: the give-up path's test hook.
__device__ bool mbar_wait(uint64_t* bar, uint32_t parity, volatile int* abort_flag, uint64_t limit_ns) {
    if (limit_ns == 0) {
        *abort_flag = 1;
        return false;
    }
    if (mbar_try(bar, parity)) return true;
    const uint64_t t0 = now_ns();
    while (!mbar_try(bar, parity)) {
        if (*abort_flag) return false;
        if (now_ns() - t0 > limit_ns) {
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

// Instruction descriptor, M = 128, N = T, both operands K-major.
//   FMT 1, 2: D f32 (bits 4-5 = 1), A/B format 0 (e4m3 under kind::f8f6f4, f16 under kind::f16).
//   FMT 4 (block-scaled): A/B format 1 (e2m1 under kind::mxf4) in bits 7-9 / 10-12, scale factors ue8m0
//   (bit 23), scale-factor ids 0 (bits 4-5, 29-30).
template <int FMT>
__host__ __device__ constexpr uint32_t instr_desc() {
    constexpr uint32_t n_m = ((uint32_t)(Fmt<FMT>::T >> 3) << 17) | ((uint32_t)(128 >> 4) << 24);
    if constexpr (FMT == 4) return n_m | (1u << 7) | (1u << 10) | (1u << 23);
    else return n_m | (1u << 4);
}

// D (TMEM) += A x B, both from shared-memory descriptors.
template <int FMT>
__device__ __forceinline__ void mma_ss(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t acc, uint32_t tmem_sf) {
    if constexpr (FMT == 2) {
        asm volatile(
            "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
            " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
            "l"(a), "l"(b), "r"(instr_desc<FMT>()), "r"(acc));
    } else if constexpr (FMT == 1) {
        asm volatile(
            "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
            " tcgen05.mma.cta_group::1.kind::f8f6f4 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
            "l"(a), "l"(b), "r"(instr_desc<FMT>()), "r"(acc));
    } else {
        // Scale factors of A at tmem_sf, of B 16 columns on; every byte of those columns is 127 (2^0).
        asm volatile(
            "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
            " tcgen05.mma.cta_group::1.kind::mxf4.block_scale.scale_vec::2X [%0], %1, %2, %3, [%5], [%6], p;\n}\n" ::"r"(
                tmem_d),
            "l"(a), "l"(b), "r"(instr_desc<FMT>()), "r"(acc), "r"(tmem_sf), "r"(tmem_sf + 16));
    }
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

// Bulk (TMA) copy of `bytes` (a multiple of 16, both addresses 16-byte aligned) from global to shared memory,
// completed on `bar` (complete_tx).
__device__ __forceinline__ void bulk_copy(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                 ::"r"(smem_u32(dst)), "l"(src), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}

// One operand row of the stage: Fmt::WORDS words of the row's bits, expanded into the eight 16-byte
// chunks of row r of a SWIZZLE_128B tile (logical chunk c lives at chunk c ^ (r % 8)).
template <int FMT>
__device__ __forceinline__ void store_row(uint8_t* tile, int r, const uint64_t* x) {
    uint8_t* row = tile + (r >> 3) * 1024 + (r & 7) * 128;
#pragma unroll
    for (int c = 0; c < 8; c++) {
        uint32_t v, mask;
        int q0;
        if constexpr (FMT == 4) {  // chunk c: the 32 bits of piece c as 32 nibbles
            v = (uint32_t)(x[c >> 1] >> (32 * (c & 1)));
            q0 = 0;
            mask = 0x11111111u;
        } else if constexpr (FMT == 1) {  // chunks 2p, 2p + 1: the 32 bits of piece p as 32 bytes
            v = (uint32_t)(x[c >> 2] >> (32 * ((c >> 1) & 1)));
            q0 = 4 * (c & 1);
            mask = 0x01010101u;
        } else {  // chunks 4p .. 4p + 3: the 32 bits of piece p as 32 halves
            v = (uint32_t)(x[0] >> (32 * (c >> 2)));
            q0 = 4 * (c & 3);
            mask = 0x00010001u;
        }
        const uint4 o = make_uint4((v >> q0) & mask, (v >> (q0 + 1)) & mask, (v >> (q0 + 2)) & mask,
                                   (v >> (q0 + 3)) & mask);
        *reinterpret_cast<uint4*>(row + ((c ^ (r & 7)) << 4)) = o;
    }
}

template <int FMT, bool STAGED>
__global__ void __launch_bounds__(STAGED ? ST_THREADS : THREADS, 1) gram_kernel(
    const uint64_t* __restrict__ src, const int64_t* __restrict__ cbase, const int64_t* __restrict__ cwords,
    const int64_t* __restrict__ cld, const int32_t* __restrict__ grp_size, const int64_t* __restrict__ cand_off,
    const int64_t* __restrict__ work_groups, const int64_t* __restrict__ work_off, int64_t n_work, int64_t chunk_base,
    const uint8_t* __restrict__ cls, int32_t min_count, int32_t* __restrict__ out, uint32_t* __restrict__ surv,
    unsigned long long* __restrict__ work_counter, uint64_t first_wait_ns, bool blocked) {
    constexpr int T = Fmt<FMT>::T;
    constexpr int TH = T / 2;  // A rows per accumulator
    constexpr int WORDS = Fmt<FMT>::WORDS;
    constexpr int PF = Fmt<FMT>::PF;
    constexpr int BW = PF * WORDS;
    constexpr int NST = STAGED ? ST_OPS : STAGES;  // operand stages
    static_assert(!STAGED || (FMT == 4 && T * 32 == RAW_BLOCK), "the staged form serves packed e2m1 operands");
    extern __shared__ uint8_t dsmem[];
    __shared__ __align__(8) uint64_t full_bar[NST];
    __shared__ __align__(8) uint64_t empty_bar[NST];
    __shared__ __align__(8) uint64_t raw_full[STAGED ? RAW_STAGES : 1];
    __shared__ __align__(8) uint64_t raw_empty[STAGED ? RAW_STAGES : 1];
    __shared__ __align__(8) uint64_t acc_bar;
    __shared__ __align__(8) uint64_t drain_bar;
    __shared__ uint32_t tmem_sh;
    __shared__ int abort_sh;
    // Member row offsets of the block pair (the producers of the unstaged form load their rows themselves).
    __shared__ int64_t off_a[STAGED ? 1 : 256];
    __shared__ int64_t off_b[STAGED ? 1 : 256];
    __shared__ int64_t next_sh;

    uint8_t* slots = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(dsmem) + 1023) & ~uintptr_t(1023));
    uint8_t* raw = slots + NST * SLOT_BYTES;  // staged form: RAW_STAGES slots of RAW_SLOT bytes
    const int tid = threadIdx.x;
    const int warp = tid >> 5, lane = tid & 31;

    if (tid == 0) {
        for (int s = 0; s < NST; s++) {
            mbar_init(&full_bar[s], PRODUCERS);
            mbar_init(&empty_bar[s], 1);
        }
        if constexpr (STAGED) {
            for (int s = 0; s < RAW_STAGES; s++) {
                mbar_init(&raw_full[s], 1);
                mbar_init(&raw_empty[s], PRODUCERS);
            }
        }
        mbar_init(&acc_bar, 1);
        mbar_init(&drain_bar, 1);
        abort_sh = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == MMA_WARP) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_sh)),
                     "r"(TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
        tc_fence_before();
    }
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_sh;
    volatile int* abort_flag = &abort_sh;
    if constexpr (FMT == 4) {
        // Unit scale factors: warp w (w < 4) fills lanes 32 w .. 32 w + 31 of columns 480-511 with 127s.
        if (warp < 4) {
            const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16) + SF_COL;
            const uint32_t u = 0x7F7F7F7Fu;
            asm volatile(
                "tcgen05.st.sync.aligned.32x32b.x32.b32 [%0], {%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,"
                "%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1};" ::"r"(taddr),
                "r"(u)
                : "memory");
            asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
        }
        tc_fence_before();
        __syncthreads();
        tc_fence_after();
    }

    const int64_t total = work_off[n_work];
    int64_t gstage = 0;
    int64_t raw_issued = 0;  // loader: stages whose raw copies were issued
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
        const int64_t nb = ceil_div<int64_t>(m, T);
        int64_t ua, ub1;
        tri_decode(tp - work_off[wi], nb + 1, &ua, &ub1);
        const int64_t ub = ub1 - 1;
        const bool diag = ua == ub;
        const int64_t a0 = ua * T, b0 = ub * T;
        const int64_t cb = cand_off[g] - chunk_base;
        const int64_t words = cwords[wi];
        const int64_t n_stages = ceil_div<int64_t>(words, WORDS);
        if (!STAGED && tid < 256) {
            const int64_t ia = a0 + tid, ib = b0 + tid;
            // Row-major rows: member i at cbase + i cld. Blocked rows (blocks of T members stored 4-word chunk
            // by chunk, each chunk as two 2-word halves, so a stage's words of one block are one run): member i
            // at cbase + (i / T) T cld + 2 (i % T).
            const int64_t cw = cld[wi];
            off_a[tid] = tid < T && ia < m ? cbase[wi] + (blocked ? ua * T * cw + 2 * tid : ia * cw) : -1;
            off_b[tid] = tid < T && ib < m ? cbase[wi] + (blocked ? ub * T * cw + 2 * tid : ib * cw) : -1;
        }
        int any = cls == nullptr;
        if (!any && tid < T) {
            const int64_t i = a0 + tid;
            for (int c = 0; c < T && !any; c++) {
                const int64_t j = b0 + c;
                any = i < j && j < m && cls[cb + tri_index(i, j, m)] == ETM_CAND_COUNT;
            }
        }
        if (!__syncthreads_or(any)) continue;

        if (warp < MMA_WARP) {
            // ---- producers ----
            const bool is_b = tid >= 256;
            const int prow = is_b ? tid - 256 : tid;
            const bool idle = prow >= T || (!is_b && diag);  // on a diagonal block pair the A rows are B rows
            const int64_t off = (STAGED || idle) ? -1 : (is_b ? off_b[prow] : off_a[prow]);
            // B row r: row r of the 256-row B tile; A row r: row r % TH of A half r / TH.
            const int dst = is_b ? 2 * HALF_BYTES : (prow / TH) * HALF_BYTES;
            const int hrow = is_b ? prow : prow % TH;
            if constexpr (STAGED) {
                // Raw bits from the loader's ring (A block at 0, B block at RAW_BLOCK of a slot): wait for the
                // slot, read this row's two 16-byte halves (words 0-1 at 16 prow, words 2-3 at 16 (T + prow):
                // a warp reads two contiguous 512-byte runs), expand them into the stage, then release the slot.
                // The release comes after the expansion has consumed the loaded words, so the loader's next
                // bulk copy into the slot (async proxy) cannot land before these reads (generic proxy) are done.
                const bool skip = idle || (is_b ? b0 : a0) + prow >= m;
                const int raw_off = (is_b ? RAW_BLOCK : 0) + prow * 16;
                for (int64_t s = 0; s < n_stages; s++) {
                    const int64_t G = gstage + s;
                    const int rs = (int)(G % RAW_STAGES);
                    const uint32_t ruse = (uint32_t)(G / RAW_STAGES);
                    const int os = (int)(G % NST);
                    const uint32_t ouse = (uint32_t)(G / NST);
                    if (!mbar_wait(&raw_full[rs], ruse & 1u, abort_flag, WAIT_NS)) break;
                    uint64_t x[4] = {0, 0, 0, 0};
                    if (!skip) {
                        const uint4* r = reinterpret_cast<const uint4*>(raw + rs * RAW_SLOT + raw_off);
                        const uint4 v0 = r[0], v1 = r[T];
                        x[0] = (uint64_t)v0.x | ((uint64_t)v0.y << 32);
                        x[1] = (uint64_t)v0.z | ((uint64_t)v0.w << 32);
                        x[2] = (uint64_t)v1.x | ((uint64_t)v1.y << 32);
                        x[3] = (uint64_t)v1.z | ((uint64_t)v1.w << 32);
                    }
                    if (!mbar_wait(&empty_bar[os], (ouse & 1u) ^ 1u, abort_flag, WAIT_NS)) break;
                    if (!skip) {
                        store_row<FMT>(slots + os * SLOT_BYTES + dst, hrow, x);
                        fence_proxy_async();
                    }
                    mbar_arrive(&full_bar[os]);
                    mbar_arrive(&raw_empty[rs]);
                }
            } else {
                uint64_t cur[BW], nxt[BW];
                // Words past the row's last stage are not read (they may lie past the buffer).
                const int64_t lim = n_stages * WORDS;
                auto load_batch = [&](int64_t s0, uint64_t* x) {
    #pragma unroll
                    for (int q = 0; q < BW; q += 2) {
                        const int64_t w = s0 * WORDS + q;
                        ulonglong2 v = make_ulonglong2(0, 0);
                        const int64_t at = off + (blocked ? (w >> 2) * (4 * T) + ((w >> 1) & 1) * (2 * T) + (w & 1) : w);
                        if (off >= 0 && w + 1 < lim) v = __ldg(reinterpret_cast<const ulonglong2*>(src + at));
                        else if (off >= 0 && w < lim) v.x = __ldg(src + at);
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
                        const int slot = (int)(G % STAGES);
                        const uint32_t use = (uint32_t)(G / STAGES);
                        if (!mbar_wait(&empty_bar[slot], (use & 1u) ^ 1u, abort_flag, WAIT_NS)) break;
                        if (off >= 0) {
                            store_row<FMT>(slots + slot * SLOT_BYTES + dst, hrow, cur + j * WORDS);
                            fence_proxy_async();
                        }
                        mbar_arrive(&full_bar[slot]);
                    }
    #pragma unroll
                    for (int q = 0; q < BW; q++) cur[q] = nxt[q];
                }
            }
            // ---- epilogue: warp w reads lanes 32 (w % 4) .. of accumulator w / 8, columns 128 ((w / 4) % 2) .. ----
            // Every lane observes the accumulator barrier itself (its own acquire before its tcgen05 fence), and
            // the warp takes one decision, as the tcgen05.ld below needs the whole warp.
            const bool got_acc = n_stages == 0 || mbar_wait(&acc_bar, tile_iter & 1u, abort_flag, WAIT_NS);
            const bool ok = __all_sync(0xffffffffu, got_acc);
            if (ok) {
                tc_fence_after();
                const int lane_base = (warp & 3) * 32;
                const int accn = warp >> 3;
                const int64_t i = a0 + accn * TH + lane_base + lane;
                const bool row_ok = lane_base + lane < TH && i < m;
                for (int q = 0; q < 4; q++) {
                    const int col0 = ((warp >> 2) & 1) * 128 + q * 32;
                    if (col0 >= T) break;  // warp-uniform
                    uint32_t v[32];
                    if (n_stages > 0) {
                        const uint32_t taddr = tmem + ((uint32_t)lane_base << 16) + (uint32_t)(accn * T + col0);
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
                    if (!row_ok) continue;
                    const int64_t j0 = b0 + col0;
                    const int64_t t0 = cb + tri_index(i, j0, m);  // slot of (i, j0 + c) is t0 + c when j0 + c > i
                    uint32_t bits = 0;
#pragma unroll
                    for (int c = 0; c < 32; c++) {
                        const int64_t j = j0 + c;
                        if (i < j && j < m && col0 + c < T) {
                            const int64_t t = t0 + c;
                            if (cls == nullptr || cls[t] == ETM_CAND_COUNT) {
                                const int32_t cnt =
                                    n_stages > 0 ? __float2int_rn(__uint_as_float(v[c]) * Fmt<FMT>::SCALE) : 0;
                                if (surv == nullptr) {
                                    out[t] = cnt;
                                } else if (cnt >= min_count) {
                                    out[t] = cnt;
                                    bits |= 1u << c;
                                }
                            }
                        }
                    }
                    if (bits != 0u) {
                        // Survivor bits of slots t0 + c, c in the mask: at most two words of the bitmask.
                        const int c1 = __ffs(bits) - 1;
                        const int64_t t1 = t0 + c1;
                        const uint32_t sh = (uint32_t)(t1 & 31);
                        const uint32_t mb = bits >> c1;
                        atomicOr(surv + (t1 >> 5), mb << sh);
                        if (sh != 0u && (mb >> (32u - sh)) != 0u) atomicOr(surv + (t1 >> 5) + 1, mb >> (32u - sh));
                    }
                }
            }
            tc_fence_before();
        } else if (warp == MMA_WARP && lane == 0) {
            // ---- MMA issuer: two M = 128 MMAs per K step, sharing the B tile ----
            tc_fence_after();
            for (int64_t s = 0; s < n_stages; s++) {
                const int64_t G = gstage + s;
                const int slot = (int)(G % NST);
                const uint32_t use = (uint32_t)(G / NST);
                if (!mbar_wait(&full_bar[slot], use & 1u, abort_flag, first_wait_ns)) break;
                tc_fence_after();
                const uint32_t base = smem_u32(slots + slot * SLOT_BYTES);
                const uint32_t b_addr = base + 2 * HALF_BYTES;
                // A half h: rows h TH .. of block ua; on a diagonal block pair, rows of the B tile.
                const uint32_t a_lo = diag ? b_addr : base;
                const uint32_t a_hi = diag ? b_addr + TH * 128 : base + HALF_BYTES;
#pragma unroll
                for (int k = 0; k < 4; k++) {
                    const uint32_t acc = (s > 0 || k > 0) ? 1u : 0u;
                    const uint64_t bd = smem_desc(b_addr + 32 * k);
                    mma_ss<FMT>(tmem, smem_desc(a_lo + 32 * k), bd, acc, tmem + SF_COL);
                    mma_ss<FMT>(tmem + T, smem_desc(a_hi + 32 * k), bd, acc, tmem + SF_COL);
                }
                mma_commit(&empty_bar[slot]);
            }
            // A block pair without stages (an empty prefix) issues no MMA and commits nothing: its producers do
            // not wait for the accumulator, and acc_bar's phases stay one per block pair with stages, so a
            // later pair's epilogue can never take an earlier phase for its own.
            if (n_stages > 0) mma_commit(&acc_bar);
        } else if (STAGED && warp == LOAD_WARP && lane == 0) {
            // ---- loader: the raw chunk of block ua (unless diagonal) and of block ub for every stage ----
            const int64_t cw = cld[wi];
            const uint64_t* src_a = src + cbase[wi] + ua * T * cw;
            const uint64_t* src_b = src + cbase[wi] + ub * T * cw;
            for (int64_t s = 0; s < n_stages; s++) {
                const int64_t G = gstage + s;
                const int rs = (int)(G % RAW_STAGES);
                const uint32_t ruse = (uint32_t)(G / RAW_STAGES);
                if (!mbar_wait(&raw_empty[rs], (ruse & 1u) ^ 1u, abort_flag, WAIT_NS)) break;
                mbar_expect_tx(&raw_full[rs], diag ? RAW_BLOCK : 2 * RAW_BLOCK);
                if (!diag) bulk_copy(raw + rs * RAW_SLOT, src_a + s * 4 * T, RAW_BLOCK, &raw_full[rs]);
                bulk_copy(raw + rs * RAW_SLOT + RAW_BLOCK, src_b + s * 4 * T, RAW_BLOCK, &raw_full[rs]);
                raw_issued = G + 1;
            }
        }
        gstage += n_stages;
        if (n_stages > 0) tile_iter += 1;  // one acc_bar phase per block pair with stages
        __syncthreads();
        if (*abort_flag) break;
    }

    if (STAGED && warp == LOAD_WARP && lane == 0 && *abort_flag) {
        // Every bulk copy this CTA issued lands before the CTA exits: wait (bounded) for the last phase issued
        // on each raw slot (earlier phases of a slot complete first).
        for (int64_t G = max64(0, raw_issued - RAW_STAGES); G < raw_issued; G++) {
            const uint64_t t0 = now_ns();
            while (!mbar_test(&raw_full[G % RAW_STAGES], (uint32_t)(G / RAW_STAGES) & 1u) && now_ns() - t0 < WAIT_NS)
                __nanosleep(256);
        }
    }
    if (warp == MMA_WARP) {
        if (lane == 0 && *abort_flag) {
            // Wait (bounded) for every MMA this CTA issued before its tensor memory is freed.
            mma_commit(&drain_bar);
            const uint64_t t0 = now_ns();
            while (!mbar_test(&drain_bar, 0) && now_ns() - t0 < WAIT_NS) __nanosleep(256);
        }
        __syncwarp();
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS) : "memory");
    }
    if (tid == 0 && *abort_flag) atomicExch(&g_tc_status, ETM_ETIMEOUT);
}

// Issue rate of the Gram's own MMA shape: one CTA per SM, one thread issuing `iters` back-to-back MMAs
// (M = 128, N = T, the format's K per instruction) on a zeroed shared-memory tile into one accumulator,
// then a bounded wait for their completion. The roofline's tensor peak for that operand format.
template <int FMT>
__global__ void __launch_bounds__(128, 1) mma_rate_kernel(int64_t iters, int* status) {
    extern __shared__ uint8_t dsmem[];
    __shared__ __align__(8) uint64_t done_bar;
    __shared__ uint32_t tmem_sh;
    uint8_t* tiles = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(dsmem) + 1023) & ~uintptr_t(1023));
    const int tid = threadIdx.x, warp = tid >> 5;
    for (int i = tid; i < 3 * HALF_BYTES / 16; i += blockDim.x) reinterpret_cast<uint4*>(tiles)[i] = make_uint4(0, 0, 0, 0);
    if (tid == 0) {
        mbar_init(&done_bar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    fence_proxy_async();
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_sh)),
                     "r"(TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
        tc_fence_before();
    }
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_sh;
    if constexpr (FMT == 4) {
        const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16) + SF_COL;
        const uint32_t u = 0x7F7F7F7Fu;
        asm volatile(
            "tcgen05.st.sync.aligned.32x32b.x32.b32 [%0], {%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,"
            "%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1};" ::"r"(taddr),
            "r"(u)
            : "memory");
        asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
        tc_fence_before();
        __syncthreads();
        tc_fence_after();
    }
    if (tid == 0) {
        const uint32_t a = smem_u32(tiles), b = a + HALF_BYTES;
        for (int64_t it = 0; it < iters; it++) {
            const int k = (int)(it & 3);
            mma_ss<FMT>(tmem, smem_desc(a + 32 * k), smem_desc(b + 32 * k), it > 0 ? 1u : 0u, tmem + SF_COL);
        }
        mma_commit(&done_bar);
        const uint64_t t0 = now_ns();
        bool ok = true;
        while (!mbar_test(&done_bar, 0)) {
            if (now_ns() - t0 > WAIT_NS) {
                ok = false;
                break;
            }
            __nanosleep(128);
        }
        if (!ok) atomicExch(status, ETM_ETIMEOUT);
    }
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS) : "memory");
    }
}

std::mutex g_cfg_lock;
// The MMA thread's wait for a filled stage: WAIT_NS unless a test set it (0 = give up at once).
uint64_t g_first_wait_ns = WAIT_NS;

// ETM_GRAM_STAGED=0 in the environment keeps packed e2m1 over blocked rows on the producer-load form
// (both are exact; the staged form is the faster one on GB300).
bool staged_enabled() {
    static const bool on = [] {
        const char* v = getenv("ETM_GRAM_STAGED");
        return v == nullptr || v[0] != '0';
    }();
    return on;
}

template <int FMT, bool STAGED>
int launch_gram_kernel(const uint64_t* cbuf, const int64_t* cbase, const int64_t* cwords, const int64_t* cld,
                       const int32_t* grp_size, const int64_t* cand_off, const int64_t* work_groups,
                       const int64_t* work_off, int64_t n_work, int64_t n_tiles, int64_t chunk_base,
                       const uint8_t* cls, int32_t min_count, int32_t* out, uint32_t* surv, int64_t* work_counter,
                       bool blocked, cudaStream_t s) {
    constexpr int smem = STAGED ? ST_SMEM : SMEM_BYTES;
    constexpr int threads = STAGED ? ST_THREADS : THREADS;
    static bool configured = false;
    uint64_t first_wait;
    {
        std::lock_guard<std::mutex> guard(g_cfg_lock);
        if (!configured) {
            ETM_CUDA(cudaFuncSetAttribute(gram_kernel<FMT, STAGED>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
            configured = true;
        }
        first_wait = g_first_wait_ns;
    }
    const int64_t sms = max(1, sm_count());
    const int grid = (int)max64(1, min64(sms, n_tiles > 0 ? n_tiles : sms));
    if (work_counter != nullptr) ETM_CUDA(cudaMemsetAsync(work_counter, 0, sizeof(int64_t), s));
    gram_kernel<FMT, STAGED><<<grid, threads, smem, s>>>(cbuf, cbase, cwords, cld, grp_size, cand_off, work_groups,
                                                         work_off, n_work, chunk_base, cls, min_count, out, surv,
                                                         reinterpret_cast<unsigned long long*>(work_counter),
                                                         first_wait, blocked);
    ETM_LAUNCHED("gram_tc");
    return ETM_OK;
}

template <int FMT>
int launch_gram(const uint64_t* cbuf, const int64_t* cbase, const int64_t* cwords, const int64_t* cld,
                const int32_t* grp_size, const int64_t* cand_off, const int64_t* work_groups, const int64_t* work_off,
                int64_t n_work, int64_t n_tiles, int64_t chunk_base, const uint8_t* cls, int32_t min_count,
                int32_t* out, uint32_t* surv, int64_t* work_counter, bool blocked, cudaStream_t s) {
    if constexpr (FMT == 4) {
        if (blocked && staged_enabled())
            return launch_gram_kernel<4, true>(cbuf, cbase, cwords, cld, grp_size, cand_off, work_groups, work_off,
                                               n_work, n_tiles, chunk_base, cls, min_count, out, surv, work_counter,
                                               blocked, s);
    }
    return launch_gram_kernel<FMT, false>(cbuf, cbase, cwords, cld, grp_size, cand_off, work_groups, work_off, n_work,
                                          n_tiles, chunk_base, cls, min_count, out, surv, work_counter, blocked, s);
}

}  // namespace

namespace etm {

int gram_block_members(int32_t elem) {
    const int e = elem & ~(ETM_TC_WIDE | ETM_TC_BLOCKED);
    return e == ETM_TC_MXF4 ? Fmt<4>::T : e == 1 || e == 2 ? Fmt<1>::T : 0;
}

int gram_tc(const uint64_t* cbuf, const int64_t* cbase, const int64_t* cwords, const int64_t* cld,
            const int32_t* grp_size, const int64_t* cand_off, const int64_t* work_groups, const int64_t* work_off,
            int64_t n_work, int64_t n_tiles, int64_t chunk_base, const uint8_t* cls, int32_t elem, int32_t min_count,
            int32_t* out, uint32_t* surv, int64_t* work_counter, cudaStream_t s) {
    // elem: 1 = e4m3, 2 = f16, ETM_TC_MXF4 = packed e2m1; ETM_TC_WIDE is accepted and changes nothing;
    // + ETM_TC_BLOCKED: the member rows are in the projection's blocked layout with blocks of T members.
    const bool blocked = (elem & ETM_TC_BLOCKED) != 0;
    const int e = elem & ~(ETM_TC_WIDE | ETM_TC_BLOCKED);
    ETM_REQUIRE(e == 1 || e == 2 || e == ETM_TC_MXF4, ETM_EINVAL,
                "gram_tc: element code %d (1 = e4m3, 2 = f16, %d = e2m1 block-scaled)", elem, ETM_TC_MXF4);
#define ETM_GRAM_ARGS cbuf, cbase, cwords, cld, grp_size, cand_off, work_groups, work_off, n_work, n_tiles, chunk_base, cls, min_count, out, surv, work_counter, blocked, s
    if (e == ETM_TC_MXF4) return launch_gram<4>(ETM_GRAM_ARGS);
    return e == 2 ? launch_gram<2>(ETM_GRAM_ARGS) : launch_gram<1>(ETM_GRAM_ARGS);
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
                        chunk_base, cls, elem, 0, out_counts, nullptr, work_counter, as_stream(stream));
}

extern "C" int etm_count_tiles_tc_sel(const uint64_t* cbuf, const int64_t* cbase, const int64_t* cwords,
                                      const int64_t* cld, const int32_t* grp_size, const int64_t* cand_off,
                                      const int64_t* work_groups, const int64_t* work_off, int64_t n_work,
                                      int64_t n_tiles, int64_t chunk_base, const uint8_t* cls, int32_t elem,
                                      int32_t min_count, int32_t* out_counts, uint32_t* surv_bits,
                                      int64_t* work_counter, void* stream) {
    ETM_REQUIRE((reinterpret_cast<uintptr_t>(cbuf) & 15) == 0, ETM_EINVAL,
                "etm_count_tiles_tc_sel: cbuf must be 16-byte aligned");
    ETM_REQUIRE(surv_bits != nullptr, ETM_EINVAL, "etm_count_tiles_tc_sel: surv_bits is required");
    if (n_work <= 0) return ETM_OK;
    return etm::gram_tc(cbuf, cbase, cwords, cld, grp_size, cand_off, work_groups, work_off, n_work, n_tiles,
                        chunk_base, cls, elem, min_count, out_counts, surv_bits, work_counter, as_stream(stream));
}

extern "C" int etm_gram_block_members(int32_t elem) { return etm::gram_block_members(elem); }

namespace {
template <int FMT>
int mma_rate(int64_t iters, int* status, cudaStream_t s) {
    constexpr int smem = 3 * HALF_BYTES + 1024;
    ETM_CUDA(cudaFuncSetAttribute(mma_rate_kernel<FMT>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    mma_rate_kernel<FMT><<<max(1, sm_count()), 128, smem, s>>>(iters, status);
    ETM_LAUNCHED("mma_rate");
    return ETM_OK;
}
}  // namespace

extern "C" int etm_tc_mma_rate(int32_t elem, int64_t iters, double* out_tflops, void* stream) {
    // Times `iters` MMAs per SM of the Gram's shape for `elem` on every SM (CUDA events on `stream`, which is
    // synchronized) and returns the dense rate in TFLOP/s: 2 M N K per MMA.
    const int e = elem & ~ETM_TC_WIDE;
    ETM_REQUIRE(e == 1 || e == 2 || e == ETM_TC_MXF4, ETM_EINVAL, "etm_tc_mma_rate: element code %d", elem);
    ETM_REQUIRE(iters > 0 && iters < (1LL << 32) && out_tflops != nullptr, ETM_EINVAL, "etm_tc_mma_rate: bad iters");
    cudaStream_t s = as_stream(stream);
    int* status = nullptr;
    ETM_CUDA(cudaGetSymbolAddress(reinterpret_cast<void**>(&status), g_tc_status));
    cudaEvent_t e0, e1;
    ETM_CUDA(cudaEventCreate(&e0));
    ETM_CUDA(cudaEventCreate(&e1));
    int st = ETM_OK;
    auto run = [&]() { return e == ETM_TC_MXF4 ? mma_rate<4>(iters, status, s) : e == 2 ? mma_rate<2>(iters, status, s)
                                                                                         : mma_rate<1>(iters, status, s); };
    st = run();  // warm-up
    if (st == ETM_OK) {
        cudaEventRecord(e0, s);
        st = run();
        cudaEventRecord(e1, s);
    }
    float ms = 0.f;
    if (st == ETM_OK) {
        const cudaError_t err = cudaEventSynchronize(e1);
        if (err != cudaSuccess) {
            etm::set_error("etm_tc_mma_rate: %s", cudaGetErrorString(err));
            st = ETM_ECUDA;
        } else {
            cudaEventElapsedTime(&ms, e0, e1);
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (st != ETM_OK) return st;
    const double k = e == ETM_TC_MXF4 ? 64.0 : e == 1 ? 32.0 : 16.0;
    const double n = e == ETM_TC_MXF4 ? Fmt<4>::T : Fmt<1>::T;
    const double flops = 2.0 * 128.0 * n * k * (double)iters * (double)max(1, sm_count());
    *out_tflops = ms > 0.f ? flops / (ms * 1e-3) / 1e12 : 0.0;
    return ETM_OK;
}

extern "C" int etm_set_wait_limits(int64_t gram_first_wait_ns, int64_t proj_first_wait_ns) {
    {
        std::lock_guard<std::mutex> guard(g_cfg_lock);
        g_first_wait_ns = gram_first_wait_ns < 0 ? WAIT_NS : (uint64_t)gram_first_wait_ns;
    }
    etm::proj_set_first_wait(proj_first_wait_ns);
    return ETM_OK;
}

extern "C" int etm_device_status(void* stream) {
    // Both status words are read and cleared on every call, so a stale word never outlives the call
    // that reports it.
    int v = 0;
    ETM_CUDA(cudaMemcpyFromSymbolAsync(&v, g_tc_status, sizeof(int), 0, cudaMemcpyDeviceToHost, as_stream(stream)));
    ETM_CUDA(cudaStreamSynchronize(as_stream(stream)));
    if (v != 0) {
        const int zero = 0;
        ETM_CUDA(cudaMemcpyToSymbolAsync(g_tc_status, &zero, sizeof(int), 0, cudaMemcpyHostToDevice, as_stream(stream)));
        ETM_CUDA(cudaStreamSynchronize(as_stream(stream)));
    }
    int p = 0;
    const int st = etm::proj_status_take(as_stream(stream), &p);
    if (st != ETM_OK) return st;
    if (v != 0 && p != 0)
        etm::set_error("a tensor-core counting kernel (status %d) and the projection (status %d) gave up bounded waits",
                       v, p);
    else if (v != 0)
        etm::set_error("a tensor-core counting kernel gave up a bounded wait (status %d)", v);
    else if (p == ETM_EINVAL)
        etm::set_error("the row-major projection met a member column past its row-major copy (status %d)", p);
    else if (p != 0)
        etm::set_error("the projection gave up a bounded wait for its bulk copies (status %d)", p);
    return v != 0 ? v : p;
}
