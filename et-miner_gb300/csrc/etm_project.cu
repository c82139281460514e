// Prefix projection: count a prefix group over only the transactions its
// prefix holds. The reference's CPU route does this for wide groups
// (_count_group_proj, core/cpu_miner.py:720-791: a Gram over the prefix's
// tidset); here it is device passes per chunk of groups:
//
//   1. prefix counts:    popcount of the AND of the group's prefix columns
//                        (plans the chunks; coalesced reads)
//   2. prefix segments:  the same popcount per segment of ETM_PROJ_SEG_WORDS
//                        words, giving each segment's piece of the projected
//                        row its word offset
//   3. projection:       per (segment, group): the segment's prefix rows listed
//                        in shared memory; per member its segment words staged
//                        in shared memory by a TMA bulk copy and gathered at
//                        the listed rows, 64 per word by two warp ballots
//   (prefix rows:        the ascending transaction ids of the prefix AND, kept
//                        as an entry point for callers that want the tidset)
//
// after which the tile-pair kernel counts the group on words that hold only
// the prefix's rows: a group whose prefix holds a fraction d of the rows
// costs d of the AND+popcount work it would cost on the full bitvectors.
#include <atomic>

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

// Occupancy word ow of the prefix: bit b set when every prefix column holds a row in tile 64 ow + b (all ones
// without an occupancy). Words of a tile whose bit is clear have a zero prefix AND and are not read.
constexpr int64_t OCC_SPAN = 64 * ETM_OCC_TILE_WORDS;  // words per occupancy word
__device__ inline uint64_t prefix_live(const uint64_t* __restrict__ occ, int64_t occ_ld,
                                       const int32_t* __restrict__ pref, int plen, int64_t ow) {
    uint64_t m = ~0ULL;
    if (occ != nullptr)
        for (int q = 0; q < plen; q++) m &= __ldg(occ + (int64_t)pref[q] * occ_ld + ow);
    return m;
}
__device__ inline bool tile_live(uint64_t live, int64_t w) {
    return ((live >> ((w / ETM_OCC_TILE_WORDS) & 63)) & 1ULL) != 0ULL;
}

__global__ void __launch_bounds__(PT) prefix_counts_kernel(const uint64_t* __restrict__ fbv, int64_t ld,
                                                           int64_t n_words, const int32_t* __restrict__ rows,
                                                           int width, const int64_t* __restrict__ grp_first,
                                                           const int64_t* __restrict__ work_groups,
                                                           int64_t* __restrict__ out,
                                                           const uint64_t* __restrict__ occ, int64_t occ_ld) {
    __shared__ int32_t pref[64];
    __shared__ unsigned part[PT / 32];
    const int64_t wi = blockIdx.x;
    const int64_t first = grp_first[work_groups[wi]];
    const int plen = width - 1;
    if (threadIdx.x < plen) pref[threadIdx.x] = rows[first * width + threadIdx.x];
    __syncthreads();
    unsigned s = 0;
    for (int64_t w0 = 0; w0 < n_words; w0 += OCC_SPAN) {
        const uint64_t live = prefix_live(occ, occ_ld, pref, plen, w0 / OCC_SPAN);
        if (live == 0ULL) continue;  // block-uniform
        const int64_t w1 = min64(n_words, w0 + OCC_SPAN);
        for (int64_t w = w0 + threadIdx.x; w < w1; w += PT)
            if (tile_live(live, w)) s += __popcll(prefix_word(fbv, ld, pref, plen, w));
    }
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

// Segmented projection. The rows are cut into segments of SEG_W bitvector words (64 SEG_W rows); the
// projected row of a member is the concatenation over the segments of its bits at the prefix rows of
// that segment, each segment's piece zero-padded to whole 64-bit words (zero rows add nothing to a
// count). Units are (segment, work entry) in segment-major order, so the CTAs running at one time read
// the same row range of the columns and the column words stay in L2 between groups.
constexpr int SEG_W = ETM_PROJ_SEG_WORDS;
static_assert(OCC_SPAN % SEG_W == 0, "a projection segment lies within one occupancy word");
constexpr int LIST_CAP = 8192;         // prefix rows listed per pass (a segment holds at most 64 SEG_W)
constexpr int MPI = 4;                 // members gathered per block barrier (independent chains)
constexpr int NSTAGE = 2 * MPI;        // member segments in shared memory: the current MPI and the next MPI
constexpr int STAGE_BYTES = SEG_W * 8 + 16;  // a member's segment words, then 16 zero bytes
constexpr int ID_RING = 512;           // member column ids held in shared memory
constexpr int MAX_CHUNKS = (LIST_CAP / 64 / 4 + (PT / 32) - 1) / (PT / 32);
constexpr int P_WARPS = PT / 32;
constexpr int PROJ_SMEM = STAGE_BYTES * NSTAGE + SEG_W * 8 + LIST_CAP * 2;
static_assert(MPI == 4 && MAX_CHUNKS % 2 == 0, "the blocked store maps a warp onto 4 members x 2 chunks");

__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }
// Bulk (TMA) copies of whole member segments into shared memory, completed on an mbarrier.
// Every wait for them is bounded in time (%globaltimer).
constexpr uint64_t BULK_WAIT_NS = 2000000000ull;
// Limit of the first wait for a group's copies (a test sets 0 to drive the give-up path).
std::atomic<uint64_t> g_proj_first_wait_ns{BULK_WAIT_NS};
__device__ int g_proj_status;
__device__ __forceinline__ uint64_t now_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
__device__ __forceinline__ void bar_init(uint64_t* bar) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(bar)) : "memory");
}
__device__ __forceinline__ void bar_expect(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void bulk_copy(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                 ::"r"(smem_addr(dst)), "l"(src), "r"(bytes), "r"(smem_addr(bar))
                 : "memory");
}
__device__ __forceinline__ bool bar_try(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// Waits for the phase of `parity`; false when `limit_ns` ran out first (a limit of 0 gives up at once:
// the give-up path's test hook).
__device__ __forceinline__ bool bar_wait(uint64_t* bar, uint32_t parity, uint64_t limit_ns) {
    if (limit_ns == 0) return false;
    if (bar_try(bar, parity)) return true;
    const uint64_t t0 = now_ns();
    while (!bar_try(bar, parity))
        if (now_ns() - t0 > limit_ns) return false;
    return true;
}

// One block per work entry: the words of every segment's piece, their exclusive prefix (seg_off, n_seg + 1
// entries per work entry) and the total (out_words).
__global__ void __launch_bounds__(PT) prefix_segments_kernel(const uint64_t* __restrict__ fbv, int64_t ld,
                                                             int64_t n_words, const int32_t* __restrict__ rows,
                                                             int width, const int64_t* __restrict__ grp_first,
                                                             const int64_t* __restrict__ work_groups, int64_t n_seg,
                                                             int64_t* __restrict__ seg_off,
                                                             int64_t* __restrict__ out_words,
                                                             const uint64_t* __restrict__ occ, int64_t occ_ld) {
    __shared__ int32_t pref[64];
    __shared__ unsigned part[P_WARPS];
    const int64_t wi = blockIdx.x;
    const int64_t first = grp_first[work_groups[wi]];
    const int plen = width - 1;
    if (threadIdx.x < plen) pref[threadIdx.x] = rows[first * width + threadIdx.x];
    __syncthreads();
    int64_t* so = seg_off + wi * (n_seg + 1);
    int64_t run = 0;  // meaningful in thread 0
    for (int64_t s = 0; s < n_seg; s++) {
        const int64_t w1 = min64(n_words, (s + 1) * SEG_W);
        unsigned c = 0;
        // A segment lies within one occupancy word (SEG_W divides OCC_SPAN).
        const uint64_t live = prefix_live(occ, occ_ld, pref, plen, (s * SEG_W) / OCC_SPAN);
        if (live != 0ULL)
            for (int64_t w = s * SEG_W + threadIdx.x; w < w1; w += PT)
                if (tile_live(live, w)) c += __popcll(prefix_word(fbv, ld, pref, plen, w));
        c = __reduce_add_sync(0xffffffffu, c);
        if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = c;
        __syncthreads();
        if (threadIdx.x == 0) {
            unsigned t = 0;
            for (int i = 0; i < P_WARPS; i++) t += part[i];
            so[s] = run;
            run += ((t + 63) / 64 + 3) & ~3u;  // whole 4-word chunks
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        so[n_seg] = run;
        out_words[wi] = run;
    }
}

// Projected member rows: row-major (blk = 0: word w of member j at j stride + w), or blocked (blk > 0: the
// members in blocks of blk, each block stored 4-word chunk by chunk, and each chunk as two halves: words
// 0-1 of every member of the block, then words 2-3; word w of member j at (j / blk) stride blk +
// (w / 4) 4 blk + ((w / 2) % 2) 2 blk + (j % blk) 2 + w % 2). A Gram stage's words of a block are then one
// contiguous run, and consecutive members' 16-byte halves are adjacent, so a warp reading one half of 32
// members' chunks reads 512 contiguous bytes. Offsets are in words from the work entry's base; the two
// parts add: proj_member_offset(j) + proj_word_offset(w).
__host__ __device__ inline int64_t proj_member_offset(int64_t j, int64_t stride, int64_t blk) {
    return blk > 0 ? (j / blk) * stride * blk + (j % blk) * 2 : j * stride;
}
__host__ __device__ inline int64_t proj_word_offset(int64_t w, int64_t blk) {
    return blk > 0 ? (w >> 2) * 4 * blk + ((w >> 1) & 1) * 2 * blk + (w & 1) : w;
}

struct PassArgs {
    const uint64_t* fbv;
    int64_t ld;
    const int32_t* rows;
    int width;
    int64_t first, m, w0;
    int nw;
    uint64_t* stage;
    const uint32_t* l32;
    int pass_rows, pass_words;
    uint64_t* dst;        // the work entry's projected rows (cbuf + cbase)
    int64_t stride, out0; // words per member row; word of the row where this pass's words start
    int64_t blk;          // members per layout block (0: row-major member rows)
    uint64_t* park;  // MPI x 4 MAX_CHUNKS words per warp of shared memory
    uint64_t* bars;  // two mbarriers (shared memory): group slots 0 and 1 of the stage buffers
    int32_t* ids;    // ID_RING member column ids (shared memory)
    uint64_t first_wait_ns;  // limit of each wait for a group's copies
};

// Every member of the group through the stage buffers, for one pass of listed rows. The pass's output
// words go to the warps in chunks of 4 (chunk c to warp c % P_WARPS, at most MAX_CHUNKS per warp).
// Per lane and word, the stage-buffer byte offset of the 32-bit word holding each of its two rows and
// the row's bit are computed once per pass; rows past the pass point at the zero pad after the
// buffer. Per member a word then costs two shared loads, two bit tests and two ballots; members go MPI
// at a time (independent chains, one block barrier per MPI members); lane 0 parks the words in shared
// memory and the warp stores them with coalesced stores.
__device__ __forceinline__ bool gather_members(const PassArgs& a, uint32_t& phase) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int m = (int)a.m;
    const int n_chunks = (a.pass_words + 3) >> 2;
    uint32_t ra[MAX_CHUNKS * 4], rb[MAX_CHUNKS * 4], ma[MAX_CHUNKS * 4], mb[MAX_CHUNKS * 4];
    uint32_t valid = 0;  // bit 4 k + q: word q of the warp's k-th chunk is a word of the pass
#pragma unroll
    for (int k = 0; k < MAX_CHUNKS; k++) {
#pragma unroll
        for (int q = 0; q < 4; q++) {
            const int i = 4 * k + q;
            const int t = 4 * (warp + P_WARPS * k) + q;
            const int r0 = 64 * t + lane, r1 = r0 + 32;
            const uint32_t e = t < a.pass_words ? a.l32[32 * t + lane] : 0u;
            const uint32_t l0 = e & 0xFFFFu, l1 = e >> 16;
            ra[i] = r0 < a.pass_rows ? (l0 >> 5) << 2 : SEG_W * 8;  // else the zero pad
            rb[i] = r1 < a.pass_rows ? (l1 >> 5) << 2 : SEG_W * 8;
            ma[i] = 1u << (l0 & 31u);
            mb[i] = 1u << (l1 & 31u);
            // Every word of a chunk holding a word of the pass (the words past the pass are zero: pieces are
            // padded to whole 4-word chunks).
            valid |= ((warp + P_WARPS * k) < ((a.pass_words + 3) >> 2) ? 1u : 0u) << i;
        }
    }
    // Copies: members t MPI .. t MPI + MPI - 1 (group t) go to group slot t % 2 (stage buffers
    // (t % 2) MPI ..), each member segment one bulk (TMA) copy issued by thread 0 and completed on the
    // slot's mbarrier; group t + 1 is issued once every warp is past group t - 1. Member column ids come
    // from a ring of ID_RING entries in shared memory, refilled half a ring ahead.
    const int32_t* colp = a.rows + a.first * a.width + a.width - 1;
    const uint32_t seg_bytes = (uint32_t)((a.nw + 1) & ~1) * 8;  // whole 16-byte pieces (ld is even)
    const int n_groups = (m + MPI - 1) / MPI;
    auto issue = [&](int t) {
        if (threadIdx.x != 0 || t >= n_groups) return;
        const int slot = t & 1;
        const int nv = min(MPI, m - t * MPI);
        bar_expect(&a.bars[slot], (uint32_t)nv * seg_bytes);
        for (int v = 0; v < nv; v++) {
            const int j = t * MPI + v;
            const uint64_t* src = a.fbv + (int64_t)a.ids[j & (ID_RING - 1)] * a.ld + a.w0;
            bulk_copy(reinterpret_cast<uint8_t*>(a.stage) + (slot * MPI + v) * STAGE_BYTES, src, seg_bytes,
                      &a.bars[slot]);
        }
    };
    auto fill_ids = [&](int j1) {  // members [j1, j1 + ID_RING / 2)
        for (int t = threadIdx.x; t < ID_RING / 2; t += PT) {
            const int j = j1 + t;
            a.ids[j & (ID_RING - 1)] = j < m ? colp[(int64_t)j * a.width] : 0;
        }
    };
    fill_ids(0);
    fill_ids(ID_RING / 2);
    __syncthreads();
    issue(0);
    const uint8_t* sbytes = reinterpret_cast<const uint8_t*>(a.stage);
    uint64_t* park = a.park + warp * MPI * 4 * MAX_CHUNKS;
    const bool my_store = lane < 4 * MAX_CHUNKS && ((valid >> lane) & 1u);
    // Lane l stores word (l & 3) of the pass's 4-word chunk warp + P_WARPS (l >> 2), for members j .. j + MPI - 1.
    const int64_t wpos = a.out0 + 4 * (warp + P_WARPS * (lane >> 2));
    uint64_t* out_w = a.dst + wpos + (lane & 3);  // row-major stores (blk = 0)
    for (int j0 = 0; j0 < m; j0 += NSTAGE) {
        // Unrolled over the stage buffers: members j0 + u .. j0 + u + MPI - 1 sit in buffers u ...
#pragma unroll
        for (int u = 0; u < NSTAGE; u += MPI) {
            const int j = j0 + u;
            if (j >= m) break;
            const int slot = u / MPI;  // group j / MPI
            const bool got = bar_wait(&a.bars[slot], (phase >> slot) & 1u, a.first_wait_ns);
            phase ^= 1u << slot;
            // Members j .. j + MPI - 1 have landed and every warp is past the previous group (or a wait ran out).
            if (__syncthreads_or(!got)) {
                // Only this slot's copies can be in flight (the other slot's were consumed before these were
                // issued): every thread waits for them, bounded, before the block stops. If even that wait
                // runs out, the status says so: copies may still land in this SM's shared memory, and the
                // caller must stop using the device.
                const bool drained = got || bar_wait(&a.bars[slot], (phase >> slot) & 1u ^ 1u, BULK_WAIT_NS);
                if (threadIdx.x == 0) atomicExch(&g_proj_status, drained ? ETM_ETIMEOUT : ETM_EUNSAFE);
                __syncthreads();
                return false;
            }
            issue(j / MPI + 1);  // into the other slot
            if ((j & (ID_RING / 2 - 1)) == 0 && j > 0) fill_ids(j + ID_RING / 2);
            const uint8_t* sa = sbytes + u * STAGE_BYTES;
#pragma unroll
            for (int k = 0; k < MAX_CHUNKS; k++) {
                if (warp + P_WARPS * k >= n_chunks) break;
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    const int i = 4 * k + q;
                    uint32_t x0[MPI], x1[MPI];
#pragma unroll
                    for (int v = 0; v < MPI; v++) {
                        x0[v] = *reinterpret_cast<const uint32_t*>(sa + v * STAGE_BYTES + ra[i]);
                        x1[v] = *reinterpret_cast<const uint32_t*>(sa + v * STAGE_BYTES + rb[i]);
                    }
#pragma unroll
                    for (int v = 0; v < MPI; v++) {
                        const unsigned lo = __ballot_sync(0xffffffffu, (x0[v] & ma[i]) != 0u);
                        const unsigned hi = __ballot_sync(0xffffffffu, (x1[v] & mb[i]) != 0u);
                        if (lane == 0) park[v * 4 * MAX_CHUNKS + i] = (uint64_t)lo | ((uint64_t)hi << 32);
                    }
                }
            }
            __syncwarp();
            if (a.blk == 0) {
                if (my_store) {
#pragma unroll
                    for (int v = 0; v < MPI; v++)
                        if (j + v < m) out_w[(int64_t)(j + v) * a.stride] = park[v * 4 * MAX_CHUNKS + lane];
                }
            } else {
                // Blocked rows: the same chunk half of consecutive members is contiguous, so lane l stores word
                // l % 4 of chunk kk + l / 16 for member j + (l / 4) % 4: four full 64-byte runs per store.
                const uint32_t bk = (uint32_t)a.blk;
                const int v = (lane >> 2) & 3;
                uint32_t q = (uint32_t)(j + v) / bk, r = (uint32_t)(j + v) - q * bk;
                const int64_t moff = (int64_t)q * a.stride * bk + 2 * (int64_t)r;
#pragma unroll
                for (int kk = 0; kk < MAX_CHUNKS; kk += 2) {
                    const int k = kk + (lane >> 4);
                    const int i = 4 * k + (lane & 3);
                    if (k < MAX_CHUNKS && ((valid >> i) & 1u) && j + v < m)
                        a.dst[moff + proj_word_offset(a.out0 + 4 * (warp + P_WARPS * k) + (lane & 3), a.blk)] =
                            park[v * 4 * MAX_CHUNKS + i];
                }
            }
            __syncwarp();
        }
    }
    return true;
}

// Unit (segment s, work entry wi): the prefix words of the segment, the list of its prefix rows (local
// row ids, 16 bits), both in shared memory, then for every member its segment words staged in
// shared memory (one bulk copy per member, NSTAGE buffers in two slots of MPI, the next slot's copies
// in flight while one slot is gathered) and gathered at the listed rows with two ballots per 64 rows.
__global__ void __launch_bounds__(PT, 2) project_seg_kernel(const uint64_t* __restrict__ fbv, int64_t ld,
                                                         int64_t n_words, const int32_t* __restrict__ rows,
                                                         int width, const int64_t* __restrict__ grp_first,
                                                         const int32_t* __restrict__ grp_size,
                                                         const int64_t* __restrict__ work_groups, int64_t n_work,
                                                         int64_t n_seg, const int64_t* __restrict__ seg_off,
                                                         const int64_t* __restrict__ cbase,
                                                         const int64_t* __restrict__ cld,
                                                         uint64_t* __restrict__ cbuf,
                                                         unsigned long long* __restrict__ work_counter,
                                                         uint64_t first_wait_ns, int64_t blk) {
    extern __shared__ __align__(16) uint8_t psmem[];
    uint64_t* stage = reinterpret_cast<uint64_t*>(psmem);  // NSTAGE x (SEG_W member words + zero pad)
    uint64_t* pw = reinterpret_cast<uint64_t*>(psmem + NSTAGE * STAGE_BYTES);  // SEG_W prefix words
    uint16_t* list = reinterpret_cast<uint16_t*>(pw + SEG_W);
    __shared__ int32_t pref[64];
    __shared__ uint64_t park[P_WARPS * MPI * 4 * MAX_CHUNKS];
    __shared__ int32_t ids[ID_RING];
    __shared__ int64_t next_sh;
    __shared__ __align__(8) uint64_t bars[2];
    const int plen = width - 1;
    const int64_t total = n_seg * n_work;
    if (threadIdx.x == 0) {
        bar_init(&bars[0]);
        bar_init(&bars[1]);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    uint32_t phase = 0;  // bit s: parity of the next phase of group slot s
    bool stop = false;
    if (threadIdx.x < 2 * NSTAGE)  // the zero pads after the stage buffers (the copies never write them)
        reinterpret_cast<uint64_t*>(psmem + (threadIdx.x >> 1) * STAGE_BYTES + SEG_W * 8)[threadIdx.x & 1] = 0ULL;
    // Units in segment-major order; with a work counter each CTA claims the next unclaimed one.
    auto next_unit = [&](int64_t q) -> int64_t {
        if (threadIdx.x == 0)
            next_sh = work_counter != nullptr ? (int64_t)gridDim.x + (int64_t)atomicAdd(work_counter, 1ULL)
                                               : q + gridDim.x;
        __syncthreads();
        return next_sh;
    };
    for (int64_t q = blockIdx.x; q < total; q = next_unit(q)) {
        const int64_t s = q / n_work, wi = q - s * n_work;
        const int64_t g = work_groups[wi];
        const int64_t m = grp_size[g];
        const int64_t first = grp_first[g];
        const int64_t w0 = s * SEG_W;
        const int nw = (int)min64(SEG_W, n_words - w0);
        const int64_t* so = seg_off + wi * (n_seg + 1);
        const int64_t stride = cld[wi];
        uint64_t* dst = cbuf + cbase[wi];
        __syncthreads();  // the previous unit is done with the shared buffers (and with next_sh)
        // A segment without prefix rows adds no words to any member (the last one still zeroes the padding).
        if (s != n_seg - 1 && so[s + 1] == so[s]) continue;
        if (threadIdx.x < plen) pref[threadIdx.x] = rows[first * width + threadIdx.x];
        __syncthreads();
        int my = 0;
#pragma unroll
        for (int k = 0; k < SEG_W / PT; k++) {
            const int w = threadIdx.x * (SEG_W / PT) + k;
            const uint64_t p = w < nw ? prefix_word(fbv, ld, pref, plen, w0 + w) : 0ULL;
            pw[w] = p;
            my += __popcll(p);
        }
        int64_t cnt;
        const int64_t my_base = block_exclusive_scan(my, &cnt);
        for (int64_t p0 = 0; p0 < cnt; p0 += LIST_CAP) {
            // The prefix rows [p0, p0 + LIST_CAP) of the segment, as local row ids.
            int64_t at = my_base;
#pragma unroll
            for (int k = 0; k < SEG_W / PT; k++) {
                const int w = threadIdx.x * (SEG_W / PT) + k;
                uint64_t bits = pw[w];
                const int c = __popcll(bits);
                if (at + c > p0 && at < p0 + LIST_CAP) {
                    int64_t a = at;
                    while (bits) {
                        const int b = __ffsll((long long)bits) - 1;
                        if (a >= p0 && a < p0 + LIST_CAP) {
                            // Interleaved: rows 64 t + l and 64 t + 32 + l share 32-bit entry 32 t + l.
                            const int64_t x = a - p0;
                            list[((x >> 6) << 6) + ((x & 31) << 1) + ((x >> 5) & 1)] = (uint16_t)(w * 64 + b);
                        }
                        ++a;
                        bits &= bits - 1;
                    }
                }
                at += c;
            }
            const int pass_rows = (int)min64(LIST_CAP, cnt - p0);
            const int pass_words = (pass_rows + 63) >> 6;
            // Entries past the pass's last row name local row 0 (an in-range word); the store masks their bits.
            for (int x = pass_rows + threadIdx.x; x < ((pass_words + 3) & ~3) * 64; x += PT)
                list[((x >> 6) << 6) + ((x & 31) << 1) + ((x >> 5) & 1)] = 0;
            __syncthreads();
            const PassArgs pa{fbv, ld, rows, width, first, m, w0, nw, stage, reinterpret_cast<const uint32_t*>(list),
                              pass_rows, pass_words, dst, stride, so[s] + (p0 >> 6), blk, park, bars, ids,
                              first_wait_ns};
            if (!gather_members(pa, phase)) {
                stop = true;
                break;
            }
            __syncthreads();  // the next pass rewrites the list
        }
        if (stop) break;  // a bulk copy did not land within its bounded wait (block-uniform)
        if (s == n_seg - 1) {
            // Zero the words after the last piece, up to the member stride.
            const int64_t used = so[n_seg];
            const int64_t pad = stride - used;
            for (int64_t idx = threadIdx.x; idx < m * pad; idx += PT) {
                const int64_t j = idx / pad;
                const int64_t w = used + (idx - j * pad);
                dst[proj_member_offset(j, stride, blk) + proj_word_offset(w, blk)] = 0ULL;
            }
        }
    }
}

// ---- row-major projection -------------------------------------------------------------------------------------
//
// The same projected rows as project_seg_kernel, made from a row-major copy of the bitvectors (xt: word c of
// row r holds bit r of columns 32 c .. 32 c + 31). Per unit (segment, work entry) the segment's prefix rows
// are listed as before; then each warp takes 128 listed rows x 128 columns at a time: every lane loads the
// 16-byte word group of four listed rows, and four 32 x 32 bit transposes per 32-column chunk (five shuffle
// rounds each) turn rows into columns, so lane k ends with column 32 c + k's bits at the 128 rows: two
// projected words, stored with one 16-byte store when that column is a member of the group. Only the prefix
// rows' words are read (a segment's prefix rows are a few per cent of its rows at the densities the
// projection serves), where the column form reads every member's whole segment; a transpose costs about
// half an instruction per projected 32-bit word, a gather by ballots about three.
constexpr int RT = 256;
constexpr int R_WARPS = RT / 32;
constexpr int R_LIST = 8192;  // prefix rows listed per pass (128-row blocks: 64)

// Lane i holds row i of a 32 x 32 bit matrix (bit k = column k); the call returns column `lane` (bit i = row
// i). Round j swaps the off-diagonal j x j blocks of every 2j x 2j block, with the partner row taken by a
// shuffle (Hacker's Delight, "transpose32"): for j = 16 and 8 the swap moves whole bytes, one byte permute
// with a per-lane selector; for j = 4, 2, 1 the partner row is rotated by j one way or the other (a funnel
// shift by a per-lane amount) and merged under a per-lane mask (one three-input logic op). The per-lane
// constants are set once per thread.
struct Transpose32 {
    uint32_t sel16, sel8, rot4, rot2, rot1, keep4, keep2, keep1;
    __device__ explicit Transpose32(int lane) {
        sel16 = (lane & 16) ? 0x3276u : 0x5410u;
        sel8 = (lane & 8) ? 0x3715u : 0x6240u;
        rot4 = (lane & 4) ? 4u : 28u;
        rot2 = (lane & 2) ? 2u : 30u;
        rot1 = (lane & 1) ? 1u : 31u;
        keep4 = (lane & 4) ? ~0x0F0F0F0Fu : 0x0F0F0F0Fu;
        keep2 = (lane & 2) ? ~0x33333333u : 0x33333333u;
        keep1 = (lane & 1) ? ~0x55555555u : 0x55555555u;
    }
    __device__ __forceinline__ uint32_t operator()(uint32_t x) const {
        x = __byte_perm(x, __shfl_xor_sync(0xffffffffu, x, 16), sel16);
        x = __byte_perm(x, __shfl_xor_sync(0xffffffffu, x, 8), sel8);
        uint32_t y = __shfl_xor_sync(0xffffffffu, x, 4);
        x = (x & keep4) | (__funnelshift_r(y, y, rot4) & ~keep4);
        y = __shfl_xor_sync(0xffffffffu, x, 2);
        x = (x & keep2) | (__funnelshift_r(y, y, rot2) & ~keep2);
        y = __shfl_xor_sync(0xffffffffu, x, 1);
        x = (x & keep1) | (__funnelshift_r(y, y, rot1) & ~keep1);
        return x;
    }
};

__device__ __forceinline__ uint32_t u4_word(const uint4& v, int c) {
    return c == 0 ? v.x : c == 1 ? v.y : c == 2 ? v.z : v.w;
}

// xt [64 n_words][ldr]: one CTA of 256 threads per 128 rows x 256 columns; warp w transposes chunk 8 y + w of
// the two words of its 32 columns, and the tile goes out as 32 contiguous bytes per row (two threads a row).
constexpr int XT_THREADS = 256;
__global__ void __launch_bounds__(XT_THREADS) rows_transpose_kernel(const uint64_t* __restrict__ fbv, int64_t ld,
                                                           int64_t n_words, int64_t n_cols,
                                                           uint32_t* __restrict__ xt, int64_t ldr) {
    __shared__ uint32_t tile[128][9];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int64_t w = 2 * (int64_t)blockIdx.x;
    const int64_t c = (int64_t)blockIdx.y * 8 + warp;
    const int64_t col = c * 32 + lane;
    uint64_t a = 0, b = 0;
    if (col < n_cols) {
        a = __ldg(fbv + col * ld + w);
        if (w + 1 < n_words) b = __ldg(fbv + col * ld + w + 1);
    }
    const Transpose32 tp(lane);
    tile[lane][warp] = tp((uint32_t)a);
    tile[32 + lane][warp] = tp((uint32_t)(a >> 32));
    tile[64 + lane][warp] = tp((uint32_t)b);
    tile[96 + lane][warp] = tp((uint32_t)(b >> 32));
    __syncthreads();
    const int r = threadIdx.x >> 1, h = threadIdx.x & 1;
    const int64_t row = w * 64 + r;
    const int64_t c0 = (int64_t)blockIdx.y * 8 + 4 * h;
    if (row < n_words * 64 && c0 < ldr)
        *reinterpret_cast<uint4*>(xt + row * ldr + c0) =
            make_uint4(tile[r][4 * h], tile[r][4 * h + 1], tile[r][4 * h + 2], tile[r][4 * h + 3]);
}

__global__ void __launch_bounds__(RT, 3) project_rows_kernel(
    const uint64_t* __restrict__ fbv, int64_t ld, int64_t n_words, const uint32_t* __restrict__ xt, int64_t ldr,
    const int32_t* __restrict__ rows, int width, const int64_t* __restrict__ grp_first,
    const int32_t* __restrict__ grp_size, const int64_t* __restrict__ work_groups, int64_t n_work, int64_t n_seg,
    const int64_t* __restrict__ seg_off, const int64_t* __restrict__ cbase, const int64_t* __restrict__ cld,
    uint64_t* __restrict__ cbuf, int64_t blk) {
    extern __shared__ __align__(16) uint8_t rsm[];
    uint64_t* pw = reinterpret_cast<uint64_t*>(rsm);                  // SEG_W prefix words
    uint16_t* list = reinterpret_cast<uint16_t*>(pw + SEG_W);         // R_LIST listed rows (local ids)
    uint32_t* cmask = reinterpret_cast<uint32_t*>(list + R_LIST);     // the group's members per 32-column chunk
    int32_t* crank = reinterpret_cast<int32_t*>(cmask + ldr);         // members before each chunk
    int32_t* cgl = crank + ldr;                                       // 4-chunk groups holding a member
    __shared__ int32_t pref[64];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const Transpose32 tp(lane);
    const int plen = width - 1;
    const int64_t total = n_seg * n_work;
    // Units round-robin in segment-major order (CTA b takes b, b + grid, ...): the units are many and small, and
    // a fixed assignment keeps every launch's schedule independent of other streams' kernels.
    for (int64_t q = blockIdx.x; q < total; q += gridDim.x) {
        const int64_t s = q / n_work, wi = q - s * n_work;
        // Per-chunk tables (rewritten at the same addresses chunk after chunk) are read through L2 only.
        const int64_t g = __ldcg(work_groups + wi);
        const int64_t m = __ldcg(grp_size + g);
        const int64_t first = __ldcg(grp_first + g);
        const int64_t w0 = s * SEG_W;
        const int nw = (int)min64(SEG_W, n_words - w0);
        const int64_t* so = seg_off + wi * (n_seg + 1);
        const int64_t stride = __ldcg(cld + wi);
        const int64_t base = __ldcg(cbase + wi);
        uint64_t* dst = cbuf + base;
        __syncthreads();  // the previous unit is done with the shared buffers
        if (m <= 0) continue;
        // A segment without prefix rows adds no words to any member (the last one still zeroes the padding).
        if (s != n_seg - 1 && __ldcg(so + s + 1) == __ldcg(so + s)) continue;
        const int32_t* colp = rows + first * width + width - 1;
        const int c_lo = (colp[0] >> 5) & ~3;
        const int nch = ((colp[(m - 1) * width] >> 5) - c_lo + 4) & ~3;  // chunks covered, whole 4-chunk groups
        // Refused units (the status word reports them): a member past the row-major copy, or member rows that
        // are not 16-byte aligned (odd base or stride), which the 16-byte stores below need.
        if (c_lo + nch > ldr || ((base | stride) & 1) != 0) {
            if (threadIdx.x == 0) atomicExch(&g_proj_status, ETM_EINVAL);
            continue;
        }
        if (threadIdx.x < plen) pref[threadIdx.x] = rows[first * width + threadIdx.x];
        for (int t = threadIdx.x; t < nch; t += RT) cmask[t] = 0u;
        __syncthreads();
        for (int64_t i = threadIdx.x; i < m; i += RT) {
            const int it = colp[i * width];
            atomicOr(&cmask[(it >> 5) - c_lo], 1u << (it & 31));
        }
        __syncthreads();
        // Member ranks per chunk and the list of non-empty 4-chunk groups (ordered scans).
        int64_t carry = 0, n_cg = 0;
        for (int c0 = 0; c0 < nch; c0 += RT) {
            const int c = c0 + threadIdx.x;
            const uint32_t mk = c < nch ? cmask[c] : 0u;
            int64_t tot, tg;
            const int64_t ex = block_exclusive_scan(__popc(mk), &tot);
            if (c < nch) crank[c] = (int32_t)(carry + ex);
            carry += tot;
            const int head = c < nch && (c & 3) == 0 && (cmask[c] | cmask[c + 1] | cmask[c + 2] | cmask[c + 3]) != 0u;
            const int64_t eg = block_exclusive_scan(head, &tg);
            if (head) cgl[n_cg + eg] = c;
            n_cg += tg;
        }
        int my = 0;
#pragma unroll
        for (int k = 0; k < SEG_W / RT; k++) {
            const int w = threadIdx.x * (SEG_W / RT) + k;
            const uint64_t p = w < nw ? prefix_word(fbv, ld, pref, plen, w0 + w) : 0ULL;
            pw[w] = p;
            my += __popcll(p);
        }
        int64_t cnt;
        const int64_t my_base = block_exclusive_scan(my, &cnt);
        const int64_t row0 = w0 * 64;
        for (int64_t p0 = 0; p0 < cnt; p0 += R_LIST) {
            int64_t at = my_base;
#pragma unroll
            for (int k = 0; k < SEG_W / RT; k++) {
                const int w = threadIdx.x * (SEG_W / RT) + k;
                uint64_t bits = pw[w];
                const int c = __popcll(bits);
                if (at + c > p0 && at < p0 + R_LIST) {
                    int64_t a = at;
                    while (bits) {
                        const int b = __ffsll((long long)bits) - 1;
                        if (a >= p0 && a < p0 + R_LIST) list[a - p0] = (uint16_t)(w * 64 + b);
                        ++a;
                        bits &= bits - 1;
                    }
                }
                at += c;
            }
            const int pass_rows = (int)min64(R_LIST, cnt - p0);
            const int pass_words = (pass_rows + 63) >> 6;
            const int nblk = ((pass_words + 3) & ~3) >> 1;  // 128-row blocks up to the piece's 4-word chunk
            const int64_t out0 = __ldcg(so + s) + (p0 >> 6);
            __syncthreads();
            const int64_t n_it = (int64_t)nblk * n_cg;
            for (int64_t it = warp; it < n_it; it += R_WARPS) {
                const int b = (int)(it / n_cg);
                const int cg = cgl[it - (int64_t)b * n_cg];
                uint4 v[4];
#pragma unroll
                for (int qq = 0; qq < 4; qq++) {
                    const int x = b * 128 + qq * 32 + lane;
                    v[qq] = make_uint4(0u, 0u, 0u, 0u);
                    if (x < pass_rows)
                        v[qq] = __ldg(reinterpret_cast<const uint4*>(xt + (row0 + list[x]) * ldr + c_lo + cg));
                }
                const int64_t wo = proj_word_offset(out0 + 2 * b, blk);  // words 2b and 2b + 1 are adjacent
#pragma unroll
                for (int cc = 0; cc < 4; cc++) {
                    const uint32_t mk = cmask[cg + cc];
                    if (mk == 0u) continue;  // warp-uniform
                    const uint32_t t0 = tp(u4_word(v[0], cc));
                    const uint32_t t1 = tp(u4_word(v[1], cc));
                    const uint32_t t2 = tp(u4_word(v[2], cc));
                    const uint32_t t3 = tp(u4_word(v[3], cc));
                    if ((mk >> lane) & 1u) {
                        const int64_t i = crank[cg + cc] + __popc(mk & ((1u << lane) - 1u));
                        *reinterpret_cast<ulonglong2*>(dst + proj_member_offset(i, stride, blk) + wo) =
                            make_ulonglong2((uint64_t)t0 | ((uint64_t)t1 << 32), (uint64_t)t2 | ((uint64_t)t3 << 32));
                    }
                }
            }
            __syncthreads();  // the next pass rewrites the list
        }
        if (s == n_seg - 1) {
            // Zero the words after the last piece, up to the member stride.
            const int64_t used = __ldcg(so + n_seg);
            const int64_t pad = stride - used;
            for (int64_t idx = threadIdx.x; idx < m * pad; idx += RT) {
                const int64_t j = idx / pad;
                const int64_t w = used + (idx - j * pad);
                dst[proj_member_offset(j, stride, blk) + proj_word_offset(w, blk)] = 0ULL;
            }
        }
    }
}

}  // namespace

namespace etm {

void proj_set_first_wait(int64_t ns) { g_proj_first_wait_ns.store(ns < 0 ? BULK_WAIT_NS : (uint64_t)ns); }

// The projection's status word (ETM_ETIMEOUT after a bulk copy outlived its bounded wait), read and
// cleared on `s`.
int proj_status_take(cudaStream_t s, int* out) {
    int v = 0;
    ETM_CUDA(cudaMemcpyFromSymbolAsync(&v, g_proj_status, sizeof(int), 0, cudaMemcpyDeviceToHost, s));
    ETM_CUDA(cudaStreamSynchronize(s));
    if (v != 0) {
        const int zero = 0;
        ETM_CUDA(cudaMemcpyToSymbolAsync(g_proj_status, &zero, sizeof(int), 0, cudaMemcpyHostToDevice, s));
        ETM_CUDA(cudaStreamSynchronize(s));
    }
    *out = v;
    return ETM_OK;
}

}  // namespace etm

extern "C" int etm_prefix_counts(const uint64_t* fbv, int64_t ld, int64_t n_words, const int32_t* rows, int32_t width,
                                 const int64_t* grp_first, const int64_t* work_groups, int64_t n_work,
                                 int64_t* out_counts, const uint64_t* occ, int64_t occ_ld, void* stream) {
    ETM_REQUIRE(width >= 2 && width <= 64, ETM_EINVAL, "etm_prefix_counts: width %d out of range (2..64)", width);
    ETM_REQUIRE(ld >= n_words, ETM_EINVAL, "etm_prefix_counts: ld < n_words");
    ETM_REQUIRE(n_work < (1LL << 31), ETM_EINVAL, "etm_prefix_counts: too many groups");
    ETM_REQUIRE(occ == nullptr || occ_ld >= ceil_div<int64_t>(n_words, OCC_SPAN), ETM_EINVAL,
                "etm_prefix_counts: occ_ld too small for n_words");
    if (n_work <= 0) return ETM_OK;
    prefix_counts_kernel<<<(unsigned)n_work, PT, 0, as_stream(stream)>>>(fbv, ld, n_words, rows, width, grp_first,
                                                                         work_groups, out_counts, occ, occ_ld);
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

extern "C" int etm_prefix_segments(const uint64_t* fbv, int64_t ld, int64_t n_words, const int32_t* rows,
                                   int32_t width, const int64_t* grp_first, const int64_t* work_groups,
                                   int64_t n_work, int64_t* seg_off, int64_t* out_words, const uint64_t* occ,
                                   int64_t occ_ld, void* stream) {
    ETM_REQUIRE(width >= 2 && width <= 64, ETM_EINVAL, "etm_prefix_segments: width %d out of range (2..64)", width);
    ETM_REQUIRE(ld >= n_words && n_words >= 0, ETM_EINVAL, "etm_prefix_segments: bad n_words / ld");
    ETM_REQUIRE(occ == nullptr || occ_ld >= ceil_div<int64_t>(n_words, OCC_SPAN), ETM_EINVAL,
                "etm_prefix_segments: occ_ld too small for n_words");
    ETM_REQUIRE(n_work < (1LL << 31), ETM_EINVAL, "etm_prefix_segments: too many groups");
    if (n_work <= 0) return ETM_OK;
    const int64_t n_seg = ceil_div<int64_t>(n_words, SEG_W);
    prefix_segments_kernel<<<(unsigned)n_work, PT, 0, as_stream(stream)>>>(fbv, ld, n_words, rows, width, grp_first,
                                                                           work_groups, n_seg, seg_off, out_words,
                                                                           occ, occ_ld);
    ETM_LAUNCHED("prefix_segments");
    return ETM_OK;
}

static int project_impl(const uint64_t* fbv, int64_t ld, int64_t n_words, const int32_t* rows, int32_t width,
                        const int64_t* grp_first, const int32_t* grp_size, const int64_t* work_groups, int64_t n_work,
                        const int64_t* seg_off, const int64_t* cbase, const int64_t* cld, uint64_t* cbuf,
                        int64_t* work_counter, int64_t blk, void* stream) {
    ETM_REQUIRE(blk >= 0 && blk <= 4096, ETM_EINVAL, "etm_project: blk %lld out of range (0..4096)", (long long)blk);
    ETM_REQUIRE(width >= 2 && width <= 64, ETM_EINVAL, "etm_project: width %d out of range (2..64)", width);
    ETM_REQUIRE(ld >= n_words && n_words >= 0 && ld % 2 == 0, ETM_EINVAL, "etm_project: ld must be even and >= n_words");
    ETM_REQUIRE((reinterpret_cast<uintptr_t>(fbv) & 15) == 0, ETM_EINVAL, "etm_project: fbv must be 16-byte aligned");
    if (n_work <= 0 || n_words == 0) return ETM_OK;
    static bool configured = false;
    if (!configured) {
        ETM_CUDA(cudaFuncSetAttribute(project_seg_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, PROJ_SMEM));
        configured = true;
    }
    const int64_t n_seg = ceil_div<int64_t>(n_words, SEG_W);
    const int64_t units = n_seg * n_work;
    const int grid = (int)min64(units, (int64_t)max(1, sm_count()) * 2);
    if (work_counter != nullptr) ETM_CUDA(cudaMemsetAsync(work_counter, 0, sizeof(int64_t), as_stream(stream)));
    project_seg_kernel<<<grid, PT, PROJ_SMEM, as_stream(stream)>>>(fbv, ld, n_words, rows, width, grp_first, grp_size,
                                                                   work_groups, n_work, n_seg, seg_off, cbase, cld,
                                                                   cbuf,
                                                                   reinterpret_cast<unsigned long long*>(work_counter),
                                                                   g_proj_first_wait_ns.load(), blk);
    ETM_LAUNCHED("project");
    return ETM_OK;
}

extern "C" int etm_project(const uint64_t* fbv, int64_t ld, int64_t n_words, const int32_t* rows, int32_t width,
                           const int64_t* grp_first, const int32_t* grp_size, const int64_t* work_groups,
                           int64_t n_work, const int64_t* seg_off, const int64_t* cbase, const int64_t* cld,
                           uint64_t* cbuf, int64_t* work_counter, void* stream) {
    return project_impl(fbv, ld, n_words, rows, width, grp_first, grp_size, work_groups, n_work, seg_off, cbase, cld,
                        cbuf, work_counter, 0, stream);
}

extern "C" int etm_project_blocked(const uint64_t* fbv, int64_t ld, int64_t n_words, const int32_t* rows,
                                   int32_t width, const int64_t* grp_first, const int32_t* grp_size,
                                   const int64_t* work_groups, int64_t n_work, const int64_t* seg_off,
                                   const int64_t* cbase, const int64_t* cld, int64_t blk, uint64_t* cbuf,
                                   int64_t* work_counter, void* stream) {
    ETM_REQUIRE(blk >= 1, ETM_EINVAL, "etm_project_blocked: blk must be >= 1");
    return project_impl(fbv, ld, n_words, rows, width, grp_first, grp_size, work_groups, n_work, seg_off, cbase, cld,
                        cbuf, work_counter, blk, stream);
}

extern "C" int etm_rows_transpose(const uint64_t* fbv, int64_t ld, int64_t n_words, int64_t n_cols, uint32_t* xt,
                                  int64_t ldr, void* stream) {
    ETM_REQUIRE(ld >= n_words && n_words >= 0 && n_cols >= 0, ETM_EINVAL, "etm_rows_transpose: bad sizes");
    ETM_REQUIRE(ldr % 4 == 0 && ldr * 32 >= n_cols, ETM_EINVAL,
                "etm_rows_transpose: ldr must be a multiple of 4 with 32 ldr >= n_cols");
    ETM_REQUIRE((reinterpret_cast<uintptr_t>(xt) & 15) == 0, ETM_EINVAL, "etm_rows_transpose: xt must be 16-byte aligned");
    ETM_REQUIRE(n_words < (1LL << 32) && ldr / 8 < 65535, ETM_EINVAL, "etm_rows_transpose: too large");
    if (n_words == 0 || ldr == 0) return ETM_OK;
    const dim3 grid((unsigned)ceil_div<int64_t>(n_words, 2), (unsigned)ceil_div<int64_t>(ldr, 8));
    rows_transpose_kernel<<<grid, XT_THREADS, 0, as_stream(stream)>>>(fbv, ld, n_words, n_cols, xt, ldr);
    ETM_LAUNCHED("rows_transpose");
    return ETM_OK;
}

extern "C" int etm_project_rows(const uint64_t* fbv, int64_t ld, int64_t n_words, const uint32_t* xt, int64_t ldr,
                                const int32_t* rows, int32_t width, const int64_t* grp_first, const int32_t* grp_size,
                                const int64_t* work_groups, int64_t n_work, const int64_t* seg_off,
                                const int64_t* cbase, const int64_t* cld, int64_t blk, uint64_t* cbuf, void* stream) {
    ETM_REQUIRE(blk >= 0 && blk <= 4096, ETM_EINVAL, "etm_project_rows: blk %lld out of range (0..4096)", (long long)blk);
    ETM_REQUIRE(width >= 2 && width <= 64, ETM_EINVAL, "etm_project_rows: width %d out of range (2..64)", width);
    ETM_REQUIRE(ld >= n_words && n_words >= 0, ETM_EINVAL, "etm_project_rows: ld < n_words");
    ETM_REQUIRE(ldr % 4 == 0 && ldr > 0, ETM_EINVAL, "etm_project_rows: ldr must be a positive multiple of 4");
    ETM_REQUIRE((reinterpret_cast<uintptr_t>(xt) & 15) == 0 && (reinterpret_cast<uintptr_t>(cbuf) & 15) == 0,
                ETM_EINVAL, "etm_project_rows: xt and cbuf must be 16-byte aligned");
    if (n_work <= 0 || n_words == 0) return ETM_OK;
    const int smem = SEG_W * 8 + R_LIST * 2 + (int)ldr * 8 + (int)(ldr / 4 + 1) * 4;
    ETM_REQUIRE(smem <= 200 * 1024, ETM_EINVAL, "etm_project_rows: %lld row words need too much shared memory",
                (long long)ldr);
    static int configured = 0;
    if (smem > 48 * 1024 && smem > configured) {
        ETM_CUDA(cudaFuncSetAttribute(project_rows_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
        configured = smem;
    }
    const int64_t n_seg = ceil_div<int64_t>(n_words, SEG_W);
    const int64_t units = n_seg * n_work;
    const int grid = (int)min64(units, (int64_t)max(1, sm_count()) * 3);
    project_rows_kernel<<<grid, RT, smem, as_stream(stream)>>>(fbv, ld, n_words, xt, ldr, rows, width, grp_first,
                                                               grp_size, work_groups, n_work, n_seg, seg_off, cbase,
                                                               cld, cbuf, blk);
    ETM_LAUNCHED("project_rows");
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
                                          chunk_base, cls, out_counts, as_stream(stream), 0, nullptr);
}

extern "C" int etm_count_tiles_proj_sel(const uint64_t* cbuf, const int64_t* cbase, const int64_t* cwords,
                                        const int64_t* cld, const int32_t* grp_size, const int64_t* cand_off,
                                        const int64_t* work_groups, const int64_t* work_off, int64_t n_work,
                                        int64_t chunk_base, const uint8_t* cls, int32_t min_count, int32_t* out_counts,
                                        uint32_t* surv_bits, void* stream) {
    ETM_REQUIRE((reinterpret_cast<uintptr_t>(cbuf) & 15) == 0, ETM_EINVAL,
                "etm_count_tiles_proj_sel: cbuf must be 16-byte aligned");
    ETM_REQUIRE(surv_bits != nullptr, ETM_EINVAL, "etm_count_tiles_proj_sel: surv_bits is required");
    if (n_work <= 0) return ETM_OK;
    return etm::count_tiles_proj_popcount(cbuf, cbase, cwords, cld, grp_size, cand_off, work_groups, work_off, n_work,
                                          chunk_base, cls, out_counts, as_stream(stream), min_count, surv_bits);
}
