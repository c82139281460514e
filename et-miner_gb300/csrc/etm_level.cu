// Level bookkeeping on the device: prefix groups of a sorted level, the
// (k-1)-subset test with count inference, order-preserving survivor
// compaction (which decodes candidates straight into the next level's
// lexsorted rows), free flags, and the free-set prune.
//
// Every pass is one thread per element over arrays in HBM; the compactions
// are the three-launch ordered scans of etm_scan.cuh, so no host sort and no
// host decode is ever needed.
#include <mutex>

#include "etm_scan.cuh"

namespace {

using namespace etm;

constexpr int MAXK = 64;  // longest itemset handled (the reference caps K at 62, loader.py:25-37)

// Row of the sorted level rows[n][width] equal to items[] without position `skip`
// (items holds width+1 columns), or -1.
__device__ int64_t find_subset(const int32_t* __restrict__ rows, int64_t n, int width, const int32_t* items,
                               int skip) {
    int64_t lo = 0, hi = n;
    while (lo < hi) {
        const int64_t mid = lo + ((hi - lo) >> 1);
        const int32_t* r = rows + mid * width;
        int cmp = 0;
        for (int t = 0; t < width; t++) {
            const int32_t v = items[t < skip ? t : t + 1];
            const int32_t x = __ldg(r + t);
            if (x != v) {
                cmp = x < v ? -1 : 1;
                break;
            }
        }
        if (cmp == 0) return mid;
        if (cmp < 0) lo = mid + 1;
        else hi = mid;
    }
    return -1;
}

// Row of the sorted level rows[n][m] equal to items[0..m), or -1.
__device__ int64_t find_items(const int32_t* __restrict__ rows, int64_t n, int m, const int32_t* items) {
    int64_t lo = 0, hi = n;
    while (lo < hi) {
        const int64_t mid = lo + ((hi - lo) >> 1);
        const int32_t* r = rows + mid * m;
        int cmp = 0;
        for (int t = 0; t < m && cmp == 0; t++) {
            const int32_t x = __ldg(r + t);
            cmp = x < items[t] ? -1 : (x > items[t] ? 1 : 0);
        }
        if (cmp == 0) return mid;
        if (cmp < 0) lo = mid + 1;
        else hi = mid;
    }
    return -1;
}

// ---- deduction bounds ----------------------------------------------------------
//
// The count of an itemset X of k items is bounded by inclusion-exclusion over its subsets (Calders &
// Goethals 2002; the depth <= 3 rules of _deduce, gpu/kernels/_src/_subset_index.cu:95-136):
//   upper u = min( min_a s(X-a), min_{a<b<c} s(X-a)+s(X-b)+s(X-c) - s(X-ab)-s(X-ac)-s(X-bc) + s(X-abc) )
//   lower l = max( 0, max_{a<b} s(X-a) + s(X-b) - s(X-ab) )
// with s(X-a) from level k-1, s(X-ab) from level k-2 and s(X-abc) from level k-3 (the empty set's count,
// the row count, at k = 3). u < min_count: X is infrequent; l = u: X's count is u. Both hold exactly for
// integer counts, so settling a candidate by them changes no result.
constexpr int BOUNDS_MAX_K = 24;

struct DeepLevels {
    const int32_t* rows2;   // level k-2: rows [n2][k-2], sorted, and counts
    int64_t n2;
    const int32_t* counts2;
    const int32_t* rows3;   // level k-3 (k > 3)
    int64_t n3;
    const int32_t* counts3;
    int64_t n_total;        // the row count: s of the empty set (k = 3)
};

// ETM_CAND_SKIP, ETM_CAND_INFER (count in *inferred) or ETM_CAND_COUNT for X = items[0..k), c1[t] = s(X - item t).
__device__ __noinline__ uint8_t deduce(const int32_t* items, int k, const int32_t* c1, const DeepLevels& deep,
                                       int32_t min_count, int32_t* inferred) {
    int32_t s2[BOUNDS_MAX_K * (BOUNDS_MAX_K - 1) / 2];
    int32_t sub[BOUNDS_MAX_K];
    int64_t lower = 0, upper = 0x7FFFFFFF;
    for (int t = 0; t < k; t++) upper = min(upper, (int64_t)c1[t]);
    for (int j = 1; j < k; j++) {
        for (int i = 0; i < j; i++) {
            int n = 0;
            for (int t = 0; t < k; t++)
                if (t != i && t != j) sub[n++] = items[t];
            const int64_t r = find_items(deep.rows2, deep.n2, k - 2, sub);
            if (r < 0) return ETM_CAND_COUNT;  // an infrequent (k-2)-subset: counting settles it
            const int32_t c = deep.counts2[r];
            s2[j * (j - 1) / 2 + i] = c;
            lower = max(lower, (int64_t)c1[i] + c1[j] - c);
        }
    }
    for (int l = 2; l < k && lower < upper && upper >= min_count; l++) {
        for (int j = 1; j < l && lower < upper; j++) {
            for (int i = 0; i < j && lower < upper; i++) {
                int64_t c3 = deep.n_total;
                if (k > 3) {
                    int n = 0;
                    for (int t = 0; t < k; t++)
                        if (t != i && t != j && t != l) sub[n++] = items[t];
                    const int64_t r = find_items(deep.rows3, deep.n3, k - 3, sub);
                    if (r < 0) return ETM_CAND_COUNT;
                    c3 = deep.counts3[r];
                }
                const int64_t u3 = (int64_t)c1[i] + c1[j] + c1[l] - s2[j * (j - 1) / 2 + i] - s2[l * (l - 1) / 2 + i] -
                                   s2[l * (l - 1) / 2 + j] + c3;
                upper = min(upper, u3);
            }
        }
    }
    if (upper < min_count) return ETM_CAND_SKIP;
    if (lower == upper) {
        *inferred = (int32_t)upper;
        return ETM_CAND_INFER;
    }
    return ETM_CAND_COUNT;
}

// ---- prefix groups --------------------------------------------------------

struct RunStart {
    const int32_t* rows;
    int64_t n;
    int width;
    __device__ int64_t operator()(int64_t t) const {
        if (t >= n) return 0;
        if (t == 0) return 1;
        const int32_t* a = rows + t * width;
        const int32_t* b = a - width;
        for (int c = 0; c < width - 1; c++)
            if (a[c] != b[c]) return 1;
        return 0;
    }
};

struct WriteAt {
    int64_t* out;
    __device__ void operator()(int64_t t, int64_t off) const { out[off] = t; }
};

struct RunIsGroup {
    const int64_t* run_first;
    const int64_t* n_runs;
    int64_t n;
    __device__ int64_t size(int64_t r) const {
        const int64_t R = *n_runs;
        if (r >= R) return 0;
        return (r + 1 < R ? run_first[r + 1] : n) - run_first[r];
    }
    __device__ int64_t operator()(int64_t r) const { return size(r) >= 2 ? 1 : 0; }
};

struct EmitGroup {
    RunIsGroup runs;
    int64_t* grp_first;
    int32_t* grp_size;
    __device__ void operator()(int64_t r, int64_t off) const {
        grp_first[off] = runs.run_first[r];
        grp_size[off] = (int32_t)runs.size(r);
    }
};

struct GroupPairs {
    const int32_t* grp_size;
    const int64_t* n_groups;
    __device__ int64_t operator()(int64_t g) const {
        return g < *n_groups ? pairs_of((int64_t)grp_size[g]) : 0;
    }
};

struct WriteOffset {
    int64_t* out;
    __device__ void operator()(int64_t g, int64_t off) const { out[g] = off; }
};

__global__ void finish_groups_kernel(int64_t* cand_off, int64_t* counters, const int64_t* n_groups,
                                     const int64_t* total) {
    counters[0] = *n_groups;
    counters[1] = *total;
    cand_off[*n_groups] = *total;
}

// ---- subset test / inference ------------------------------------------------

struct Cand {
    int64_t g, i, j, local;
};

__device__ inline Cand decode_candidate(const int64_t* __restrict__ cand_off, const int32_t* __restrict__ grp_size,
                                        int64_t g0, int64_t g1, int64_t abs_t) {
    Cand c;
    c.g = g0 + upper_find(cand_off + g0, g1 - g0, abs_t);
    c.local = abs_t - cand_off[c.g];
    tri_decode(c.local, grp_size[c.g], &c.i, &c.j);
    return c;
}

// items[0..width] of candidate (group first, members i < j): prefix + s_i + s_j.
__device__ inline void candidate_items(const int32_t* __restrict__ rows, int width, int64_t first, int64_t i,
                                       int64_t j, int32_t* items) {
    const int32_t* ri = rows + (first + i) * width;
    for (int c = 0; c < width; c++) items[c] = ri[c];
    items[width] = rows[(first + j) * width + width - 1];
}

__global__ void classify_kernel(const int32_t* __restrict__ rows, int width, int64_t n_rows,
                                const int32_t* __restrict__ counts, const uint8_t* __restrict__ free_flags,
                                const int64_t* __restrict__ grp_first, const int32_t* __restrict__ grp_size,
                                const int64_t* __restrict__ cand_off, int64_t g0, int64_t g1, int mode,
                                uint8_t* __restrict__ out_cls, int32_t* __restrict__ out_counts, int32_t min_count,
                                uint32_t* __restrict__ surv, DeepLevels deep) {
    const int64_t base = cand_off[g0];
    const int64_t n = cand_off[g1] - base;
    const bool prune = mode & ETM_SUBSET_PRUNE, infer = (mode & ETM_SUBSET_INFER) && free_flags && counts;
    const bool bounds = infer && (mode & ETM_SUBSET_BOUNDS) && width + 1 <= BOUNDS_MAX_K && deep.rows2 != nullptr;
    int32_t items[MAXK];
    int32_t c1[BOUNDS_MAX_K];
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
        const Cand c = decode_candidate(cand_off, grp_size, g0, g1, base + t);
        const int64_t first = grp_first[c.g];
        candidate_items(rows, width, first, c.i, c.j, items);
        uint8_t cls = ETM_CAND_COUNT;
        int32_t lowest = 0x7fffffff;
        bool not_free = false, missing = false;
        // Subsets dropping a prefix item; the two dropping a suffix are the members i and j.
        for (int d = 0; d < width - 1 && !missing; d++) {
            const int64_t r = find_subset(rows, n_rows, width, items, d);
            if (r < 0) {
                missing = true;
            } else if (infer) {
                lowest = min(lowest, counts[r]);
                not_free |= free_flags[r] == 0;
                if (bounds) c1[d] = counts[r];
            }
        }
        if (missing) {
            cls = prune ? ETM_CAND_SKIP : ETM_CAND_COUNT;
        } else if (infer) {
            const int64_t ri = first + c.i, rj = first + c.j;
            lowest = min(lowest, min(counts[ri], counts[rj]));
            not_free |= (free_flags[ri] == 0) | (free_flags[rj] == 0);
            int32_t value = lowest;
            if (not_free) {
                cls = ETM_CAND_INFER;
            } else if (bounds) {
                // X without s_i is member j's row, X without s_j is member i's row.
                c1[width - 1] = counts[rj];
                c1[width] = counts[ri];
                cls = deduce(items, width + 1, c1, deep, min_count, &value);
            }
            if (cls == ETM_CAND_INFER) {
                out_counts[t] = value;
                if (surv != nullptr && value >= min_count) atomicOr(surv + (t >> 5), 1u << (t & 31));
            }
        }
        out_cls[t] = cls;
    }
}

// ---- survivor compaction --------------------------------------------------------

struct Survives {
    const int32_t* counts;
    const uint8_t* cls;
    int64_t n;
    int32_t min_count;
    __device__ int64_t operator()(int64_t t) const {
        if (t >= n) return 0;
        if (cls && cls[t] == ETM_CAND_SKIP) return 0;
        return counts[t] >= min_count ? 1 : 0;
    }
};

struct EmitSurvivor {
    const int32_t* counts;
    const int32_t* rows;
    int width;
    const int64_t* grp_first;
    const int32_t* grp_size;
    const int64_t* cand_off;
    int64_t g0, g1;
    int32_t* out_rows;
    int32_t* out_counts;
    int64_t cap;
    __device__ void operator()(int64_t t, int64_t off) const {
        if (off >= cap) return;
        const Cand c = decode_candidate(cand_off, grp_size, g0, g1, cand_off[g0] + t);
        const int64_t first = grp_first[c.g];
        const int32_t* ri = rows + (first + c.i) * width;
        int32_t* o = out_rows + off * (width + 1);
        for (int q = 0; q < width; q++) o[q] = ri[q];
        o[width] = rows[(first + c.j) * width + width - 1];
        out_counts[off] = counts[t];
    }
};

// Survivor bits of a counted chunk from its dense counts: one thread per 32-candidate word.
__global__ void threshold_bits_kernel(const int32_t* __restrict__ counts, const uint8_t* __restrict__ cls, int64_t n,
                                      int32_t min_count, uint32_t* __restrict__ surv) {
    const int64_t n_w = (n + 31) >> 5;
    for (int64_t w = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; w < n_w; w += (int64_t)gridDim.x * blockDim.x) {
        uint32_t bits = 0;
        const int64_t t0 = w << 5;
        const int nb = (int)min64(32, n - t0);
        for (int b = 0; b < nb; b++) {
            const int64_t t = t0 + b;
            const bool keep = counts[t] >= min_count && (cls == nullptr || cls[t] != ETM_CAND_SKIP);
            bits |= (keep ? 1u : 0u) << b;
        }
        surv[w] = bits;
    }
}

// Ordered compaction over a survivor bitmask: the scan runs over 32-candidate words.
struct WordSurvivors {
    const uint32_t* surv;
    int64_t n;
    __device__ uint32_t bits(int64_t w) const {
        const int64_t t0 = w << 5;
        if (t0 >= n) return 0u;
        const uint32_t b = surv[w];
        return n - t0 >= 32 ? b : b & ((1u << (n - t0)) - 1u);
    }
    __device__ int64_t operator()(int64_t w) const { return __popc(bits(w)); }
};

// The survivors of one 32-candidate word, in order. The word's first survivor is decoded in full (group by
// binary search, (i, j) from the triangular index); each later one by walking (group, i, j) forward over the
// candidates between them, with integer steps only: no search and no square root per survivor, which is what
// bounds words dense in survivors.
struct EmitWordSurvivors {
    WordSurvivors words;
    EmitSurvivor emit;
    __device__ void operator()(int64_t w, int64_t off) const {
        uint32_t b = words.bits(w);
        if (b == 0u) return;
        int64_t pos = (w << 5) + (__ffs(b) - 1);
        const Cand c = decode_candidate(emit.cand_off, emit.grp_size, emit.g0, emit.g1, emit.cand_off[emit.g0] + pos);
        int64_t g = c.g, i = c.i, j = c.j;
        int64_t m = emit.grp_size[g], first = emit.grp_first[g];
        const int width = emit.width;
        for (;;) {
            if (off < emit.cap) {
                const int32_t* ri = emit.rows + (first + i) * width;
                int32_t* o = emit.out_rows + off * (width + 1);
                for (int q = 0; q < width; q++) o[q] = ri[q];
                o[width] = emit.rows[(first + j) * width + width - 1];
                emit.out_counts[off] = emit.counts[pos];
            }
            ++off;
            b &= b - 1u;
            if (b == 0u) return;
            const int64_t next = (w << 5) + (__ffs(b) - 1);
            for (int64_t d = next - pos; d > 0; d--) {
                if (++j == m) {
                    if (++i == m - 1) {  // past the group's last pair: the next group holding a pair
                        do {
                            ++g;
                        } while (g + 1 < emit.g1 && emit.grp_size[g] < 2);
                        m = emit.grp_size[g];
                        first = emit.grp_first[g];
                        i = 0;
                    }
                    j = i + 1;
                }
            }
            pos = next;
        }
    }
};

// ---- free flags / subset presence --------------------------------------------------------

__global__ void subsets_kernel(const int32_t* __restrict__ new_rows, const int32_t* __restrict__ new_counts,
                               int64_t n_new, int width, const int32_t* __restrict__ prev_rows,
                               const int32_t* __restrict__ prev_counts, int64_t n_prev, uint8_t* __restrict__ out_free,
                               uint8_t* __restrict__ out_present) {
    int32_t items[MAXK];
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n_new; t += (int64_t)gridDim.x * blockDim.x) {
        const int32_t* r = new_rows + t * (width + 1);
        for (int c = 0; c <= width; c++) items[c] = r[c];
        const int32_t cnt = new_counts[t];
        bool free_ = true, present = true;
        for (int d = 0; d <= width; d++) {
            const int64_t p = find_subset(prev_rows, n_prev, width, items, d);
            if (p < 0) present = false;
            else if (prev_counts[p] == cnt) free_ = false;
        }
        if (out_free) out_free[t] = free_;
        if (out_present) out_present[t] = present;
    }
}

struct Kept {
    const uint8_t* a;
    const uint8_t* b;
    int64_t n;
    __device__ int64_t operator()(int64_t t) const {
        if (t >= n) return 0;
        return (a[t] != 0 && (b == nullptr || b[t] != 0)) ? 1 : 0;
    }
};

struct CopyRow {
    const int32_t* rows;
    const int32_t* counts;
    const uint8_t* flag_src;
    int width;
    int32_t* out_rows;
    int32_t* out_counts;
    uint8_t* out_flag;
    int64_t cap;
    __device__ void operator()(int64_t t, int64_t off) const {
        if (off >= cap) return;
        for (int c = 0; c < width; c++) out_rows[off * width + c] = rows[t * width + c];
        out_counts[off] = counts[t];
        if (out_flag && flag_src) out_flag[off] = flag_src[t];
    }
};

int grid_for(int64_t n, int threads) {
    const int64_t want = ceil_div<int64_t>(n, threads);
    const int64_t cap = (int64_t)max(1, sm_count()) * 16;
    return (int)max64(1, min(want, cap));
}

}  // namespace

extern "C" int etm_level_groups(const int32_t* rows, int64_t n, int32_t width, int64_t* grp_first, int32_t* grp_size,
                                int64_t* cand_off, int64_t* counters, int64_t* ws, int64_t ws_words, void* stream) {
    ETM_REQUIRE(width >= 1 && width < MAXK, ETM_EINVAL, "etm_level_groups: width %d out of range", width);
    ETM_REQUIRE(n >= 0, ETM_EINVAL, "etm_level_groups: negative n");
    const int64_t need = 3 + scan_workspace_words(n);
    ETM_REQUIRE(ws_words >= need, ETM_ENOSPACE, "etm_level_groups: workspace %lld words, need %lld",
                (long long)ws_words, (long long)need);
    cudaStream_t s = as_stream(stream);
    int64_t* n_runs = ws;
    int64_t* n_groups = ws + 1;
    int64_t* total = ws + 2;
    int64_t* scan_ws = ws + 3;
    ETM_CUDA(cudaMemsetAsync(ws, 0, 3 * sizeof(int64_t), s));
    ETM_CUDA(cudaMemsetAsync(counters, 0, 2 * sizeof(int64_t), s));
    if (n == 0) {
        ETM_CUDA(cudaMemsetAsync(cand_off, 0, sizeof(int64_t), s));
        return ETM_OK;
    }
    // Run starts (into cand_off as scratch), then runs of >= 2 members, then candidate offsets.
    int st = scan_apply(n, RunStart{rows, n, width}, WriteAt{cand_off}, scan_ws, ws_words - 3, n_runs, s);
    if (st) return st;
    RunIsGroup runs{cand_off, n_runs, n};
    st = scan_apply(n, runs, EmitGroup{runs, grp_first, grp_size}, scan_ws, ws_words - 3, n_groups, s);
    if (st) return st;
    st = scan_apply(n, GroupPairs{grp_size, n_groups}, WriteOffset{cand_off}, scan_ws, ws_words - 3, total, s);
    if (st) return st;
    finish_groups_kernel<<<1, 1, 0, s>>>(cand_off, counters, n_groups, total);
    ETM_LAUNCHED("finish_groups");
    return ETM_OK;
}

extern "C" int etm_classify(const int32_t* rows, int32_t width, int64_t n_rows, const int32_t* counts,
                            const uint8_t* free_flags, const int64_t* grp_first, const int32_t* grp_size,
                            const int64_t* cand_off, int64_t g0, int64_t g1, int32_t mode, uint8_t* out_cls,
                            int32_t* out_counts, void* stream) {
    ETM_REQUIRE(width >= 1 && width < MAXK, ETM_EINVAL, "etm_classify: width %d out of range", width);
    ETM_REQUIRE(g0 >= 0 && g1 >= g0, ETM_EINVAL, "etm_classify: bad group range");
    if (g1 == g0) return ETM_OK;
    classify_kernel<<<max(1, sm_count()) * 8, 256, 0, as_stream(stream)>>>(
        rows, width, n_rows, counts, free_flags, grp_first, grp_size, cand_off, g0, g1, mode & ~ETM_SUBSET_BOUNDS,
        out_cls, out_counts, 0, nullptr, DeepLevels{nullptr, 0, nullptr, nullptr, 0, nullptr, 0});
    ETM_LAUNCHED("classify");
    return ETM_OK;
}

extern "C" int etm_classify_sel(const int32_t* rows, int32_t width, int64_t n_rows, const int32_t* counts,
                                const uint8_t* free_flags, const int64_t* grp_first, const int32_t* grp_size,
                                const int64_t* cand_off, int64_t g0, int64_t g1, int32_t mode, int32_t min_count,
                                const int32_t* deep2_rows, int64_t deep2_n, const int32_t* deep2_counts,
                                const int32_t* deep3_rows, int64_t deep3_n, const int32_t* deep3_counts,
                                int64_t n_transactions, uint8_t* out_cls, int32_t* out_counts, uint32_t* surv_bits,
                                void* stream) {
    ETM_REQUIRE(width >= 1 && width < MAXK, ETM_EINVAL, "etm_classify_sel: width %d out of range", width);
    ETM_REQUIRE(g0 >= 0 && g1 >= g0, ETM_EINVAL, "etm_classify_sel: bad group range");
    ETM_REQUIRE(surv_bits != nullptr, ETM_EINVAL, "etm_classify_sel: surv_bits is required");
    ETM_REQUIRE(!(mode & ETM_SUBSET_BOUNDS) || (deep2_rows != nullptr && (width + 1 <= 3 || deep3_rows != nullptr)),
                ETM_EINVAL, "etm_classify_sel: the deduction bounds need levels k-2 and (k > 3) k-3");
    if (g1 == g0) return ETM_OK;
    const DeepLevels deep{(mode & ETM_SUBSET_BOUNDS) ? deep2_rows : nullptr, deep2_n, deep2_counts, deep3_rows, deep3_n,
                          deep3_counts, n_transactions};
    classify_kernel<<<max(1, sm_count()) * 8, 256, 0, as_stream(stream)>>>(
        rows, width, n_rows, counts, free_flags, grp_first, grp_size, cand_off, g0, g1, mode, out_cls, out_counts,
        min_count, surv_bits, deep);
    ETM_LAUNCHED("classify");
    return ETM_OK;
}

extern "C" int etm_threshold_bits(const int32_t* counts, const uint8_t* cls, int64_t n_cands, int32_t min_count,
                                  uint32_t* surv_bits, void* stream) {
    ETM_REQUIRE(n_cands >= 0, ETM_EINVAL, "etm_threshold_bits: negative n_cands");
    if (n_cands == 0) return ETM_OK;
    threshold_bits_kernel<<<grid_for((n_cands + 31) / 32, 256), 256, 0, as_stream(stream)>>>(counts, cls, n_cands,
                                                                                            min_count, surv_bits);
    ETM_LAUNCHED("threshold_bits");
    return ETM_OK;
}

extern "C" int etm_level_compact_bits(const uint32_t* surv_bits, const int32_t* counts, int64_t n_cands,
                                      const int32_t* rows, int32_t width, const int64_t* grp_first,
                                      const int32_t* grp_size, const int64_t* cand_off, int64_t g0, int64_t g1,
                                      int32_t* out_rows, int32_t* out_counts, int64_t cap, int64_t* acc, int64_t* ws,
                                      int64_t ws_words, void* stream) {
    ETM_REQUIRE(width >= 1 && width + 1 < MAXK, ETM_EINVAL, "etm_level_compact_bits: width %d out of range", width);
    if (n_cands <= 0) return ETM_OK;
    WordSurvivors words{surv_bits, n_cands};
    EmitSurvivor emit{counts, rows, width, grp_first, grp_size, cand_off, g0, g1, out_rows, out_counts, cap};
    return scan_apply((n_cands + 31) / 32, words, EmitWordSurvivors{words, emit}, ws, ws_words, acc, as_stream(stream));
}

extern "C" int etm_level_compact(const int32_t* counts, const uint8_t* cls, int64_t n_cands, const int32_t* rows,
                                 int32_t width, const int64_t* grp_first, const int32_t* grp_size,
                                 const int64_t* cand_off, int64_t g0, int64_t g1, int32_t min_count,
                                 int32_t* out_rows, int32_t* out_counts, int64_t cap, int64_t* acc, int64_t* ws,
                                 int64_t ws_words, void* stream) {
    ETM_REQUIRE(width >= 1 && width + 1 < MAXK, ETM_EINVAL, "etm_level_compact: width %d out of range", width);
    if (n_cands <= 0) return ETM_OK;
    Survives val{counts, cls, n_cands, min_count};
    EmitSurvivor act{counts, rows, width, grp_first, grp_size, cand_off, g0, g1, out_rows, out_counts, cap};
    return scan_apply(n_cands, val, act, ws, ws_words, acc, as_stream(stream));
}

// ---- survivor compaction without caller-provided scratch ------------------------------
//
// etm_level_compact needs a small int64 workspace for its scan (one partial sum
// per 4096 candidates). Some callers cannot hand one over: a serving process
// that reserved all of its device memory up front and forbids allocations
// once requests flow, or a host runtime that reaches this library through a
// plain C call and owns no allocator of its own. For them the workspace lives
// in this file, as one fixed device array per GPU.

namespace {

// Largest chunk the static workspace serves: 65,536 scan blocks of 4096
// candidates, i.e. 268,435,456 candidates (the array is 512 KB + 16 bytes and
// stays resident on every GPU that loads the library, until the process exits).
constexpr int64_t STATIC_SCAN_BLOCKS = 65536;
constexpr int64_t STATIC_SCAN_WORDS = STATIC_SCAN_BLOCKS + 2;
constexpr int64_t STATIC_MAX_CANDS = STATIC_SCAN_BLOCKS * SCAN_TILE;
constexpr int MAX_DEVICES = 64;

static __device__ __align__(256) int64_t g_static_scan_ws[STATIC_SCAN_WORDS];

// Device address of g_static_scan_ws, looked up once per device (with that device current).
// On the host the symbol name is only a stand-in, never a device address.
int64_t* static_scan_ws(int* status) {
    static std::mutex lock;
    static int64_t* addr[MAX_DEVICES] = {nullptr};
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess || dev < 0 || dev >= MAX_DEVICES) {
        set_error("etm_level_compact_static: no usable current device (%s)",
                  e != cudaSuccess ? cudaGetErrorString(e) : "device index out of range");
        *status = ETM_ECUDA;
        return nullptr;
    }
    std::lock_guard<std::mutex> guard(lock);
    if (addr[dev] == nullptr) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_static_scan_ws);
        if (e != cudaSuccess || p == nullptr) {
            set_error("etm_level_compact_static: cudaGetSymbolAddress failed on device %d: %s", dev,
                      cudaGetErrorString(e));
            *status = ETM_ECUDA;
            return nullptr;
        }
        addr[dev] = static_cast<int64_t*>(p);
    }
    *status = ETM_OK;
    return addr[dev];
}

}  // namespace

extern "C" int etm_level_compact_static(const int32_t* counts, const uint8_t* cls, int64_t n_cands,
                                        const int32_t* rows, int32_t width, const int64_t* grp_first,
                                        const int32_t* grp_size, const int64_t* cand_off, int64_t g0, int64_t g1,
                                        int32_t min_count, int32_t* out_rows, int32_t* out_counts, int64_t cap,
                                        int64_t* acc, void* stream) {
    ETM_REQUIRE(width >= 1 && width + 1 < MAXK, ETM_EINVAL, "etm_level_compact_static: width %d out of range", width);
    ETM_REQUIRE(n_cands <= STATIC_MAX_CANDS, ETM_ENOSPACE,
                "etm_level_compact_static: %lld candidates exceed the static workspace's limit of %lld per call; "
                "split the chunk or use etm_level_compact with a workspace",
                (long long)n_cands, (long long)STATIC_MAX_CANDS);
    int status = ETM_OK;
    int64_t* ws = static_scan_ws(&status);
    if (status != ETM_OK) return status;
    if (n_cands <= 0) return ETM_OK;
    // Every call rewrites the partial sums it reads (phase 1 writes each block's sum,
    // phase 2 the offsets), so nothing left by an earlier call needs clearing.
    Survives val{counts, cls, n_cands, min_count};
    EmitSurvivor act{counts, rows, width, grp_first, grp_size, cand_off, g0, g1, out_rows, out_counts, cap};
    return scan_apply(n_cands, val, act, ws, STATIC_SCAN_WORDS, acc, as_stream(stream));
}

extern "C" int etm_level_subsets(const int32_t* new_rows, const int32_t* new_counts, int64_t n_new, int32_t width,
                                 const int32_t* prev_rows, const int32_t* prev_counts, int64_t n_prev,
                                 uint8_t* out_free, uint8_t* out_present, void* stream) {
    ETM_REQUIRE(width >= 1 && width + 1 < MAXK, ETM_EINVAL, "etm_level_subsets: width %d out of range", width);
    if (n_new <= 0) return ETM_OK;
    subsets_kernel<<<grid_for(n_new, 256), 256, 0, as_stream(stream)>>>(new_rows, new_counts, n_new, width, prev_rows,
                                                                        prev_counts, n_prev, out_free, out_present);
    ETM_LAUNCHED("level_subsets");
    return ETM_OK;
}

extern "C" int etm_select_rows(const int32_t* rows, const int32_t* counts, const uint8_t* keep_a,
                               const uint8_t* keep_b, int64_t n, int32_t width, int32_t* out_rows, int32_t* out_counts,
                               uint8_t* out_flag_src, uint8_t* out_flag, int64_t cap, int64_t* acc, int64_t* ws,
                               int64_t ws_words, void* stream) {
    ETM_REQUIRE(width >= 1 && width <= MAXK, ETM_EINVAL, "etm_select_rows: width %d out of range", width);
    if (n <= 0) return ETM_OK;
    return scan_apply(n, Kept{keep_a, keep_b, n},
                      CopyRow{rows, counts, out_flag_src, width, out_rows, out_counts, out_flag, cap}, ws, ws_words,
                      acc, as_stream(stream));
}
