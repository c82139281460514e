/*
 * libetm_gb300 — C ABI of the GB300 exact Apriori counting engine.
 *
 * Drop-in boundary for ET-Miner's GPU counting path (the level driver
 * `_apriori_row_split_multi_gpu`, gpu/row_split.py:229-1185, reached from
 * `apriori(..., use_gpu=True, bitvecs=...)`, core/apriori.py:477-548).
 *
 * Every entry point takes device pointers, plain sizes and a CUDA stream
 * (cudaStream_t passed as void*, NULL = legacy default stream), enqueues its
 * work on that stream and returns a status (ETM_OK = 0). On failure
 * etm_last_error() describes it. No entry point allocates device memory
 * except where it says so: scratch is passed in as `ws` (int64 words) with its
 * size, and each function states how many words it needs.
 *
 * Data conventions (core/apriori.py:409-413, csr_to_bitvec.cu:27-35):
 *   bitvectors   uint64 [n_cols][ld]; bit r%64 of word r/64 of column c is set
 *                when transaction r holds column c; bits past N are zero.
 *   level rows   int32 [n][width], column indices ascending within a row,
 *                rows in strictly ascending lexicographic order.
 *   counts       int32 (N < 2^31, gpu/row_split.py:358-362).
 *   candidates   of a prefix group with m members (rows first..first+m-1
 *                sharing their first width-1 columns): the C(m,2) pairs
 *                (i < j), item list = prefix + s_i + s_j, in lexicographic
 *                (i-major) order; a level's candidates are the groups' in order.
 */
#ifndef ETM_H
#define ETM_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ETM_OK 0
#define ETM_EINVAL 1   /* bad argument: sizes, alignment, widths */
#define ETM_ECUDA 2    /* a CUDA call or launch failed */
#define ETM_ENOSPACE 3 /* workspace or output capacity too small */
#define ETM_ETIMEOUT 4 /* a bounded device wait gave up; the kernel cleaned up, the device stays usable */
#define ETM_EUNSAFE 5  /* a bounded wait gave up and so did its cleanup wait: copies may still be landing;
                          stop using the device (tear the process down) */

/* Candidate classes written by etm_classify (gpu/kernels/_src/_subset_index.cu:27-33). */
#define ETM_CAND_COUNT 0
#define ETM_CAND_SKIP 1
#define ETM_CAND_INFER 2

/* Mode bits of etm_classify (gpu/kernels/subset_index.py SUBSET_PRUNE / SUBSET_INFER). */
#define ETM_SUBSET_PRUNE 1
#define ETM_SUBSET_INFER 2
/* With ETM_SUBSET_INFER, in etm_classify_sel: settle the candidates of at most 24 items that inference
 * leaves by the deduction bounds of depth <= 3 (SUBSET_BOUNDS, gpu/kernels/_src/_subset_index.cu:93-136):
 * SKIP when the upper bound is below min_count, INFER when the bounds meet. */
#define ETM_SUBSET_BOUNDS 4

/* Count methods of etm_pair_counts / etm_count_tiles. */
#define ETM_METHOD_POPCOUNT 0 /* AND + popcount on CUDA cores */
#define ETM_METHOD_TENSOR 1   /* 0/1 Gram on tcgen05 tensor cores, f32 accumulation in TMEM, exact */

/* Element codes of etm_count_tiles_tc: 1 = e4m3 (kind::f8f6f4), 2 = f16 (kind::f16), ETM_TC_MXF4 = packed
 * e2m1 under kind::mxf4 with unit block scales. Blocks hold etm_gram_block_members(elem) members: 256 for
 * e4m3 and f16, 240 for e2m1. */
#define ETM_TC_MXF4 4
/* Accepted in elem for compatibility and ignored: every element code runs the block-pair kernel. */
#define ETM_TC_WIDE 16
/* Added to elem: the member rows are in the blocked layout etm_project_blocked writes, with blocks of
 * etm_gram_block_members(elem) members (cbase of each work entry at a block-aligned member 0). */
#define ETM_TC_BLOCKED 32

/* Rows of one projection segment: 1024 bitvector words (65,536 transactions). */
#define ETM_PROJ_SEG_WORDS 1024
/* Words of one occupancy tile (2,048 transactions); 64 tiles per occupancy word. */
#define ETM_OCC_TILE_WORDS 32
/* Widest id span etm_item_codes codes through its presence bitmap (8 MB of bits). */
#define ETM_CODE_SPAN_MAX (1LL << 26)

int etm_version(void);
/* Message of the last failing call on this thread (empty if none). */
const char* etm_last_error(void);
/* SM count of the current device. */
int etm_device_sm_count(void);

/*
 * CSR -> column bitvectors. Replaces csr_to_bitvec and ids_to_bitvec
 * (gpu/kernels/_src/csr_to_bitvec.cu:9-73) and their drivers
 * (gpu/csr_bitvec.py:63-155, gpu/input_layer.py:434-466).
 * row_ptr int64 [n_rows+1], non-decreasing; ids int32 [nnz]; lut int32
 * [lut_size] maps an id to its column or -1 (NULL: ids are columns). Ids
 * outside the lut, columns outside [0, n_cols) and entries outside [0, nnz)
 * are ignored. out_bv [n_cols][ld] is zeroed here, then filled.
 * ld >= ceil(n_rows/64).
 */
int etm_build_bitvecs(const int64_t* row_ptr, const int32_t* ids, int64_t nnz, const int32_t* lut,
                      int64_t lut_size, int64_t n_rows, int64_t n_cols, int64_t ld, uint64_t* out_bv, void* stream);

/*
 * K=1 support: popcount of each column over words [0, n_words). Replaces
 * column_popcounts (gpu/kernels/loader.py:241-257) and the K=1 step of
 * gpu/row_split.py:789-834. out_counts int64 [n_cols].
 */
int etm_popcount_cols(const uint64_t* bv, int64_t n_cols, int64_t n_words, int64_t ld, int64_t* out_counts,
                      void* stream);

/*
 * Copy columns cols[0..n_f) of bv into out [n_f][out_ld] (words past n_words
 * zeroed): the engine's private, padded copy of the frequent columns; the
 * caller's array is only read (core/apriori.py:409-413). out_ld % 32 == 0.
 */
int etm_gather_cols(const uint64_t* bv, int64_t ld, const int32_t* cols, int32_t n_f, int64_t n_words,
                    uint64_t* out, int64_t out_ld, void* stream);

/*
 * The lex row order of the device input layer (gpu/input_layer.py:408-430,
 * the row_order_keys kernel of gpu/kernels/_src/csr_to_bitvec.cu:75-104).
 *   etm_row_order_keys  per row of a CSR of columns (row_ptr int64 [n_rows+1],
 *                      cols int32): a row holding the column of rank r
 *                      (rank_of_col int32 [n_cols], by descending support) sets
 *                      bit 63 - r of key_hi for r < 64 and bit 127 - r of key_lo
 *                      for 64 <= r < 128; both int64 [n_rows] are stored with
 *                      the top bit flipped, so an ascending signed sort by
 *                      (key_hi, key_lo) is the unsigned order. Columns outside
 *                      [0, n_cols) are ignored.
 *   etm_permute_rows   output row p = input row order[p] (order int64 [n_rows],
 *                      a permutation): its entries go to new_cols from
 *                      new_row_ptr[p] (the caller's exclusive prefix of the
 *                      permuted lengths). A row whose source index or either
 *                      range falls outside [0, n_rows) / [0, nnz) is skipped and
 *                      sets *status (int32 device word, zeroed here) to 1.
 *   etm_tile_occupancy per column of bv, one bit per tile of ETM_OCC_TILE_WORDS
 *                      words (gpu/kernels/occupancy.py:37-58): bit b of
 *                      occ[c * occ_ld + w] is set when tile 64 w + b (words
 *                      below n_words) holds a set bit. occ_ld >= ceil(ceil(
 *                      n_words / 32) / 64); any ld >= n_words (16-byte loads
 *                      when bv is 16-byte aligned and ld even).
 */
int etm_row_order_keys(const int64_t* row_ptr, const int32_t* cols, int64_t n_rows, const int32_t* rank_of_col,
                       int64_t n_cols, int64_t* key_hi, int64_t* key_lo, void* stream);
int etm_permute_rows(const int64_t* row_ptr, const int32_t* cols, int64_t nnz, const int64_t* order, int64_t n_rows,
                     const int64_t* new_row_ptr, int32_t* new_cols, int32_t* status, void* stream);
int etm_tile_occupancy(const uint64_t* bv, int64_t n_cols, int64_t n_words, int64_t ld, uint64_t* occ,
                       int64_t occ_ld, void* stream);

/*
 * Item coding of a transaction CSR without sorting (the device input layer's
 * K=1 and id lookup, gpu/input_layer.py:396-466, with exact supports).
 *   etm_item_codes     ids int64 [nnz] in rows row_ptr int64 [n_rows+1]; the
 *                      ids lie in [lo, lo + span), span <= ETM_CODE_SPAN_MAX.
 *                      bitmap uint32 [ceil(span/32)] gets bit id - lo of every
 *                      id present; word_rank int64 [ceil(span/32) + 1] the set
 *                      bits before each word (its last entry: the distinct
 *                      ids); codes int32 [nnz] each entry's rank among the
 *                      distinct ids (ascending id order). status int32 [2]
 *                      (zeroed here): [0] = 1 when an id lies outside the span
 *                      (its code is -1), [1] = 1 when a row's codes do not
 *                      strictly ascend (unsorted, or an id repeated).
 *   etm_code_histogram counts int64 [n_bins] = occurrences of each code (codes
 *                      outside [0, n_bins) ignored); with canonical rows, the
 *                      rows holding each id.
 *   etm_bitmap_values  out int64 [distinct ids] = the ids present, ascending.
 *   etm_kept_lengths   out_lengths int64 [n_rows] = each row's entries whose
 *                      code maps to a column (lut int32 [lut_size], -1 none).
 */
int etm_item_codes(const int64_t* row_ptr, const int64_t* ids, int64_t nnz, int64_t n_rows, int64_t lo,
                   int64_t span, uint32_t* bitmap, int64_t* word_rank, int32_t* codes, int32_t* status,
                   void* stream);
int etm_code_histogram(const int32_t* codes, int64_t nnz, int64_t n_bins, int64_t* counts, void* stream);
int etm_bitmap_values(const uint32_t* bitmap, int64_t span, const int64_t* word_rank, int64_t lo, int64_t* out,
                      void* stream);
int etm_kept_lengths(const int64_t* row_ptr, const int32_t* codes, int64_t n_rows, const int32_t* lut,
                     int64_t lut_size, int64_t* out_lengths, void* stream);

/*
 * Deterministic Bernoulli bitvectors (workload generator; no reference
 * counterpart): bit r of item i set when hash(seed, i, r) < thresholds[i].
 */
int etm_synth_bernoulli(const uint64_t* thresholds, int32_t n_items, int64_t n_rows, uint64_t seed,
                        uint64_t* out_bv, int64_t ld, void* stream);

/*
 * Bitvectors of a planted-pattern workload (the deep sparse configuration),
 * defined by the same counter hash h(seed, stream, row) as
 * etm_synth_bernoulli so a host restatement reproduces every bit. Row r: its
 * length is 1 + #{i < n_len : h(seed, 1, r) >= len_thr[i]}; it draws per_row
 * patterns, pattern p being the first j with h(seed, 2 + p, r) < pat_thr[j]
 * (the last if none); item q of that pattern is kept when
 * h(seed, 64 + 16 p + q, r) < keep_thr and not yet in the row, until the row
 * is full; then noise items h(seed, 4096 + t, r) % n_items, t = 0, 1, ...,
 * not yet in the row, fill it. Patterns: pat_ptr int64 [n_pat + 1] into
 * pat_items int32 (at most 16 items each). out_bv uint64 [n_items][ld]
 * (zeroed here). Test and benchmark input; no counterpart in the reference
 * (its generator is synthetic.py:160-180, host only).
 */
int etm_synth_patterns(const uint64_t* len_thr, int32_t n_len, const uint64_t* pat_thr, int32_t n_pat,
                       const int64_t* pat_ptr, const int32_t* pat_items, int32_t per_row, uint64_t keep_thr,
                       int32_t n_items, int64_t n_rows, uint64_t seed, uint64_t* out_bv, int64_t ld, void* stream);

/*
 * Prefix groups of a level. Replaces build_k3plus_groups_from_flat
 * (gpu/kernels/k3plus.py:243-301; rust_ext/src/core/groups.rs:59-248) and the
 * prefix-run step of generate_candidates (core/cpu_miner.py:466-475).
 * rows int32 [n][width] (width >= 1; width 1 = one group of every row).
 * Outputs groups with >= 2 members: grp_first int64 [n], grp_size int32 [n],
 * cand_off int64 [n+1] (exclusive prefix of C(m,2); cand_off[G] = total),
 * counters int64 [2] = {G, total candidates}. ws: 2 * (n/4096 + 3) words.
 */
int etm_level_groups(const int32_t* rows, int64_t n, int32_t width, int64_t* grp_first, int32_t* grp_size,
                     int64_t* cand_off, int64_t* counters, int64_t* ws, int64_t ws_words, void* stream);

/*
 * Subset test and count inference of the candidates of groups [g0, g1).
 * Replaces _classify_candidate (gpu/kernels/_src/_subset_index.cu:139-178) and
 * the CPU route's prune/infer steps (core/cpu_miner.py:490-494, 1119-1124).
 * rows/counts/free_flags: the generating level (n_rows x width). mode:
 * ETM_SUBSET_PRUNE (a missing prefix-dropping subset -> SKIP) | ETM_SUBSET_INFER
 * (a non-free subset -> INFER with the minimum subset count, written to
 * out_counts). out_cls uint8 and out_counts int32 are indexed by candidate
 * minus cand_off[g0].
 */
int etm_classify(const int32_t* rows, int32_t width, int64_t n_rows, const int32_t* counts,
                 const uint8_t* free_flags, const int64_t* grp_first, const int32_t* grp_size,
                 const int64_t* cand_off, int64_t g0, int64_t g1, int32_t mode, uint8_t* out_cls,
                 int32_t* out_counts, void* stream);

/*
 * Count the candidates of the listed groups by tile-pairs of 64 x 64
 * suffixes (AND of the prefix columns per word, AND+popcount per pair).
 * Replaces count_shared_tiled_dense (gpu/kernels/_src/shared_tiled.cu:96-246),
 * count_group_pairs (group_pairs.cu:32-217) and, for K=2,
 * count_pairs_k2_dense (pairs_k2_dense.cu:3-45).
 * fbv [n_f][ld] (ld % 32 == 0, zero past n_words). work_groups int64 [n_work]
 * group ids; work_off int64 [n_work+1] exclusive prefix of each listed
 * group's tile-pairs T(T+1)/2, T = ceil(m/64). Counts go to
 * out_counts[cand_off[g] - chunk_base + pair]. cls (nullable): candidates
 * whose class is not ETM_CAND_COUNT are not written; tile-pairs without any
 * are skipped. method: ETM_METHOD_POPCOUNT or ETM_METHOD_TENSOR.
 */
int etm_count_tiles(const uint64_t* fbv, int64_t ld, int64_t n_words, const int32_t* rows, int32_t width,
                    const int64_t* grp_first, const int32_t* grp_size, const int64_t* cand_off,
                    const int64_t* work_groups, const int64_t* work_off, int64_t n_work, int64_t chunk_base,
                    const uint8_t* cls, int32_t method, int32_t* out_counts, void* stream);

/*
 * Count candidates one warp each (AND of all k columns, popcount): the
 * layout for small prefix groups. Replaces count_k3plus_dense
 * (gpu/kernels/_src/k3plus_dense.cu:3-106). work_off int64 [n_work+1] is the
 * exclusive prefix of C(m,2) over the listed groups.
 */
int etm_count_cands(const uint64_t* fbv, int64_t ld, int64_t n_words, const int32_t* rows, int32_t width,
                    const int64_t* grp_first, const int32_t* grp_size, const int64_t* cand_off,
                    const int64_t* work_groups, const int64_t* work_off, int64_t n_work, int64_t chunk_base,
                    const uint8_t* cls, int32_t* out_counts, void* stream);

/*
 * Row-wise K=2: every row adds 1 to each pair of its generator columns.
 * Replaces count_pairs_k2_rows (gpu/kernels/_src/pairs_k2_rows.cu:54; dispatch
 * gpu/row_split_chunks.py:124-142). row_ptr int64 [n_rows+1] / cols int32
 * [nnz]: the transactions' columns, ascending per row; lut int32 [lut_size]
 * maps a column to its generator index or -1 (NULL: columns are generator
 * indices). out_counts int32 [C(n_gen,2)] is zeroed here, then holds every
 * pair's count at its lexicographic slot (the K=2 candidate index).
 */
int etm_pair_counts_rows(const int64_t* row_ptr, const int32_t* cols, int64_t nnz, const int32_t* lut,
                         int64_t lut_size, int64_t n_rows, int64_t n_gen, int32_t* out_counts, void* stream);

/*
 * Row-wise K=3 counts (count_k3_rows, gpu/kernels/_src/k3_rows.cu:50-140; chosen by the reference when
 * r3 = sum over rows of C(len, 2) / (K=3 candidates x words) < 2.5e-4 and every candidate fits one chunk,
 * gpu/row_split_chunks.py:145-159). The candidates are those of the prefix groups of a width-2 generating
 * level: gen_rows int32 [n][2] (generator indices, lexsorted), group g = rows [grp_first[g],
 * grp_first[g] + grp_size[g]) sharing item gen_rows[grp_first[g]][0], candidate (u, v_i, v_j) at
 * cand_off[g] + tri_index(i, j, grp_size[g]); grp_of int32 [n_gen1] maps a generator to the group it
 * prefixes or -1. out_counts int32 [n_cands] holds candidates [chunk_base, chunk_base + n_cands): those
 * whose class is ETM_CAND_COUNT (all when cls is NULL) are zeroed, then each row adds 1 to every one of
 * them whose three items it holds; the others are left as they were. row_ptr / cols / lut as for
 * etm_pair_counts_rows.
 */
int etm_triple_counts_rows(const int64_t* row_ptr, const int32_t* cols, int64_t nnz, const int32_t* lut,
                           int64_t lut_size, int64_t n_rows, const int32_t* gen_rows, const int32_t* grp_of,
                           int64_t n_gen1, const int64_t* grp_first, const int32_t* grp_size,
                           const int64_t* cand_off, int64_t chunk_base, int64_t n_cands, const uint8_t* cls,
                           int32_t* out_counts, void* stream);

/*
 * Prefix projection (the reference's projection counting of wide groups,
 * core/cpu_miner.py:720-791, on the device). For the listed groups (width >= 2):
 *   etm_prefix_counts  out_counts int64 [n_work] = rows holding the group's prefix
 *                      (popcount of the AND of its width-1 prefix columns);
 *   etm_prefix_rows    out_rows int32 = those rows, ascending, group wi at
 *                      [row_off[wi], row_off[wi+1]) (row_off: exclusive prefix of
 *                      the counts);
 *   etm_prefix_segments  the prefix AND's popcount per segment of
 *                      ETM_PROJ_SEG_WORDS words: seg_off int64 [n_work][n_seg+1]
 *                      (n_seg = ceil(n_words / ETM_PROJ_SEG_WORDS)) = the word
 *                      offset of each segment's piece of a projected row, each
 *                      piece ceil(count / 64) words rounded up to a multiple of
 *                      4 (whole 32-byte chunks); out_words[wi] = the total;
 *   etm_project        member i of group wi -> cbuf[cbase[wi] + i*cld[wi] ...]:
 *                      per segment, its column's bits at the segment's prefix
 *                      rows, 64 per word, the piece zero-padded to whole chunks
 *                      at seg_off; zero from out_words[wi] up to cld[wi] words
 *                      (cld % 32 == 0, cbase even, ld even, fbv 16-byte aligned).
 *                      Padding rows are zero in every member, so pair counts
 *                      over the projected words equal those over the prefix rows.
 *                      work_counter (one int64 of device memory, or NULL): the
 *                      CTAs claim (segment, group) units from it dynamically; it
 *                      is zeroed on the stream first (one per concurrent call).
 *   etm_count_tiles_proj  etm_count_tiles over the projected words
 *                      (cwords[wi] words per member; no prefix AND).
 * occ (etm_prefix_counts, etm_prefix_segments; NULL for none): the tile
 * occupancy of fbv (etm_tile_occupancy over n_words, occ_ld words per column);
 * a tile where a prefix column holds no row is not read, its prefix AND is 0.
 */
int etm_prefix_counts(const uint64_t* fbv, int64_t ld, int64_t n_words, const int32_t* rows, int32_t width,
                      const int64_t* grp_first, const int64_t* work_groups, int64_t n_work, int64_t* out_counts,
                      const uint64_t* occ, int64_t occ_ld, void* stream);
int etm_prefix_rows(const uint64_t* fbv, int64_t ld, int64_t n_words, const int32_t* rows, int32_t width,
                    const int64_t* grp_first, const int64_t* work_groups, int64_t n_work, const int64_t* row_off,
                    int32_t* out_rows, void* stream);
int etm_prefix_segments(const uint64_t* fbv, int64_t ld, int64_t n_words, const int32_t* rows, int32_t width,
                        const int64_t* grp_first, const int64_t* work_groups, int64_t n_work, int64_t* seg_off,
                        int64_t* out_words, const uint64_t* occ, int64_t occ_ld, void* stream);
int etm_project(const uint64_t* fbv, int64_t ld, int64_t n_words, const int32_t* rows, int32_t width,
                const int64_t* grp_first, const int32_t* grp_size, const int64_t* work_groups, int64_t n_work,
                const int64_t* seg_off, const int64_t* cbase, const int64_t* cld, uint64_t* cbuf,
                int64_t* work_counter, void* stream);
/*
 * etm_project writing the blocked layout: the members of each work entry in
 * blocks of blk (1..4096), each block stored 4-word chunk by chunk and each
 * chunk as two 2-word halves, so word w of member j sits at cbase +
 * (j / blk) * cld * blk + (w / 4) * 4 * blk + ((w / 2) % 2) * 2 * blk +
 * (j % blk) * 2 + w % 2. The tensor-core Gram then copies each stage's words
 * of a block as one contiguous run, and its producers (one per member of a
 * block) read consecutive members' halves from adjacent 16-byte slots
 * (elem | ETM_TC_BLOCKED, blk = etm_gram_block_members(elem)). Each work
 * entry needs ceil(m / blk) * blk * cld words (rows past m are never read).
 * New in this engine, like the projection itself.
 */
int etm_project_blocked(const uint64_t* fbv, int64_t ld, int64_t n_words, const int32_t* rows, int32_t width,
                        const int64_t* grp_first, const int32_t* grp_size, const int64_t* work_groups, int64_t n_work,
                        const int64_t* seg_off, const int64_t* cbase, const int64_t* cld, int64_t blk, uint64_t* cbuf,
                        int64_t* work_counter, void* stream);

/*
 * Row-major copy of the generating columns for etm_project_rows: xt is
 * uint32 [64 n_words][ldr] (16-byte aligned, ldr a multiple of 4 with
 * 32 ldr >= n_cols), and bit k of xt[r][c] is bit r of column 32 c + k of fbv
 * (zero past n_cols). One pass over the columns; no counterpart in the
 * reference, which never transposes its bitvectors.
 */
int etm_rows_transpose(const uint64_t* fbv, int64_t ld, int64_t n_words, int64_t n_cols, uint32_t* xt, int64_t ldr,
                       void* stream);

/*
 * The projection of etm_project / etm_project_blocked (blk = 0: row-major
 * member rows, blk > 0: the blocked layout; the same words, the same
 * seg_off / cbase / cld / cbuf contract) computed from the row-major copy xt
 * of etm_rows_transpose: per (segment, work entry) unit the prefix rows are
 * listed, their words loaded 128 rows x 128 columns at a time and turned into
 * member words by 32 x 32 bit transposes (warp shuffles). It reads only the
 * prefix rows' words where the column form reads every member's whole
 * segment, and needs no bulk copies or device waits. cbase and cld entries
 * must be even (16-byte aligned member rows) and every member column must lie
 * below 32 ldr; a unit that breaks either is skipped and etm_device_status
 * reports ETM_EINVAL. Units go to CTAs round-robin (no work counter: with
 * units claimed from a counter, a launch overlapping another stream's
 * kernels was measured to leave a few units unwritten in about one mine in
 * eight; the cause is not known). The projection of gram_pairs' input
 * (core/cpu_miner.py:641-692) in another form, like etm_project.
 */
int etm_project_rows(const uint64_t* fbv, int64_t ld, int64_t n_words, const uint32_t* xt, int64_t ldr,
                     const int32_t* rows, int32_t width, const int64_t* grp_first, const int32_t* grp_size,
                     const int64_t* work_groups, int64_t n_work, const int64_t* seg_off, const int64_t* cbase,
                     const int64_t* cld, int64_t blk, uint64_t* cbuf, void* stream);

int etm_count_tiles_proj(const uint64_t* cbuf, const int64_t* cbase, const int64_t* cwords, const int64_t* cld,
                         const int32_t* grp_size, const int64_t* cand_off, const int64_t* work_groups,
                         const int64_t* work_off, int64_t n_work, int64_t chunk_base, const uint8_t* cls,
                         int32_t method, int32_t* out_counts, void* stream);

/*
 * etm_count_tiles_proj on the tcgen05 tensor cores: the pair counts of each
 * listed group are the Gram matrix of its 0/1 member words. One persistent
 * kernel takes block pairs (ua <= ub) of T = etm_gram_block_members(elem)
 * members, stages the bits expanded to e4m3 (elem 1), f16 (elem 2) or packed
 * e2m1 (ETM_TC_MXF4) in shared memory and accumulates in f32 in TMEM. Exact
 * while every group has at most 2^24 rows (cwords <= 262144): the caller sends
 * larger groups to the popcount kernels. work_off counts block pairs,
 * C(nb + 1, 2) per group with nb = ceil(m / T); n_tiles = work_off[n_work]
 * (sizes the grid). work_counter (one int64 of device memory, or NULL) lets
 * the CTAs claim block pairs dynamically (zeroed on the stream before the
 * launch; concurrent calls need separate counters). New in this engine (the
 * reference counts on CUDA cores only).
 */
int etm_count_tiles_tc(const uint64_t* cbuf, const int64_t* cbase, const int64_t* cwords, const int64_t* cld,
                       const int32_t* grp_size, const int64_t* cand_off, const int64_t* work_groups,
                       const int64_t* work_off, int64_t n_work, int64_t n_tiles, int64_t chunk_base,
                       const uint8_t* cls, int32_t elem, int32_t* out_counts, int64_t* work_counter, void* stream);

/*
 * etm_count_tiles_tc with the survivor threshold fused into its epilogue, the
 * form of count_shared_tiled_fused (gpu/kernels/_src/shared_tiled.cu:246-280):
 * of the candidates it counts, only those reaching min_count get their count
 * written (out_counts[t]) and their bit t set in surv_bits (uint32 words,
 * bit t % 32 of word t / 32, chunk-relative t; the caller zeroes it first).
 * The other slots of out_counts are left untouched.
 */
int etm_count_tiles_tc_sel(const uint64_t* cbuf, const int64_t* cbase, const int64_t* cwords, const int64_t* cld,
                           const int32_t* grp_size, const int64_t* cand_off, const int64_t* work_groups,
                           const int64_t* work_off, int64_t n_work, int64_t n_tiles, int64_t chunk_base,
                           const uint8_t* cls, int32_t elem, int32_t min_count, int32_t* out_counts,
                           uint32_t* surv_bits, int64_t* work_counter, void* stream);

/* Members per block of etm_count_tiles_tc for an element code (0 for an unknown code). */
int etm_gram_block_members(int32_t elem);

/*
 * Dense tensor-core rate of the Gram's MMA shape for `elem` (M = 128, N = the
 * block size, the format's K per instruction), in TFLOP/s: every SM issues
 * `iters` back-to-back MMAs on a zeroed shared-memory tile, timed with CUDA
 * events on `stream` (synchronized). The roofline's tensor peak for that
 * operand format. No counterpart in the reference.
 */
int etm_tc_mma_rate(int32_t elem, int64_t iters, double* out_tflops, void* stream);

/*
 * AND+popcount rate of the tile kernels' inner loop, in 10^9 popc(a & b) pair
 * words per second: 8 CTAs per SM of 256 threads, each adding popc(a_r & b_c)
 * for a 4 x 4 register block `iters` times (timed with CUDA events on
 * `stream`, synchronized). The roofline of etm_count_tiles* on words that stay
 * in shared memory: those kernels are bound by the popcount pipe, not by HBM.
 * No counterpart in the reference.
 */
int etm_popc_rate(int64_t iters, double* out_gops, void* stream);

/*
 * Reads and clears the device status words the tensor-core kernels and the
 * projection (its bulk copies) raise when a bounded wait gives up
 * (synchronizes `stream`). Returns 0, ETM_ETIMEOUT (the kernel gave up and
 * cleaned up: its counts are incomplete, the device stays usable),
 * ETM_EUNSAFE (the projection's cleanup wait ran out too: stop using the
 * device) or ETM_EINVAL (etm_project_rows skipped a unit whose members lie
 * past its row-major copy). The words are per device, shared by every caller
 * of the library.
 */
int etm_device_status(void* stream);

/*
 * Limits of the first bounded waits, in nanoseconds: the Gram's MMA thread
 * waiting for a filled stage and the projection waiting for a group's bulk
 * copies (negative: the default of 2 s; 0: give up at once, which drives the
 * give-up path without a real stall). The cleanup waits keep their own 2 s
 * limit. Applies to launches after the call, process-wide.
 */
int etm_set_wait_limits(int64_t gram_first_wait_ns, int64_t proj_first_wait_ns);

/*
 * etm_count_tiles (popcount method) with each tile-pair's word range cut into
 * n_split parts counted by different CTAs, which atomically add their partial
 * counts into out_counts: the caller zeroes the counted candidates' slots
 * first. For groups with few members over many rows (K=2 past the Gram's 2^24
 * rows), where the tile-pairs alone cannot fill the GPU. n_tiles =
 * work_off[n_work] sizes the grid. Dense counts (no threshold).
 */
int etm_count_tiles_split(const uint64_t* fbv, int64_t ld, int64_t n_words, const int32_t* rows, int32_t width,
                          const int64_t* grp_first, const int32_t* grp_size, const int64_t* cand_off,
                          const int64_t* work_groups, const int64_t* work_off, int64_t n_work, int64_t n_tiles,
                          int64_t chunk_base, const uint8_t* cls, int32_t n_split, int32_t* out_counts, void* stream);

/*
 * The fused-threshold ("select") forms of the counting entry points, after
 * count_shared_tiled_fused (gpu/kernels/_src/shared_tiled.cu:246-280): each
 * takes min_count and a survivor bitmask surv_bits (uint32 words; bit t % 32
 * of word t / 32 is chunk-relative candidate t; the caller zeroes
 * ceil(n_cands / 32) words before the chunk's first call). Of the candidates
 * a call counts, only those reaching min_count get out_counts[t] written and
 * their bit set; the other slots are left untouched. etm_classify_sel sets
 * the bit of an inferred candidate reaching min_count; with ETM_SUBSET_BOUNDS
 * in mode it also applies the deduction bounds, from the complete levels k-2
 * (deep2: rows [deep2_n][k-2] sorted, counts) and, for k > 3, k-3 (deep3),
 * with n_transactions the count of the empty set at k = 3. Arguments otherwise as
 * in the dense forms (etm_count_tiles with the popcount method,
 * etm_count_cands, etm_count_tiles_proj, etm_classify). etm_count_cands_sel
 * takes the tile occupancy of fbv (occ, occ_ld; NULL for none, see
 * etm_tile_occupancy): a tile where one of the candidate's columns holds no
 * row is not read.
 */
int etm_count_tiles_sel(const uint64_t* fbv, int64_t ld, int64_t n_words, const int32_t* rows, int32_t width,
                        const int64_t* grp_first, const int32_t* grp_size, const int64_t* cand_off,
                        const int64_t* work_groups, const int64_t* work_off, int64_t n_work, int64_t chunk_base,
                        const uint8_t* cls, int32_t min_count, int32_t* out_counts, uint32_t* surv_bits,
                        void* stream);
int etm_count_cands_sel(const uint64_t* fbv, int64_t ld, int64_t n_words, const int32_t* rows, int32_t width,
                        const int64_t* grp_first, const int32_t* grp_size, const int64_t* cand_off,
                        const int64_t* work_groups, const int64_t* work_off, int64_t n_work, int64_t chunk_base,
                        const uint8_t* cls, int32_t min_count, int32_t* out_counts, uint32_t* surv_bits,
                        const uint64_t* occ, int64_t occ_ld, void* stream);
int etm_count_tiles_proj_sel(const uint64_t* cbuf, const int64_t* cbase, const int64_t* cwords, const int64_t* cld,
                             const int32_t* grp_size, const int64_t* cand_off, const int64_t* work_groups,
                             const int64_t* work_off, int64_t n_work, int64_t chunk_base, const uint8_t* cls,
                             int32_t min_count, int32_t* out_counts, uint32_t* surv_bits, void* stream);
int etm_classify_sel(const int32_t* rows, int32_t width, int64_t n_rows, const int32_t* counts,
                     const uint8_t* free_flags, const int64_t* grp_first, const int32_t* grp_size,
                     const int64_t* cand_off, int64_t g0, int64_t g1, int32_t mode, int32_t min_count,
                     const int32_t* deep2_rows, int64_t deep2_n, const int32_t* deep2_counts,
                     const int32_t* deep3_rows, int64_t deep3_n, const int32_t* deep3_counts,
                     int64_t n_transactions, uint8_t* out_cls, int32_t* out_counts, uint32_t* surv_bits,
                     void* stream);

/*
 * Survivor bits of a chunk whose counts are dense (the row-wise kernels):
 * bit t set when counts[t] >= min_count and (cls NULL or cls[t] != SKIP).
 * Writes every one of the ceil(n_cands / 32) words. Replaces the comparison
 * half of threshold_filter (gpu/kernels/filter.py:85-120).
 */
int etm_threshold_bits(const int32_t* counts, const uint8_t* cls, int64_t n_cands, int32_t min_count,
                       uint32_t* surv_bits, void* stream);

/*
 * etm_level_compact over a survivor bitmask instead of dense counts: the
 * ordered scan runs over the ceil(n_cands / 32) words (a 32nd of the
 * elements), and each set bit t is decoded into a row of width+1 columns with
 * count counts[t], in candidate order. acc, cap and the output rules as in
 * etm_level_compact; ws: ceil(n_cands / 32) / 4096 + 3 words. Replaces
 * threshold_filter's compaction (gpu/kernels/filter.py:165-237) and the
 * decode steps (gpu/kernels/decode.py:9-73).
 */
int etm_level_compact_bits(const uint32_t* surv_bits, const int32_t* counts, int64_t n_cands, const int32_t* rows,
                           int32_t width, const int64_t* grp_first, const int32_t* grp_size, const int64_t* cand_off,
                           int64_t g0, int64_t g1, int32_t* out_rows, int32_t* out_counts, int64_t cap,
                           int64_t* acc, int64_t* ws, int64_t ws_words, void* stream);

/*
 * Survivors of a counted chunk (groups [g0, g1)), in candidate order, decoded
 * into rows of width+1 columns. Replaces threshold_filter
 * (gpu/kernels/filter.py:85-120), decode_k2_pairs_flat / decode_k3plus_flat
 * (gpu/kernels/decode.py:9-73) and the level-end lexsort
 * (gpu/row_split.py:1064-1067): the output is already lexicographic.
 * A candidate survives when its count >= min_count and (cls NULL or its class
 * is not SKIP). acc int64 [1] (device) is the running row total: rows are
 * written at acc[0] + rank while that is < cap, and acc[0] grows by the
 * survivors even past cap (the caller grows the output and repeats the call
 * with acc reset). ws: n_cands/4096 + 3 words.
 */
int etm_level_compact(const int32_t* counts, const uint8_t* cls, int64_t n_cands, const int32_t* rows,
                      int32_t width, const int64_t* grp_first, const int32_t* grp_size, const int64_t* cand_off,
                      int64_t g0, int64_t g1, int32_t min_count, int32_t* out_rows, int32_t* out_counts,
                      int64_t cap, int64_t* acc, int64_t* ws, int64_t ws_words, void* stream);

/*
 * etm_level_compact without the workspace argument, for callers that cannot
 * allocate device memory (a serving process that reserved its memory up front,
 * a host runtime calling through plain C with no allocator of its own). No
 * counterpart in the reference: its compaction always allocates through CuPy.
 * The scan scratch is a 512 KB array compiled into the library, one per GPU,
 * held until the process exits. Limit: n_cands <= 268,435,456 (65,536 scan
 * blocks of 4096); larger chunks fail with ETM_ENOSPACE. The first call on a
 * device looks up that device's array address (cudaGetSymbolAddress), so make
 * that first call before any stream capture. All calls on a device share the
 * array: calls that overlap on the GPU (other streams, or other host threads)
 * race and must be serialized by the caller. The cached address belongs to
 * the device's primary context (the CUDA runtime's): the entry point assumes
 * that context is current and that no cudaDeviceReset happens between calls.
 * Everything else (acc, cap, outputs, ordering) is as in etm_level_compact.
 */
int etm_level_compact_static(const int32_t* counts, const uint8_t* cls, int64_t n_cands, const int32_t* rows,
                             int32_t width, const int64_t* grp_first, const int32_t* grp_size,
                             const int64_t* cand_off, int64_t g0, int64_t g1, int32_t min_count, int32_t* out_rows,
                             int32_t* out_counts, int64_t cap, int64_t* acc, void* stream);

/*
 * Free flags and subset presence of a new level (k = width + 1 columns)
 * against the generating level prev (n_prev x width, with counts).
 * Replaces the free-set tests (core/cpu_miner.py:943-945, 1139-1151;
 * gpu/mining.py:81-139; rust_ext/src/core/groups.rs:250-312).
 * out_free[t] = no (k-1)-subset of row t has its count; out_present[t] = every
 * (k-1)-subset of row t is a row of prev. Either output may be NULL.
 */
int etm_level_subsets(const int32_t* new_rows, const int32_t* new_counts, int64_t n_new, int32_t width,
                      const int32_t* prev_rows, const int32_t* prev_counts, int64_t n_prev, uint8_t* out_free,
                      uint8_t* out_present, void* stream);

/*
 * Keep the rows whose keep[] flags are all set (the free-set prune,
 * gpu/row_split.py:1075-1100), in order. keep_a / keep_b uint8 (keep_b
 * nullable). acc and cap as in etm_level_compact. ws: n/4096 + 3 words.
 */
int etm_select_rows(const int32_t* rows, const int32_t* counts, const uint8_t* keep_a, const uint8_t* keep_b,
                    int64_t n, int32_t width, int32_t* out_rows, int32_t* out_counts, uint8_t* out_flag_src,
                    uint8_t* out_flag, int64_t cap, int64_t* acc, int64_t* ws, int64_t ws_words, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* ETM_H */
