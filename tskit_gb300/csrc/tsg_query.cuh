// Query parameters and workspace views shared by the statistics kernels.
#pragma once

#include "tsg_internal.cuh"

namespace tsg {

struct Term {
    int32_t type;
    int32_t idx[4];
};

struct QueryParams {
    int32_t K, KP, R, Wn;
    int32_t branch, site, polarised, f32, need_mean;
    int32_t site_int;  // site summaries from exact integer numerators (term_num)
    int32_t num_slots;
    uint32_t spin_limit;  // polls of a bounded wait before it gives up
    double inv_K;
    double set_size[TSG_MAX_SAMPLE_SETS];
    int32_t set_size_i[TSG_MAX_SAMPLE_SETS];  // the same as integers (integer kernels)
    double inv_size[TSG_MAX_SAMPLE_SETS];  // 1 / n_k
    double inv[TSG_MAX_OUTPUTS];           // reciprocal denominator of each term
    // the same in FP32 (rounded once on the host) for the FP32 evaluation
    float set_size_f[TSG_MAX_SAMPLE_SETS];
    float inv_size_f[TSG_MAX_SAMPLE_SETS];
    float inv_f[TSG_MAX_OUTPUTS];
    float inv_K_f;
    Term term[TSG_MAX_OUTPUTS];
    // the terms grouped by summary type (the grouped item evaluation gives
    // each warp one type): group g holds gterm[gfirst[g] .. gfirst[g + 1])
    int32_t ngroups;
    int32_t gfirst[TSG_MAX_OUTPUTS + 1];
    int32_t gterm[TSG_MAX_OUTPUTS];
    // the warps of one block of TSG_EVAL_BLOCK chunks: warp `sub` of a block
    // takes group gw_group[sub], lanes gw_k[sub] * 32 .. of its (chunk, term)
    // pairs
    int32_t gwpb;
    int32_t gw_group[TSG_MAX_OUTPUTS];
    int32_t gw_k[TSG_MAX_OUTPUTS];
};
// chunks per block of the grouped item evaluation
#define TSG_EVAL_BLOCK 8

struct QueryDev {
    const uint32_t *sample_mask;  // per sample index: bit k = member of set k
    const uint32_t *node_mask;    // per node: its sample-set membership bits (workspace)
    const int32_t *win_site_lo;   // per window: first site (num_windows + 1 entries)
    const double *windows;        // Wn + 1
    const int32_t *span_wlo;      // per span: first window overlapping it
    const int64_t *span_woff;     // per span: offset into span-window arrays
    const int32_t *win_span_lo;   // per window: first overlapping span
    const int32_t *win_span_hi;   // per window: last overlapping span
    // the same for the window segments (item pipeline)
    const int32_t *seg_wlo;
    const int64_t *seg_woff;
    const int32_t *win_seg_lo;
    const int32_t *win_seg_hi;
};

struct WsDev {
    int32_t *parent;  // num_slots * N
    int32_t *nchild;  // num_slots * N: children in the tree at the span start
    int32_t *arrive;  // num_slots * N: children whose counts have been added
    int32_t *x;       // num_slots * N * KP
    double *A;        // span windows
    double *B;        // span windows * R
    double *SITE;     // span windows * R
    double *D;        // spans * R
    double *RS;       // spans * R
    double *rs0;      // R
    void *items;      // replay items (item pipeline)
    void *bl;         // per item: its two branch lengths in the evaluation's arithmetic
    void *state;      // per-CTA span node state (item pipeline, global-memory form)
    uint32_t *seekcnt;    // per-CTA seek counters (item pipeline)
    uint64_t *mcnt;   // packed counts under each mutation (shared-memory sweep)
    double *dD;       // chunks * R: running-sum change of each item chunk
    uint32_t *node_mask;  // per node sample-set bits
    double *site_val;     // R * sites: per-site summary, term-major (item pipeline)
    double *site_win;     // windows * R: per-window site sums (shared-memory sweep)
    unsigned long long *leaf_area;  // 3 x windows x 2^K patterns: leaf branch areas (fixed point)
    double *leaf_dbl;     // windows x 2^K patterns: the areas
    double *leaf_win;     // windows * R: the leaves' part of the branch sums
    unsigned long long *site_acc;  // windows x R x 2: exact site-sum counters (integer form)
    uint64_t *cp0;        // (samples + 1) x 2: prefix sums along the first span's order
                          // (compact replay)
    // compact plan, per sample-range endpoint: the KQ packed counts of the
    // members before its position within its chunk of order rows; per span
    // and chunk, the chunk's total (k_compact_rows)
    uint64_t *c_pep;
    uint64_t *c_ctot;
    int32_t *err;
    int32_t *counter;
};


template <typename F>
__device__ __forceinline__ F warp_sum(F v)
{
    for (int o = 16; o > 0; o >>= 1) {
        v += __shfl_xor_sync(0xffffffffu, v, o);
    }
    return v;
}

// Allele frequency spectrum of one query.  Counts carry the K sample sets
// plus a last field with all of the tree sequence's samples.
#define TSG_AFS_KMAX 7
// fixed-point accumulation of branch areas (tsg_fixed.cuh)
#ifndef TSG_FX_LIMBS
#define TSG_FX_LIMBS 8
#define TSG_FX_FRAC 128
#endif
struct AfsParams {
    int32_t K;              // sample sets
    int32_t Wn, TW;         // windows, time windows
    int32_t polarised;
    int64_t num_samples;
    int64_t afs_size;       // prod (n_k + 1)
    int64_t dims[TSG_AFS_KMAX];    // n_k + 1
    int64_t stride[TSG_AFS_KMAX];  // C order
    const double *windows;       // Wn + 1
    const double *time_windows;  // TW + 1
    unsigned long long *acc;     // branch: Wn * TW * afs_size bins x TSG_FX_LIMBS
    double *out;                 // site: Wn * afs_size (the result)
    int32_t *err;
    int32_t *counter;
    uint32_t *seekcnt;           // per-CTA seek counters
};

// Allele frequency spectrum launchers (tsg_afs.cu).  form as for the item
// evaluation; slot_bytes: per-CTA node state in global memory (0: shared).
int launch_afs_branch(int form, unsigned grid, size_t smem, int64_t slot_bytes, void *state,
    cudaStream_t st, const TSView &v, const QueryDev &qd, const AfsParams &a);
int launch_afs_site(int form, cudaStream_t st, const TSView &v, const AfsParams &a,
    const uint64_t *mcnt);
int launch_afs_finish(cudaStream_t st, const AfsParams &a, int span_normalise, int branch,
    double *result);
void *afs_replay_kernel(int form);

// Branch genetic relatedness matrix-vector product (one query).  Work item:
// a group of consecutive spans x a block of 32 weight columns (one column
// per lane), with node state in a per-CTA slot of global memory.
#define TSG_MV_WARPS 16
struct MvParams {
    int32_t W;          // weight columns
    int32_t ncb;        // blocks of 32 columns
    int32_t Wn;         // windows
    int32_t G;          // span groups
    int64_t nf;         // focal nodes
    int64_t L;          // stateful nodes per span, at most
    int64_t slot_bytes;
    const double *windows;     // Wn + 1
    const int32_t *focal;      // nf
    const int32_t *group_span; // G + 1: first span of each group
    const int32_t *group_wlo;  // G: first window of each group (-1: none)
    const int64_t *pair_off;   // G + 1: (group, window) partial blocks
    const int32_t *win_glo;    // Wn: first group contributing to each window
    const int32_t *win_ghi;    // Wn: last group contributing (win_glo > win_ghi: none)
    const double *weights;     // n x W, as given
    double *wc;                // n x W: weights centred over samples (or as given)
    double *partial;           // pairs x nf x W
    unsigned char *slots;      // grid x slot_bytes
    int32_t *err;
    int32_t *counter;
    int32_t centre;
};

// Relatedness-vector launchers (tsg_matvec.cu).
int launch_matvec(unsigned grid, cudaStream_t st, const TSView &v, const MvParams &m,
    int span_normalise, double *result);
int64_t matvec_slot_bytes(const TSView &v, int64_t L);
const void *k_matvec_ptr();

// Arbitrary summary functions (tsg_general.cu).
int gen_collect(int form, const TSView &v, const QueryParams &q, const WsDev &w,
    const int64_t *site_off, int64_t num_site_keys, uint64_t *klo, uint64_t *khi, uint64_t *tlo,
    uint64_t *thi, int64_t *flag, int64_t *pos, void *cub_tmp, size_t cub_bytes, uint64_t *ulo,
    uint64_t *uhi, int64_t *U, cudaStream_t st);
size_t gen_cub_bytes(int64_t n);
int genw_replay(const TSView &v, const QueryParams &q, const double *W, bool node_w, int K,
    double *slots_x, int32_t *slots_par, uint8_t *slots_touched, int grid, int4 *ids, double *xs,
    double *mstate, double *init, int32_t *err, int32_t *counter, cudaStream_t st);
// node mode
int node_init(const TSView &v, int K, const double *W, bool node_w, double *init,
    cudaStream_t st);
int genw_summary_descendants(const double *states, int64_t U, int K, double *vals,
    cudaStream_t st);
size_t node_sort_bytes(int64_t I);
int node_order(const TSView &v, int K, const int4 *ids, const double *xs, const double *init,
    uint64_t *keys, uint64_t *keys_sorted, int32_t *idx, int32_t *idx_sorted, void *temp,
    size_t temp_bytes, double *states, int32_t *err, cudaStream_t st);
int node_term_values(const QueryParams &q, const double *states, int64_t U, int K, bool unpol,
    double *vals, cudaStream_t st);
int node_walk(const TSView &v, int Wn, const double *windows, const uint64_t *keys_sorted,
    const int32_t *idx_sorted, const double *vals, int R, bool span_normalise, double *result,
    int32_t *err, cudaStream_t st);
int genw_states(const TSView &v, int K, const double *W, const double *total,
    const double *mstate, const int64_t *site_off, double *site_states, double *leaf_states,
    cudaStream_t st);
int genw_summary_trait(const double *states, int64_t U, int K, int R, int kind, double n,
    const double *V, const double *total, bool complement, double *vals, cudaStream_t st);
int genw_summary_relatedness(const double *states, int64_t U, int K1, const double *total,
    const int32_t *tuples, int R, double ones, bool centred, bool complement, double *vals,
    cudaStream_t st);
int genw_eval(const TSView &v, const QueryParams &q, const QueryDev &d, const WsDev &w,
    const int4 *ids, const double *vals, const int64_t *site_off, int64_t sbase, int64_t lbase,
    unsigned long long *leaf_acc, int32_t R_total, int32_t r0, cudaStream_t st);
int gen_eval(int form, const TSView &v, const QueryParams &q, const WsDev &w,
    const int64_t *site_off, const uint64_t *ulo, const uint64_t *uhi, int64_t U, const double *F,
    int32_t R_total, int32_t r0, cudaStream_t st);
int gen_unpack(int W, const uint64_t *ulo, const uint64_t *uhi, int64_t U, int K, int32_t *out,
    cudaStream_t st);

// term budget of the item evaluation (accumulators per lane)
#define TSG_ITEM_RMAX 32

// Item replay with evaluation (tsg_eval_*.cu), FP32/FP64 x polarised/unpolarised:
// launchers and kernel handles.  form: count width and words,
// (W == 16 ? 0 : 2) + (KQ == 1 ? 0 : 1).
#define TSG_REPLAY_EVAL_LAUNCHER(name)                                                   \
    void name(int form, unsigned grid, size_t smem, int64_t slot_bytes, cudaStream_t st, \
        const TSView &v, const QueryParams &p, const QueryDev &d, const WsDev &w)
#define TSG_REPLAY_EVAL_FN(name) void *name(int form)
TSG_REPLAY_EVAL_LAUNCHER(launch_replay_eval_f32_pol);
TSG_REPLAY_EVAL_LAUNCHER(launch_replay_eval_f32_unpol);
TSG_REPLAY_EVAL_LAUNCHER(launch_replay_eval_f64_pol);
TSG_REPLAY_EVAL_LAUNCHER(launch_replay_eval_f64_unpol);
TSG_REPLAY_EVAL_FN(replay_eval_fn_f32_pol);
TSG_REPLAY_EVAL_FN(replay_eval_fn_f32_unpol);
TSG_REPLAY_EVAL_FN(replay_eval_fn_f64_pol);
TSG_REPLAY_EVAL_FN(replay_eval_fn_f64_unpol);
// Every chunk's item values after the compact replay, which wrote each
// item's branch lengths with it (kq: count words per node, 1 or 2).
#define TSG_CHUNK_EVAL_LAUNCHER(name)                                                    \
    void name(int kq, cudaStream_t st, const TSView &v, const QueryParams &p, const WsDev &w)
TSG_CHUNK_EVAL_LAUNCHER(launch_eval_chunks_f32_pol);
TSG_CHUNK_EVAL_LAUNCHER(launch_eval_chunks_f32_unpol);
TSG_CHUNK_EVAL_LAUNCHER(launch_eval_chunks_f64_pol);
TSG_CHUNK_EVAL_LAUNCHER(launch_eval_chunks_f64_unpol);

// One query of a batched launch (tsg_batch_*), device-resident: the batched
// kernels give each query its own range of blocks (a prefix array of block
// counts per stage) and run the query's stage body on its descriptor.
struct BatchQuery {
    TSView v;
    QueryParams p;
    QueryDev d;
    WsDev w;
    double *result;
    int32_t span_normalise;
    int32_t pad;
};

// The query owning global block `blk`: the last b in [0, nq) with
// off[b] <= blk (queries with no blocks in a stage have off[b] == off[b + 1]).
__device__ __forceinline__ int batch_find(const int64_t *off, int nq, int64_t blk)
{
    int lo = 0, hi = nq;
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (off[mid] <= blk) {
            lo = mid;
        } else {
            hi = mid;
        }
    }
    return lo;
}

// Prologue of a batched stage kernel: Q, this block's query; bid, nb: the
// block's index within the query's range and the range's length.
#define TSG_BATCH_QUERY()                                                     \
    const int b_ = batch_find(off, nq, (int64_t) blockIdx.x);                \
    const BatchQuery &Q = bq[b_];                                             \
    const int64_t bid = (int64_t) blockIdx.x - off[b_];                       \
    const int64_t nb = off[b_ + 1] - off[b_]

// The chunk evaluation of a batch (kq as above): the item values, one launch
// over the batch's queries.
#define TSG_CHUNK_EVAL_BATCH_LAUNCHER(name)                                              \
    void name(int kq, cudaStream_t st, const BatchQuery *bq, int nq, const int64_t *off_eval, \
        int64_t blocks_eval)
TSG_CHUNK_EVAL_BATCH_LAUNCHER(launch_eval_chunks_batch_f32_pol);
TSG_CHUNK_EVAL_BATCH_LAUNCHER(launch_eval_chunks_batch_f32_unpol);
TSG_CHUNK_EVAL_BATCH_LAUNCHER(launch_eval_chunks_batch_f64_pol);
TSG_CHUNK_EVAL_BATCH_LAUNCHER(launch_eval_chunks_batch_f64_unpol);

// The other stages of a batch (tsg_batch.cu).
enum BatchStage {
    BS_ZERO, BS_NODE_MASK, BS_PREFIX, BS_ANCHORS, BS_EVAL, BS_SPAN_WINDOWS,
    BS_LEAF_AREAS, BS_LEAF_PREFIX, BS_LEAF_TERMS, BS_SITE_SUMS, BS_SITE_FINISH, BS_SPAN_SCAN,
    BS_REDUCE, BS_ROWS, BS_COUNT
};
int batch_launch_stage(int stage, int kq, int64_t blocks, cudaStream_t st, const BatchQuery *bq,
    int nq, const int64_t *off);
int batch_launch_replay(int kq, unsigned grid, size_t smem, cudaStream_t st, const BatchQuery *bq,
    int nq, const int64_t *span_off, int32_t *counter);
void *batch_replay_kernel(int kq);

}  // namespace tsg

#include "tsg_terms.cuh"
