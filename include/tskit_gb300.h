/*
 * tskit_gb300: GPU (sm_103a) tree-sequence statistics behind a C ABI.
 *
 * The entry points mirror the reference C library's statistics functions
 * (c/tskit/trees.h) one for one: same argument order and meaning, the same
 * TSK_STAT_* option bits, the same negative TSK_ERR_* return codes for the
 * same conditions, caller-allocated results that are zeroed and filled.  The
 * tree sequence itself is device resident (tsg_treeseq_t, built once by
 * tsg_treeseq_init) in place of the reference's host tsk_treeseq_t.
 *
 * Host-pointer entry points (tsg_treeseq_<stat>) take host arrays and a host
 * result, exactly as the reference does, and synchronise before returning.
 * The device-resident query interface (tsg_query_*) takes device arrays, a
 * workspace and a CUDA stream and does not synchronise; it is what the
 * batched and serving paths use.
 *
 * No exceptions cross this boundary; every function returns 0 or a negative
 * error code, and tsg_strerror() gives a message.
 */
#ifndef TSKIT_GB300_H
#define TSKIT_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Option bits: same values as c/tskit/trees.h:47-56. */
#define TSG_STAT_SITE (1u << 0)
#define TSG_STAT_BRANCH (1u << 1)
#define TSG_STAT_NODE (1u << 2)
#define TSG_STAT_POLARISED (1u << 10)
#define TSG_STAT_SPAN_NORMALISE (1u << 11)
#define TSG_STAT_ALLOW_TIME_UNCALIBRATED (1u << 12)
#define TSG_STAT_PAIR_NORMALISE (1u << 13)
#define TSG_STAT_NONCENTRED (1u << 14)
/* Extension bits (no reference counterpart): run both modes in one sweep,
 * and the arithmetic of the bulk accumulation. */
#define TSG_STAT_BOTH_MODES (1u << 20)
#define TSG_PRECISION_F32_KAHAN (1u << 21)
/* Use the general sweep even when the item pipeline applies (for testing
 * the general path). */
#define TSG_FORCE_GLOBAL_SWEEP (1u << 22)
/* Run the item pipeline with its span node state in global memory (32-bit
 * counts) even when it fits in shared memory (for testing that form). */
#define TSG_FORCE_GLOBAL_STATE (1u << 23)
/* For testing the bounded device waits: the evaluating warps of the general
 * replay (tree sequences without a compact plan) give up their wait for the
 * replay at once instead of after 2^27 polls, so a launch
 * records TSG_ERR_DEVICE_CHECK in its check word (its result is then not
 * valid) and returns normally; the next launch without the bit is clean. */
#define TSG_TEST_WAIT_EXPIRES (1u << 24)

/* tsg_treeseq_init options */
#define TSG_TABLES_ON_DEVICE (1u << 0)
/* tsg_treeseq_init option: the node times are uncalibrated (time_units
 * "uncalibrated"); branch-mode statistics then need
 * TSG_STAT_ALLOW_TIME_UNCALIBRATED (c/tskit/trees.c:1383, 3723) */
#define TSG_TIME_UNCALIBRATED (1u << 1)

/* Error codes: the reference's values (c/tskit/core.h:255-751) where the
 * condition is the same; GPU-specific conditions below -20000. */
#define TSG_ERR_GENERIC (-1)
#define TSG_ERR_NO_MEMORY (-2)
#define TSG_ERR_IO (-3)
#define TSG_ERR_BAD_PARAM_VALUE (-4)
#define TSG_ERR_FILE_FORMAT (-100)
#define TSG_ERR_FILE_VERSION_TOO_OLD (-101)
#define TSG_ERR_FILE_VERSION_TOO_NEW (-102)
#define TSG_ERR_REQUIRED_COL_NOT_FOUND (-103)
#define TSG_ERR_BOTH_COLUMNS_REQUIRED (-104)
#define TSG_ERR_BAD_COLUMN_TYPE (-105)
#define TSG_ERR_BAD_OFFSET (-200)
#define TSG_ERR_TIME_NONFINITE (-210)
#define TSG_ERR_NODE_OUT_OF_BOUNDS (-202)
#define TSG_ERR_BAD_NODE_TIME_ORDERING (-306)
#define TSG_ERR_DUPLICATE_SAMPLE (-600)
#define TSG_ERR_BAD_SAMPLES (-601)
#define TSG_ERR_TABLES_NOT_INDEXED (-702)
#define TSG_ERR_BAD_NUM_WINDOWS (-900)
#define TSG_ERR_BAD_WINDOWS (-901)
#define TSG_ERR_MULTIPLE_STAT_MODES (-902)
#define TSG_ERR_BAD_STATE_DIMS (-903)
#define TSG_ERR_BAD_RESULT_DIMS (-904)
#define TSG_ERR_INSUFFICIENT_SAMPLE_SETS (-905)
#define TSG_ERR_INSUFFICIENT_INDEX_TUPLES (-906)
#define TSG_ERR_BAD_SAMPLE_SET_INDEX (-907)
#define TSG_ERR_EMPTY_SAMPLE_SET (-908)
#define TSG_ERR_UNSUPPORTED_STAT_MODE (-909)
#define TSG_ERR_TIME_UNCALIBRATED (-910)
#define TSG_ERR_STAT_POLARISED_UNSUPPORTED (-911)
#define TSG_ERR_INSUFFICIENT_WEIGHTS (-913)
#define TSG_ERR_BAD_TIME_WINDOWS_DIM (-922)
#define TSG_ERR_BAD_TIME_WINDOWS (-924)
#define TSG_ERR_CUDA (-20001)
#define TSG_ERR_DEVICE_CHECK (-20002)
#define TSG_ERR_TOO_MANY_SAMPLE_SETS (-20003)
#define TSG_ERR_TOO_MANY_OUTPUTS (-20004)
#define TSG_ERR_BAD_TREE_SEQUENCE (-20005)
#define TSG_ERR_WORKSPACE_TOO_SMALL (-20006)
#define TSG_ERR_NOALLOC_TOO_LARGE (-20007)

/* Summary terms of the named statistics (c/tskit/trees.c summary funcs). */
#define TSG_DIVERSITY 1                  /* trees.c:3934  idx: i       */
#define TSG_SEGREGATING_SITES 2          /* trees.c:4221  idx: i       */
#define TSG_Y1 3                         /* trees.c:4248  idx: i       */
#define TSG_DIVERGENCE 4                 /* trees.c:4690  idx: i,j     */
#define TSG_Y2 5                         /* trees.c:4899  idx: i,j     */
#define TSG_F2 6                         /* trees.c:4938  idx: i,j     */
#define TSG_Y3 7                         /* trees.c:5177  idx: i,j,k   */
#define TSG_F3 8                         /* trees.c:5219  idx: i,j,k   */
#define TSG_F4 9                         /* trees.c:5266  idx: i,j,k,l */
#define TSG_RELATEDNESS 10               /* trees.c:4729  idx: i,j     */
#define TSG_RELATEDNESS_NONCENTRED 11    /* trees.c:4755  idx: i,j     */

/* Limits of the device sweep. */
#define TSG_MAX_SAMPLE_SETS 32
#define TSG_MAX_OUTPUTS 64

typedef struct tsg_treeseq tsg_treeseq_t;
typedef struct tsg_workspace tsg_workspace_t;

/*
 * Columns of a tree sequence (the subset of tsk_table_collection_t the
 * statistics read).  With TSG_TABLES_ON_DEVICE every pointer is a device
 * pointer that must outlive the tsg_treeseq_t; otherwise they are host
 * pointers that are copied.  Edges must be sorted as the reference requires
 * and the two edge indexes built (c/tskit/tables.c:11393-11450).  Mutation
 * alleles are integer codes per site: 0 is the ancestral state, each new
 * derived state string takes the next code in mutation order; alt is the code
 * of the parent mutation's derived state (0 without parent).
 */
typedef struct {
    double sequence_length;
    int64_t num_nodes;
    int64_t num_edges;
    int64_t num_sites;
    int64_t num_mutations;
    const double *node_time;
    const uint32_t *node_flags;
    const double *edge_left;
    const double *edge_right;
    const int32_t *edge_parent;
    const int32_t *edge_child;
    const int32_t *edge_insertion_order;
    const int32_t *edge_removal_order;
    const double *site_position;
    const int32_t *mutation_site;
    const int32_t *mutation_node;
    const int32_t *mutation_allele;
    const int32_t *mutation_alt_allele;
} tsg_tables_t;

/* Replaces tsk_treeseq_init (c/tskit/trees.c:455-545): validates the tables
 * on the device and builds the derived per-tree-sequence state (samples,
 * tree breakpoints, per-tree edge and site ranges, span plan).  num_spans 0
 * picks a default.  Synchronous. */
int tsg_treeseq_init(tsg_treeseq_t **ts, const tsg_tables_t *tables, int64_t num_spans,
    uint32_t options);
int tsg_treeseq_free(tsg_treeseq_t *ts);
int64_t tsg_treeseq_get_num_trees(const tsg_treeseq_t *ts);
int64_t tsg_treeseq_get_num_samples(const tsg_treeseq_t *ts);
int64_t tsg_treeseq_get_num_spans(const tsg_treeseq_t *ts);
/* The compact replay plan behind the sample-count statistics (no reference
 * counterpart): short spans whose node state holds only the nodes their
 * edge events touch, for tree sequences of up to 65,535 samples.  get: its
 * span count (0 when the tree sequence uses the general replay).  set:
 * rebuild it with about num_spans spans (-1: the default count; 0: use the
 * general replay; a count
 * whose spans touch more than 4,096 nodes also leaves the general replay
 * serving); queries prepared before must not run concurrently with it, and
 * a query prepared against a plan with fewer spans or range endpoints than
 * the rebuilt one runs on the general replay (its workspace holds the
 * compact replay's per-endpoint counts for the plan it was prepared
 * against).  Results do not depend on the span count. */
int64_t tsg_treeseq_get_num_compact_spans(const tsg_treeseq_t *ts);
/* Sizes of the tree sequence's replay plans (no reference counterpart; for
 * measuring): sizes[0..7] = trees, spans of the general plan, spans of the
 * compact plan, compact nodes over all spans, their sample-range endpoints,
 * replay items, evaluation chunks, first-tree items of the compact plan (the
 * compact entries 0 without a compact plan). */
int tsg_treeseq_get_plan_sizes(const tsg_treeseq_t *ts, int64_t *sizes);
int tsg_treeseq_set_compact_spans(tsg_treeseq_t *ts, int64_t num_spans);
/* breakpoints: host array of num_trees + 1 doubles */
int tsg_treeseq_get_breakpoints(const tsg_treeseq_t *ts, double *breakpoints);
const char *tsg_strerror(int err);

/* ---------------------------------------------------------------- one-way
 * Same arguments as tsk_treeseq_diversity / segregating_sites / Y1
 * (c/tskit/trees.h, "One way sample set stats"). Host pointers. */
int tsg_treeseq_diversity(const tsg_treeseq_t *self, uint64_t num_sample_sets,
    const uint64_t *sample_set_sizes, const int32_t *sample_sets, uint64_t num_windows,
    const double *windows, uint32_t options, double *result);
int tsg_treeseq_segregating_sites(const tsg_treeseq_t *self, uint64_t num_sample_sets,
    const uint64_t *sample_set_sizes, const int32_t *sample_sets, uint64_t num_windows,
    const double *windows, uint32_t options, double *result);
int tsg_treeseq_Y1(const tsg_treeseq_t *self, uint64_t num_sample_sets,
    const uint64_t *sample_set_sizes, const int32_t *sample_sets, uint64_t num_windows,
    const double *windows, uint32_t options, double *result);

/* ---------------------------------------------------------------- k-way
 * Same arguments as tsk_treeseq_divergence / Y2 / f2 / Y3 / f3 / f4 /
 * genetic_relatedness (c/tskit/trees.h, "Two/Three/Four way sample set
 * stats"); index_tuples has num_index_tuples * k entries. */
int tsg_treeseq_divergence(const tsg_treeseq_t *self, uint64_t num_sample_sets,
    const uint64_t *sample_set_sizes, const int32_t *sample_sets,
    uint64_t num_index_tuples, const int32_t *index_tuples, uint64_t num_windows,
    const double *windows, uint32_t options, double *result);
int tsg_treeseq_Y2(const tsg_treeseq_t *self, uint64_t num_sample_sets,
    const uint64_t *sample_set_sizes, const int32_t *sample_sets,
    uint64_t num_index_tuples, const int32_t *index_tuples, uint64_t num_windows,
    const double *windows, uint32_t options, double *result);
int tsg_treeseq_f2(const tsg_treeseq_t *self, uint64_t num_sample_sets,
    const uint64_t *sample_set_sizes, const int32_t *sample_sets,
    uint64_t num_index_tuples, const int32_t *index_tuples, uint64_t num_windows,
    const double *windows, uint32_t options, double *result);
int tsg_treeseq_Y3(const tsg_treeseq_t *self, uint64_t num_sample_sets,
    const uint64_t *sample_set_sizes, const int32_t *sample_sets,
    uint64_t num_index_tuples, const int32_t *index_tuples, uint64_t num_windows,
    const double *windows, uint32_t options, double *result);
int tsg_treeseq_f3(const tsg_treeseq_t *self, uint64_t num_sample_sets,
    const uint64_t *sample_set_sizes, const int32_t *sample_sets,
    uint64_t num_index_tuples, const int32_t *index_tuples, uint64_t num_windows,
    const double *windows, uint32_t options, double *result);
int tsg_treeseq_f4(const tsg_treeseq_t *self, uint64_t num_sample_sets,
    const uint64_t *sample_set_sizes, const int32_t *sample_sets,
    uint64_t num_index_tuples, const int32_t *index_tuples, uint64_t num_windows,
    const double *windows, uint32_t options, double *result);
int tsg_treeseq_genetic_relatedness(const tsg_treeseq_t *self, uint64_t num_sample_sets,
    const uint64_t *sample_set_sizes, const int32_t *sample_sets,
    uint64_t num_index_tuples, const int32_t *index_tuples, uint64_t num_windows,
    const double *windows, uint32_t options, double *result);

/* ------------------------------------------------ allele frequency spectrum
 * Replaces tsk_treeseq_allele_frequency_spectrum (c/tskit/trees.c:3830-3928):
 * same arguments, option bits and error codes; the result holds
 * num_windows x num_time_windows x prod(sample_set_sizes[k] + 1) doubles (C
 * order).  windows / time_windows may be NULL (whole genome / [0, inf)).
 * Up to 7 sample sets while every sample count fits 16 bits and a span's
 * node state fits in shared memory, else up to 3.  Branch areas are summed
 * exactly (fixed point, 2^-128 resolution) and rounded once per bin.  Host
 * pointers. */
int tsg_treeseq_allele_frequency_spectrum(const tsg_treeseq_t *self,
    uint64_t num_sample_sets, const uint64_t *sample_set_sizes, const int32_t *sample_sets,
    uint64_t num_windows, const double *windows, uint64_t num_time_windows,
    const double *time_windows, uint32_t options, double *result);

/* ------------------------------------------ genetic relatedness x vectors
 * Replaces tsk_treeseq_genetic_relatedness_vector (c/tskit/trees.c:
 * 10782-10816): branch mode only (site and node modes return
 * TSG_ERR_UNSUPPORTED_STAT_MODE, as the reference does).  weights:
 * num_samples x num_weights (row-major); result: num_windows x num_focal x
 * num_weights.  Options: TSG_STAT_SPAN_NORMALISE, TSG_STAT_NONCENTRED.
 * windows may be NULL (whole genome); they need not cover it.  Host pointers. */
int tsg_treeseq_genetic_relatedness_vector(const tsg_treeseq_t *self, uint64_t num_weights,
    const double *weights, uint64_t num_windows, const double *windows,
    uint64_t num_focal_nodes, const int32_t *focal_nodes, double *result, uint32_t options);

/* ------------------------------------------------- divergence matrix (site)
 * Replaces tsk_treeseq_divergence_matrix (c/tskit/trees.c:8900-9001) for
 * site and branch mode: same arguments, option bits, error codes and result
 * (num_windows x K x K, K = num_sample_sets, or every sample alone when
 * sample_sets is NULL).  Site mode: the pair counts come from an exact Gram
 * matrix of the 0/1 genotypes on the tensor cores.  Branch mode: each pair's
 * path length through its MRCA per tree (c/tskit/trees.c:8578-8672), one CTA
 * per 32 x 32 tile of pairs.  Node mode returns
 * TSG_ERR_UNSUPPORTED_STAT_MODE, as the reference does.  Host pointers;
 * synchronous. */
int tsg_treeseq_divergence_matrix(const tsg_treeseq_t *self, uint64_t num_sample_sets,
    const uint64_t *sample_set_sizes, const int32_t *sample_sets, uint64_t num_windows,
    const double *windows, uint32_t options, double *result);
/* genetic_relatedness_matrix (python/tskit/trees.py:8978-9102, site mode):
 * the divergence matrix followed by the same normalisation, on the device.
 * No C counterpart in the reference (its normalisation is Python code). */
int tsg_treeseq_genetic_relatedness_matrix(const tsg_treeseq_t *self,
    uint64_t num_sample_sets, const uint64_t *sample_set_sizes, const int32_t *sample_sets,
    uint64_t num_windows, const double *windows, uint32_t options, double *result);
/* The derived-allele indicator of every sample at sites [site_start,
 * site_stop) as E4M3 bytes (0x38 when the sample carries a derived allele,
 * else 0x00), one row per sample (G: num_samples x ld bytes, device, column
 * s - site_start for site s; other columns untouched).  Genotypes as the
 * reference's variant decoder gives them with isolated samples ancestral
 * (c/tskit/genotypes.c).  Synchronous on `cuda_stream`. */
int tsg_treeseq_genotype_operand(const tsg_treeseq_t *self, int64_t site_start,
    int64_t site_stop, uint8_t *G, int64_t ld, void *cuda_stream);
/* P = G G^T (int32, upper-triangle 128 x 256 tiles written; P is n x ldp,
 * device) for a device operand G of n rows x ld bytes holding E4M3 0 or 1
 * (0x00 / 0x38), K = k columns (a multiple of 128; ld a multiple of 16).
 * Exact.  Synchronous on `cuda_stream`.  No reference counterpart: the
 * contraction behind the divergence matrix, exposed for testing. */
int tsg_gram_e4m3(const uint8_t *G, int64_t n, int64_t ld, int64_t k, int32_t *P, int64_t ldp,
    void *cuda_stream);

/* ------------------------------------------------------ fused sample-count
 * Generalises tsk_treeseq_sample_count_stat (c/tskit/trees.c:2174-2220) to a
 * list of summary terms evaluated in one sweep.  With TSG_STAT_BOTH_MODES the
 * result holds the branch block (num_windows x num_outputs) followed by the
 * site block.  Host pointers. */
typedef struct {
    int32_t type;   /* TSG_DIVERSITY ... */
    int32_t idx[4]; /* sample-set indexes the term reads */
} tsg_output_t;

int tsg_treeseq_sample_count_stat(const tsg_treeseq_t *self, uint64_t num_sample_sets,
    const uint64_t *sample_set_sizes, const int32_t *sample_sets, uint64_t num_outputs,
    const tsg_output_t *outputs, uint64_t num_windows, const double *windows,
    uint32_t options, double *result);

/* ------------------------------------------- arbitrary summary functions
 * general_stat / sample_count_stat with a caller-supplied summary function
 * (c/tskit/trees.c:2035-2095 with general_stat_func_t; the reference calls
 * it once per state change).  Three steps: prepare runs the sweep for the
 * sample sets (0/1 weights), windows and mode (one of site / branch) and
 * collects the distinct count vectors it meets; states returns them
 * (num_states x num_sample_sets int32); finish takes the summary values at
 * those states (num_states x num_outputs doubles: for branch mode without
 * TSG_STAT_POLARISED, f(x) + f(n - x) as the reference's unpolarised
 * wrapper, trees.c:1944-1972) and writes num_windows x num_outputs. */
typedef struct tsg_general tsg_general_t;
int tsg_general_stat_prepare(tsg_general_t **general, const tsg_treeseq_t *self,
    uint64_t num_sample_sets, const uint64_t *sample_set_sizes, const int32_t *sample_sets,
    uint64_t num_outputs, uint64_t num_windows, const double *windows, uint32_t options,
    int64_t *num_states);
int tsg_general_stat_states(tsg_general_t *general, int32_t *states);
int tsg_general_stat_finish(tsg_general_t *general, const double *values, double *result);
/* Doubles finish writes: num_windows x num_outputs, or num_windows x
 * num_nodes x num_outputs in node mode. */
int64_t tsg_general_stat_result_size(const tsg_general_t *general);
int tsg_general_stat_free(tsg_general_t *general);

/* Replaces tsk_treeseq_general_stat (c/tskit/trees.h:1032-1036,
 * c/tskit/trees.c:2035-2095) with the reference's callback form: same
 * arguments (sample_weights host [num_samples x state_dim] in sample order,
 * f called as f(state_dim, state, result_dim, out, f_params), a non-zero
 * return aborting the call with that value), option bits, default mode
 * (site), default windows (NULL: the whole genome) and errors.  f is called
 * on the host once per state the device sweep lists (each distinct count
 * vector when every weight is 0 or 1, else each state an item, a site allele
 * or a leaf needs), plus at total - state for branch and node mode without
 * TSG_STAT_POLARISED, where the reference calls it once per state change.
 * state_dim <= 32.  result: num_windows x result_dim (x num_nodes before
 * result_dim in node mode). */
typedef int tsg_general_stat_func_t(uint64_t state_dim, const double *state,
    uint64_t result_dim, double *result, void *params);
int tsg_treeseq_general_stat(const tsg_treeseq_t *self, uint64_t state_dim,
    const double *sample_weights, uint64_t result_dim, tsg_general_stat_func_t *f,
    void *f_params, uint64_t num_windows, const double *windows, uint32_t options,
    double *result);

/* general_stat with real-valued weights (tsk_treeseq_general_stat,
 * c/tskit/trees.c:2035-2095, W f64 [n x K] in sample order, K <= 32): the
 * same prepare / states / finish steps, the states being the weights below
 * each node as FP64 vectors.  Every state an item, a site allele or a leaf
 * needs is listed (real states rarely repeat): the host evaluates the
 * summary function on each of the num_states rows of
 * tsg_general_weighted_states and passes the values to
 * tsg_general_stat_finish; tsg_general_stat_free releases. */
int tsg_general_weighted_prepare(tsg_general_t **out, const tsg_treeseq_t *self, uint64_t K,
    const double *weights, uint64_t R, uint64_t num_windows, const double *windows,
    uint32_t options, int64_t *num_states);
int tsg_general_weighted_states(tsg_general_t *g, double *states);

/* Replaces tsk_treeseq_genetic_relatedness_weighted (c/tskit/trees.c:
 * 4838-4897, same arguments; weights host [n x num_weights], num_weights
 * <= 31, index tuples pairs of weight columns, which are range-checked
 * (TSG_ERR_BAD_SAMPLE_SET_INDEX) where the reference reads them unchecked;
 * TSG_STAT_NONCENTRED as the reference's TSK_STAT_NONCENTRED): the weighted
 * replay with the pair summary evaluated on the device. */
int tsg_treeseq_genetic_relatedness_weighted(const tsg_treeseq_t *self, uint64_t num_weights,
    const double *weights, uint64_t num_index_tuples, const int32_t *index_tuples,
    uint64_t num_windows, const double *windows, double *result, uint32_t options);

/* Replaces tsk_treeseq_genealogical_nearest_neighbours (c/tskit/trees.c:
 * 891-1074): the reference sets (any nodes, no node in two sets) flattened
 * with their sizes instead of an array of pointers.  Result num_focal x
 * num_sets. */
int tsg_treeseq_genealogical_nearest_neighbours(const tsg_treeseq_t *self,
    const int32_t *focal, uint64_t num_focal, uint64_t num_sets, const uint64_t *set_sizes,
    const int32_t *sets, uint32_t options, double *result);

/* Replaces tsk_treeseq_mean_descendants (c/tskit/trees.c:1076-1220): the
 * reference sets (any nodes) flattened with their sizes instead of an array
 * of pointers; at most 31 sets.  Result num_nodes x num_sets. */
int tsg_treeseq_mean_descendants(const tsg_treeseq_t *self, uint64_t num_sets,
    const uint64_t *set_sizes, const int32_t *sets, uint32_t options, double *result);

/* Replace tsk_treeseq_trait_covariance / trait_correlation /
 * trait_linear_model (c/tskit/trees.c:3976-4218, same arguments; weights
 * host [n x num_weights], covariates [n x num_covariates] already
 * standardised as the reference's Python layer does; at most 32 columns in
 * all, counting the appended frequency or count column).  Result
 * num_windows x num_weights (x num_nodes before num_weights in node mode). */
int tsg_treeseq_trait_covariance(const tsg_treeseq_t *self, uint64_t num_weights,
    const double *weights, uint64_t num_windows, const double *windows, uint32_t options,
    double *result);
int tsg_treeseq_trait_correlation(const tsg_treeseq_t *self, uint64_t num_weights,
    const double *weights, uint64_t num_windows, const double *windows, uint32_t options,
    double *result);
int tsg_treeseq_trait_linear_model(const tsg_treeseq_t *self, uint64_t num_weights,
    const double *weights, uint64_t num_covariates, const double *covariates,
    uint64_t num_windows, const double *windows, uint32_t options, double *result);

/* ----------------------------------------------- device-resident queries
 * A query is prepared once (validates and uploads sample sets, summary terms
 * and windows) and launched any number of times on a stream with a
 * workspace.  tsg_query_launch enqueues kernels only: the result (device
 * pointer, same layout as tsg_treeseq_sample_count_stat) is ready when the
 * stream reaches that point.  Launches that share a workspace must be
 * ordered on one stream. */
typedef struct tsg_query tsg_query_t;

int tsg_query_create(tsg_query_t **query, const tsg_treeseq_t *self,
    uint64_t num_sample_sets, const uint64_t *sample_set_sizes, const int32_t *sample_sets,
    uint64_t num_outputs, const tsg_output_t *outputs, uint64_t num_windows,
    const double *windows, uint32_t options);
/* The allele frequency spectrum as a device-resident query (result layout as
 * tsg_treeseq_allele_frequency_spectrum). */
int tsg_query_create_afs(tsg_query_t **query, const tsg_treeseq_t *self,
    uint64_t num_sample_sets, const uint64_t *sample_set_sizes, const int32_t *sample_sets,
    uint64_t num_windows, const double *windows, uint64_t num_time_windows,
    const double *time_windows, uint32_t options);
/* The relatedness-vector product as a device-resident query; its weights
 * (device pointer, num_samples x num_weights) are set with
 * tsg_query_set_weights before a launch and read by every later launch. */
int tsg_query_create_relatedness_vector(tsg_query_t **query, const tsg_treeseq_t *self,
    uint64_t num_weights, uint64_t num_windows, const double *windows,
    uint64_t num_focal_nodes, const int32_t *focal_nodes, uint32_t options);
int tsg_query_set_weights(tsg_query_t *query, const double *weights_device);
/* Frees the query's device arrays in stream order (cudaFreeAsync on the
 * legacy default stream), so that freeing never waits for the device: free
 * a query only after its launches have completed (or from a stream ordered
 * after them).  tsg_batch_free does the same for a batch. */
int tsg_query_free(tsg_query_t *query);
/* Device bytes the query needs in a workspace. */
int64_t tsg_query_workspace_bytes(const tsg_query_t *query);
/* Number of result doubles. */
int64_t tsg_query_result_size(const tsg_query_t *query);
int tsg_query_launch(const tsg_query_t *query, tsg_workspace_t *ws, double *result_device,
    void *cuda_stream);
/* Record cudaEvent_t `start_event` / `stop_event` (either may be NULL) on the
 * launch stream immediately before and after the sweep kernel of every later
 * launch of `query`, so callers can time the dominant kernel alone. */
int tsg_query_set_sweep_events(tsg_query_t *query, void *start_event, void *stop_event);
/* The same around the replay kernel alone (the compact replay, or the
 * general replay with its item values) of every later launch: the pipeline's
 * dominant kernel. */
int tsg_query_set_replay_events(tsg_query_t *query, void *start_event, void *stop_event);
/* Synchronous read of the device-side check word left by the last launch of
 * `query` on `ws`: 0, or TSG_ERR_DEVICE_CHECK when a kernel found an
 * inconsistent tree sequence (node id out of range, a cycle). */
int tsg_workspace_check(const tsg_workspace_t *ws, const tsg_query_t *query);

/* Workspaces are device scratch owned by the caller; they grow on demand in
 * tsg_workspace_reserve (which allocates) and never inside a launch. */
int tsg_workspace_create(tsg_workspace_t **ws);
int tsg_workspace_reserve(tsg_workspace_t *ws, int64_t bytes);
int64_t tsg_workspace_bytes(const tsg_workspace_t *ws);
int tsg_workspace_free(tsg_workspace_t *ws);

/* ----------------------------------------------------- batched launches
 * No counterpart in the reference (one call runs one statistic on one tree
 * sequence there).  A batch fuses prepared queries on any resident tree
 * sequences into one launch per pipeline stage: sample-count queries that
 * use the compact replay (tree sequences of up to 65,535 samples, up to 8
 * sample sets, integer site summaries) share each stage's kernel, the replay
 * being one persistent kernel whose blocks take (query, span) items from one
 * counter over all the queries' spans; the other queries launch on their own
 * in the same stream.  Every result is bitwise the result of the query's own
 * launch.
 *   - tsg_batch_workspace_bytes: the workspace the batch needs (the queries'
 *     own workspaces side by side, plus its counters).
 *   - tsg_batch_create binds the queries, one device result pointer each
 *     (layouts as tsg_query_launch) and the workspace; the queries, results
 *     and workspace must outlive the batch.
 *   - tsg_batch_launch enqueues the kernels on the stream (no allocation, no
 *     synchronisation; capturable in a CUDA graph).  Launches of one batch,
 *     or of batches sharing its workspace, must be ordered on one stream.
 *   - tsg_batch_check: synchronous read of every query's check word after a
 *     launch (TSG_ERR_DEVICE_CHECK with the first failing query's index).
 *   - tsg_batch_num_fused: how many of the queries run in the fused kernels. */
typedef struct tsg_batch tsg_batch_t;
int tsg_batch_workspace_bytes(uint64_t num_queries, const tsg_query_t *const *queries,
    int64_t *bytes);
int tsg_batch_create(tsg_batch_t **batch, uint64_t num_queries,
    const tsg_query_t *const *queries, double *const *results, tsg_workspace_t *ws);
int tsg_batch_launch(const tsg_batch_t *batch, void *cuda_stream);
int tsg_batch_check(const tsg_batch_t *batch, uint64_t *failed_query);
int tsg_batch_num_fused(const tsg_batch_t *batch);
void tsg_batch_free(tsg_batch_t *batch);

/* ------------------------------------------ launch without any allocation
 * No counterpart in the reference.  For callers that must not allocate device
 * memory while a query runs -- a host that gives this library a fixed
 * device-memory budget and owns all allocations, or a latency-critical
 * serving path that cannot afford cudaMalloc -- this runs a prepared query
 * (same result as tsg_query_launch) with its scratch in a fixed array that is
 * part of the library's device image: TSG_NOALLOC_SCRATCH_BYTES (32 MiB) on
 * every GPU that loads the library, held until the process exits.  It calls
 * no cudaMalloc, cudaFree or allocating library routine.
 *   - A query whose tsg_query_workspace_bytes exceeds the array is refused
 *     with TSG_ERR_NOALLOC_TOO_LARGE (small tree sequences and few windows
 *     fit; the benchmark-sized workloads need a tsg_workspace_t).
 *   - The first call on a device looks up the array's device address
 *     (cudaGetSymbolAddress, with that device current); make that first call
 *     before any stream capture.
 *   - All calls on a device share the one array and the launch clears what it
 *     needs cleared: calls whose kernels overlap on the GPU (different
 *     streams, or different host threads) race and corrupt each other's
 *     results.  Order them on one stream.
 * tsg_noalloc_check reads the device-side check word of the last
 * no-allocation launch on the current device, whichever query it ran
 * (synchronous; `query` is not used), like tsg_workspace_check: each launch
 * copies its word to a fixed device word when it ends. */
#define TSG_NOALLOC_SCRATCH_BYTES (32u << 20)
int tsg_query_launch_noalloc(const tsg_query_t *query, double *result_device, void *cuda_stream);
int tsg_noalloc_check(const tsg_query_t *query);

/* Number of kernel launches issued by this library since load (counter used
 * by the benchmarks to report launches). */
int64_t tsg_launch_count(void);

/* .trees files.  The container tskit stores its tables in (kastore;
 * replaces the reader behind tsk_table_collection_load, c/tskit/tables.c:
 * 11580-11830, and c/subprojects/kastore/kastore.c): the whole file is read
 * and its layout checked (TSG_ERR_IO, TSG_ERR_FILE_FORMAT,
 * TSG_ERR_FILE_VERSION_TOO_OLD/NEW); tsg_kastore_get finds an item by key:
 * its element type (0..9: int8, uint8, int16, uint16, int32, uint32, int64,
 * uint64, float32, float64), element count and data, valid until
 * tsg_kastore_free (TSG_ERR_REQUIRED_COL_NOT_FOUND when absent).  The
 * Python layer (tskit_gb300.load) maps the table columns. */
/* Edge orders on the device (replaces the index build of
 * tsk_table_collection_build_index, c/tskit/tables.c:11393-11450, and the
 * edge order of tsk_table_collection_sort): permutations of the edges by
 * (time[parent], parent, child, left) (sort_order), (left, time[parent],
 * parent, child) (insertion_order) and (right, -time[parent], -parent,
 * -child) (removal_order), ties in edge-table order.  All pointers are device
 * arrays; an output may be null.  Synchronous on cuda_stream. */
int tsg_edge_orders(int64_t num_edges, const double *edge_left, const double *edge_right,
    const int32_t *edge_parent, const int32_t *edge_child, const double *node_time,
    int32_t *sort_order, int32_t *insertion_order, int32_t *removal_order, void *cuda_stream);

typedef struct tsg_kastore tsg_kastore_t;
int tsg_kastore_open(const char *path, tsg_kastore_t **out);
int tsg_kastore_get(const tsg_kastore_t *k, const char *key, int32_t *type, int64_t *len,
    const void **data);
int tsg_kastore_free(tsg_kastore_t *k);

#ifdef __cplusplus
}
#endif
#endif
