// Internal definitions shared by the CUDA translation units.
#pragma once

#include <nvtx3/nvToolsExt.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <atomic>
#include <mutex>
#include <string>
#include <vector>

#include "tskit_gb300.h"

namespace tsg {

extern std::atomic<int64_t> g_launches;
void set_cuda_error(cudaError_t e, const char *where);

#define TSG_CUDA(call)                                                                   \
    do {                                                                                 \
        cudaError_t _e = (call);                                                         \
        if (_e != cudaSuccess) {                                                         \
            ::tsg::set_cuda_error(_e, #call);                                            \
            return TSG_ERR_CUDA;                                                         \
        }                                                                                \
    } while (0)

#define TSG_LAUNCHED()                                                                   \
    do {                                                                                 \
        ::tsg::g_launches.fetch_add(1, std::memory_order_relaxed);                       \
        cudaError_t _e = cudaGetLastError();                                             \
        if (_e != cudaSuccess) {                                                         \
            ::tsg::set_cuda_error(_e, "kernel launch");                                  \
            return TSG_ERR_CUDA;                                                         \
        }                                                                                \
    } while (0)

// Device-side error codes written to a flag word (first writer wins).
enum DeviceError : int32_t {
    DEV_OK = 0,
    DEV_NODE_OUT_OF_BOUNDS = 1,
    DEV_PATH_TOO_LONG = 2,
    DEV_BAD_EDGE = 3,
    DEV_BAD_TIME_ORDER = 4,
    DEV_UNSORTED_INDEX = 5,
    DEV_BAD_SITE = 6,
    DEV_BAD_MUTATION = 7,
    DEV_ITEM_PLAN = 8,
    DEV_AFS_RANGE = 9,
    DEV_WAIT_TIMEOUT = 10,
    DEV_DECODE_MUTS = 11,
};

__device__ __forceinline__ void dev_error(int32_t *flag, int32_t code)
{
    atomicCAS(flag, 0, code);
}

// Smallest index i in [0, n) with a[i] >= x (n if none).
template <typename T>
__host__ __device__ __forceinline__ int64_t lower_bound(const T *a, int64_t n, T x)
{
    int64_t lo = 0, hi = n;
    while (lo < hi) {
        int64_t mid = (lo + hi) >> 1;
        if (a[mid] < x) {
            lo = mid + 1;
        } else {
            hi = mid;
        }
    }
    return lo;
}

// Smallest index i in [0, n) with a[i] > x (n if none).
template <typename T>
__host__ __device__ __forceinline__ int64_t upper_bound(const T *a, int64_t n, T x)
{
    int64_t lo = 0, hi = n;
    while (lo < hi) {
        int64_t mid = (lo + hi) >> 1;
        if (a[mid] <= x) {
            lo = mid + 1;
        } else {
            hi = mid;
        }
    }
    return lo;
}

// Read-only view of a device-resident tree sequence, passed to kernels by value.
struct TSView {
    int64_t num_nodes, num_edges, num_sites, num_mutations, num_samples, num_trees;
    int64_t num_spans;
    double sequence_length;
    const double *node_time;
    const int32_t *sample_index;  // node -> sample index or -1
    const int32_t *samples;       // sample index -> node
    const double *breakpoints;    // num_trees + 1
    const double *tree_len;       // num_trees: breakpoints[t + 1] - breakpoints[t]
    const int32_t *tree_in;       // num_trees + 1: insertion-order offsets
    const int32_t *tree_out;      // num_trees + 1: removal-order offsets
    const int32_t *tree_sites;    // num_trees + 1
    const int32_t *site_mut;      // num_sites + 1
    const int32_t *ins_parent, *ins_child;  // edges in insertion order
    const int32_t *rem_parent, *rem_child;  // edges in removal order
    const double *site_position;
    const int32_t *mutation_node, *mutation_allele, *mutation_alt;
    const int32_t *span_tree;     // num_spans + 1
    const int64_t *span_alive_off;  // num_spans + 1
    const int2 *span_alive;       // (parent, child) alive at each span start, edge order
    const int2 *span_alive_enc;   // same edges, span-local encoding
    const int64_t *span_local_off;  // num_spans + 1: offsets into span_l2g
    const int32_t *span_l2g;      // stateful nodes of each span (global ids)
    const double *span_time;      // their times, in the same order
    const int2 *ins_enc;          // insertion order: (parent, child) span-local encoding
    const int2 *rem_enc;          // removal order: (parent, child) span-local encoding
    const int32_t *mut_enc;       // per mutation: span-local encoding of its node
    int64_t max_local;            // largest number of stateful nodes in a span
    const int64_t *tree_item_off; // num_trees + 1: replay items of each tree
    int64_t num_items;
    const int64_t *chunk_begin;   // evaluation chunks of items (within one tree)
    const int64_t *chunk_end;
    const int4 *tree_ev;          // num_trees: the edge events into each tree (removal
                                  // offset, removals, insertion offset, insertions)
    const int2 *tree_mut;         // num_trees: each tree's mutations [first, end)
    int64_t num_segs;             // window segments: runs of consecutive trees whose
    const int32_t *seg_tree;      // running sums are windowed together (num_segs + 1)
    const int32_t *chunk_tree;    // the tree of each chunk's items
    const int32_t *chunk_span;    // the span whose replay wrote the chunk's items (their
                                  // node ids are that span's local ids)
    const int64_t *tree_chunk_off;  // num_trees + 1: first chunk of each tree
    int64_t num_chunks;
    // the reference allele frequency spectrum's lazy branch accounting
    const uint8_t *node_is_parent;  // per node: a parent in some edge
    const int32_t *leaf_index;    // per node: index among the leaves (never a parent), or -1
    const int32_t *leaves;        // the leaves, by index
    int64_t num_leaves;
    const double *ins_left;       // insertion order: edge left
    const double *ins_right;      // insertion order: edge right
    const double *ins_lu;         // insertion order: the child's last update before the
                                  // insertion (null when always the insertion position)
    // compact replay plan (tsg_cplan.cu; c_num_spans 0 when the tree sequence
    // has none): short spans whose node state holds only the nodes their
    // transitions touch and their mutations' nodes
    int64_t c_num_spans;
    int64_t c_max_local;          // largest compact node set of a span
    const int32_t *c_span_tree;   // c_num_spans + 1
    const int64_t *c_local_off;   // c_num_spans + 2: node sets (the last: the anchors)
    const double *c_time;         // node times, by local id
    const uint16_t *c_par0;       // parent at the span start (local id; 0x7FFF: none)
    const int64_t *c_ep_off;      // c_num_spans + 1
    const int2 *c_ep;             // sample-range endpoints (position, local << 1 | is_end)
    const int32_t *c_ep_chunk;    // c_num_spans x (chunks + 1): per chunk of order rows,
                                  // its first endpoint (within the span's)
    const uint16_t *c_order;      // c_num_spans x compact_order_stride(num_samples): sample
                                  // indexes, depth-first
    const int2 *c_ins_enc;        // insertion order: (parent, child), compact encoding
    const int2 *c_rem_enc;        // removal order: (parent, child), compact encoding
    const int32_t *c_mut_enc;     // per mutation: compact encoding of its node
    const int32_t *c_chunk_span;  // per chunk: the numbering of its items
    const int32_t *c_chunk_order; // the chunks by decreasing item count (evaluation order)
    int64_t c_num_anchors;        // the first tree's items
    const int32_t *c_anchor_par;  // their parents (anchor ids)
    const int2 *c_anchor_range;   // their sample ranges in the first span's order
};

// largest compact node set a span may have (its node state is in shared
// memory); a tree sequence whose plan exceeds it uses the general replay
#define TSG_COMPACT_MAX_LOCAL 4096

// The compact spans' depth-first sample orders are read in rows of 32
// positions, TSG_ROWS_PER_CHUNK rows (one warp's work) to a chunk; an
// endpoint at position x belongs to row x / 32's chunk (the last chunk for
// x = num_samples).  A compact plan's spans (at most 65,535 samples, 2,048
// rows) have at most 32 chunks.
#define TSG_ROWS_PER_CHUNK 64
// entries of one span's order in the plan: the samples, padded to a
// multiple of 8 (each span's order starts 16-byte aligned)
__host__ __device__ __forceinline__ int64_t compact_order_stride(int64_t n)
{
    return (n + 7) & ~(int64_t) 7;
}
__host__ __device__ __forceinline__ int64_t compact_row_chunks(int64_t n)
{
    const int64_t c = ((n + 31) / 32 + TSG_ROWS_PER_CHUNK - 1) / TSG_ROWS_PER_CHUNK;
    return c > 0 ? c : 1;
}
__host__ __device__ __forceinline__ int64_t compact_chunk_of(int64_t x, int64_t n)
{
    const int64_t c = (x >> 5) / TSG_ROWS_PER_CHUNK, last = compact_row_chunks(n) - 1;
    return c < last ? c : last;
}

// items per evaluation chunk (one warp)
#define TSG_ITEM_CHUNK 256
// nodes one touch list of the item replay holds (a transition touching more
// stateful nodes closes the list and opens another); the span plan counts
// items with the same rule.  Transitions touch a few dozen nodes, and the
// list's shared memory (16 bytes a node) bounds how many compact replays an
// SM holds at once.
#define TSG_TOUCH_CAP 64

// Host copies of the topology the span plan is built from.
struct HostTopology {
    std::vector<double> left, right;           // edge order
    std::vector<int32_t> parent, child;        // edge order
    std::vector<int32_t> ins_parent, ins_child, rem_parent, rem_child;  // index orders
    std::vector<int32_t> ins_edge;             // insertion order (edge ids)
    std::vector<int32_t> tree_in, tree_out, tree_sites;  // num_trees + 1
    std::vector<int32_t> site_mut;             // num_sites + 1
    std::vector<int32_t> mut_node;             // num_mutations
    std::vector<int32_t> mut_allele;           // num_mutations: allele codes
    std::vector<double> node_time;             // num_nodes
};



// Device-wide exclusive scan of int64 values (in may alias out).  `tmp` must
// hold scan_tmp_elems(n) int64.
int64_t scan_tmp_elems(int64_t n);
int scan_exclusive_i64(const int64_t *in, int64_t *out, int64_t n, int64_t *tmp,
    cudaStream_t stream);

int device_count_sms();

// Host-side phase ranges for timeline tools (NVTX; nothing happens unless a
// tool is attached): the enqueue of a launch's seek + replay, evaluation,
// window and site stages, a query's preparation, a Gram.
struct NvtxRange {
    explicit NvtxRange(const char *name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange &) = delete;
    NvtxRange &operator=(const NvtxRange &) = delete;
};
// per device and kernel, asked of the runtime once: resident blocks per SM
// at a block size and dynamic shared memory, the dynamic shared memory a
// block may have (opt-in maximum less static), and that maximum allowed
int occupancy_blocks(const void *fn, int block, size_t smem);
int64_t kernel_smem_budget(const void *fn);
void allow_max_dynamic_smem(const void *fn);

}  // namespace tsg

struct tsg_treeseq;
namespace tsg {
int build_span_plan(tsg_treeseq *ts, const HostTopology &h, int64_t num_spans);
int build_compact_plan(tsg_treeseq *ts, const HostTopology &h, int64_t num_spans);
int64_t compact_default_spans(int64_t T, int64_t events, int64_t n);
}

// Opaque handle definitions.
struct tsg_treeseq {
    tsg::TSView v;
    uint32_t options;
    // host copies of small derived arrays
    std::vector<double> h_breakpoints;
    std::vector<int32_t> h_span_tree;
    std::vector<int32_t> h_seg_tree;
    std::vector<uint32_t> h_node_flags;
    std::vector<int32_t> h_sample_index;
    std::vector<int64_t> h_local_off;
    std::vector<double> h_site_position;
    int64_t max_alive;
    int64_t max_children = 0;  // most children of a node in any span's seek tree
    int64_t h_tree_item0 = 0;  // the first tree's items
    std::vector<int64_t> h_tree_chunk_off;  // num_trees + 1: first chunk of each tree
    std::vector<int32_t> h_chunk_items;     // items of each evaluation chunk
    int64_t h_compact_nodes = 0;            // compact plan: nodes over all spans
    int64_t h_compact_endpoints = 0;        // compact plan: sample-range endpoints
    tsg::HostTopology host;    // host copy of the topology (span plan, genotype decoding)
    // device allocations owned by this object
    std::vector<void *> owned;
    std::vector<void *> compact_owned;  // the compact plan's (rebuilt on demand)
    // state of the synchronous (host-pointer) entry points
    std::mutex sync_mutex;
    tsg_workspace *sync_ws = nullptr;
    void *stage = nullptr;
    int64_t stage_bytes = 0;
    cudaStream_t sync_stream = nullptr;
};

struct tsg_workspace {
    void *ptr;
    int64_t bytes;
    // side streams and events for a launch's independent stages (made by
    // tsg_workspace_create; null in descriptors made otherwise, whose
    // launches run on the caller's stream alone)
    cudaStream_t aux[2];
    cudaEvent_t ev[6];
};

namespace tsg {
// Upload a host vector into a device allocation recorded in `owner`.
template <typename T>
int upload_host_vec(std::vector<void *> &owner, const std::vector<T> &h, T **out)
{
    void *d = nullptr;
    const size_t bytes = std::max<size_t>(h.size(), 1) * sizeof(T);
    TSG_CUDA(cudaMalloc(&d, bytes));
    owner.push_back(d);
    if (!h.empty()) {
        TSG_CUDA(cudaMemcpy(d, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice));
    }
    *out = (T *) d;
    return 0;
}
}  // namespace tsg
