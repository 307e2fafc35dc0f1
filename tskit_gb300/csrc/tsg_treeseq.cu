// Device-resident tree sequence: validation and derived state.
//
// Replaces tsk_treeseq_init (c/tskit/trees.c:455-545) for the statistics
// path.  Everything is computed by kernels from the (device) tables:
//   * samples and the node -> sample index map (trees.c:404-453);
//   * tree breakpoints: the sorted distinct values of {0, L, edge lefts,
//     edge rights}, found by merging the two index-sorted coordinate lists
//     (trees.c:243-359 walks the same boundaries serially);
//   * per-tree ranges into the insertion/removal orders and the site table,
//     which is what tsk_tree_position_t steps through (trees.c:5583-5639);
//   * the span plan: trees are cut into spans of about equal edge-event work
//     and, for every span start b, the list of edges with left <= b < right
//     (the seek state of tsk_tree_position_seek_forward, trees.c:5701-5763).
#include <algorithm>
#include <cerrno>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <set>
#include <tuple>

#include "tsg_internal.cuh"

namespace tsg {

std::atomic<int64_t> g_launches{0};
static std::mutex g_err_mutex;
static std::string g_last_cuda_error;

void set_cuda_error(cudaError_t e, const char *where)
{
    std::lock_guard<std::mutex> lock(g_err_mutex);
    g_last_cuda_error = std::string(where) + ": " + cudaGetErrorString(e);
}

int device_count_sms()
{
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        return 0;
    }
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
        return 0;
    }
    return sms;
}

// Kernel attributes asked for at every query's preparation, answered once
// per device and kernel: the runtime's answers do not change for a loaded
// kernel, and the calls cost far more than a lookup.
static std::mutex g_attr_mutex;
static std::map<std::tuple<int, const void *, int, size_t>, int> g_occupancy;
static std::map<std::pair<int, const void *>, int64_t> g_smem_budget;
static std::set<std::pair<int, const void *>> g_smem_allowed;

int occupancy_blocks(const void *fn, int block, size_t smem)
{
    int dev = 0;
    cudaGetDevice(&dev);
    const auto key = std::make_tuple(dev, fn, block, smem);
    std::lock_guard<std::mutex> lock(g_attr_mutex);
    auto it = g_occupancy.find(key);
    if (it != g_occupancy.end()) {
        return it->second;
    }
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, block, smem) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    g_occupancy[key] = per_sm;
    return per_sm;
}

int64_t kernel_smem_budget(const void *fn)
{
    int dev = 0;
    cudaGetDevice(&dev);
    const auto key = std::make_pair(dev, fn);
    std::lock_guard<std::mutex> lock(g_attr_mutex);
    auto it = g_smem_budget.find(key);
    if (it != g_smem_budget.end()) {
        return it->second;
    }
    int optin = 0;
    cudaFuncAttributes attr;
    if (cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess
        || cudaFuncGetAttributes(&attr, fn) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    const int64_t b = (int64_t) optin - (int64_t) attr.sharedSizeBytes;
    g_smem_budget[key] = b;
    return b;
}

void allow_max_dynamic_smem(const void *fn)
{
    int dev = 0;
    cudaGetDevice(&dev);
    const int64_t budget = kernel_smem_budget(fn);
    std::lock_guard<std::mutex> lock(g_attr_mutex);
    if (g_smem_allowed.insert(std::make_pair(dev, fn)).second) {
        cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) budget);
    }
}

// ------------------------------------------------------------------ scan
static constexpr int SCAN_BLOCK = 1024;
static constexpr int SCAN_ITEMS = 4;
static constexpr int64_t SCAN_TILE = SCAN_BLOCK * SCAN_ITEMS;

__device__ __forceinline__ int64_t block_exclusive_scan(int64_t v, int64_t *smem, int64_t *total)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int64_t x = v;
    for (int o = 1; o < 32; o <<= 1) {
        int64_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) {
            x += y;
        }
    }
    if (lane == 31) {
        smem[warp] = x;
    }
    __syncthreads();
    if (warp == 0) {
        const int nw = blockDim.x >> 5;
        int64_t s = lane < nw ? smem[lane] : 0;
        for (int o = 1; o < 32; o <<= 1) {
            int64_t y = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) {
                s += y;
            }
        }
        if (lane < nw) {
            smem[lane] = s;
        }
    }
    __syncthreads();
    int64_t warp_prefix = warp > 0 ? smem[warp - 1] : 0;
    int64_t incl = x + warp_prefix;
    if (total != nullptr) {
        *total = smem[(blockDim.x >> 5) - 1];
    }
    __syncthreads();
    return incl - v;
}

__global__ void k_scan_tile_sums(const int64_t *in, int64_t n, int64_t *tile_sums)
{
    __shared__ int64_t smem[32];
    const int64_t base = (int64_t) blockIdx.x * SCAN_TILE;
    int64_t s = 0;
    for (int j = 0; j < SCAN_ITEMS; j++) {
        int64_t i = base + (int64_t) threadIdx.x * SCAN_ITEMS + j;
        if (i < n) {
            s += in[i];
        }
    }
    int64_t total;
    block_exclusive_scan(s, smem, &total);
    if (threadIdx.x == 0) {
        tile_sums[blockIdx.x] = total;
    }
}

__global__ void k_scan_tile_offsets(int64_t *tile_sums, int64_t num_tiles)
{
    __shared__ int64_t smem[32];
    int64_t carry = 0;
    for (int64_t base = 0; base < num_tiles; base += blockDim.x) {
        int64_t i = base + threadIdx.x;
        int64_t v = i < num_tiles ? tile_sums[i] : 0;
        int64_t total;
        int64_t ex = block_exclusive_scan(v, smem, &total);
        if (i < num_tiles) {
            tile_sums[i] = carry + ex;
        }
        carry += total;
    }
}

__global__ void k_scan_apply(const int64_t *in, int64_t *out, int64_t n, const int64_t *tile_offsets)
{
    __shared__ int64_t smem[32];
    const int64_t base = (int64_t) blockIdx.x * SCAN_TILE;
    int64_t vals[SCAN_ITEMS];
    int64_t s = 0;
    for (int j = 0; j < SCAN_ITEMS; j++) {
        int64_t i = base + (int64_t) threadIdx.x * SCAN_ITEMS + j;
        vals[j] = i < n ? in[i] : 0;
        s += vals[j];
    }
    int64_t ex = block_exclusive_scan(s, smem, nullptr) + tile_offsets[blockIdx.x];
    for (int j = 0; j < SCAN_ITEMS; j++) {
        int64_t i = base + (int64_t) threadIdx.x * SCAN_ITEMS + j;
        if (i < n) {
            out[i] = ex;
        }
        ex += vals[j];
    }
}

int64_t scan_tmp_elems(int64_t n) { return (n + SCAN_TILE - 1) / SCAN_TILE + 1; }

int scan_exclusive_i64(const int64_t *in, int64_t *out, int64_t n, int64_t *tmp,
    cudaStream_t stream)
{
    if (n <= 0) {
        return 0;
    }
    int64_t tiles = (n + SCAN_TILE - 1) / SCAN_TILE;
    k_scan_tile_sums<<<(unsigned) tiles, SCAN_BLOCK, 0, stream>>>(in, n, tmp);
    TSG_LAUNCHED();
    k_scan_tile_offsets<<<1, SCAN_BLOCK, 0, stream>>>(tmp, tiles);
    TSG_LAUNCHED();
    k_scan_apply<<<(unsigned) tiles, SCAN_BLOCK, 0, stream>>>(in, out, n, tmp);
    TSG_LAUNCHED();
    return 0;
}

// ------------------------------------------------------------ validation
struct RawTables {
    int64_t N, E, S, M;
    double L;
    const double *node_time;
    const uint32_t *node_flags;
    const double *left, *right;
    const int32_t *parent, *child, *I, *O;
    const double *site_pos;
    const int32_t *mut_site, *mut_node, *mut_allele, *mut_alt;
};

__global__ void k_validate_edges(RawTables t, int32_t *err)
{
    for (int64_t e = blockIdx.x * (int64_t) blockDim.x + threadIdx.x; e < t.E;
         e += (int64_t) gridDim.x * blockDim.x) {
        int32_t p = t.parent[e], c = t.child[e];
        if (p < 0 || p >= t.N || c < 0 || c >= t.N) {
            dev_error(err, DEV_NODE_OUT_OF_BOUNDS);
            continue;
        }
        double l = t.left[e], r = t.right[e];
        if (!(l >= 0 && r <= t.L && l < r)) {
            dev_error(err, DEV_BAD_EDGE);
        }
        if (!(t.node_time[p] > t.node_time[c])) {
            dev_error(err, DEV_BAD_TIME_ORDER);
        }
        int32_t a = t.I[e], b = t.O[e];
        if (a < 0 || a >= t.E || b < 0 || b >= t.E) {
            dev_error(err, DEV_UNSORTED_INDEX);
            continue;
        }
        if (e > 0) {
            int32_t a0 = t.I[e - 1], b0 = t.O[e - 1];
            if (a0 < 0 || a0 >= t.E || b0 < 0 || b0 >= t.E) {
                continue;
            }
            if (t.left[a0] > t.left[a] || t.right[b0] > t.right[b]) {
                dev_error(err, DEV_UNSORTED_INDEX);
            }
        }
    }
}

__global__ void k_validate_sites(RawTables t, int32_t *err)
{
    const int64_t stride = (int64_t) gridDim.x * blockDim.x;
    for (int64_t s = blockIdx.x * (int64_t) blockDim.x + threadIdx.x; s < t.S; s += stride) {
        double x = t.site_pos[s];
        if (!(x >= 0 && x < t.L) || (s > 0 && !(t.site_pos[s - 1] < x))) {
            dev_error(err, DEV_BAD_SITE);
        }
    }
    for (int64_t m = blockIdx.x * (int64_t) blockDim.x + threadIdx.x; m < t.M; m += stride) {
        int32_t s = t.mut_site[m], u = t.mut_node[m];
        if (s < 0 || s >= t.S || u < 0 || u >= t.N || t.mut_allele[m] < 0
            || t.mut_alt[m] < 0 || (m > 0 && t.mut_site[m - 1] > s)) {
            dev_error(err, DEV_BAD_MUTATION);
        }
    }
}

// ------------------------------------------------------------ derived state
__global__ void k_gather_index(RawTables t, double *ins_left, double *rem_right,
    int32_t *ins_parent, int32_t *ins_child, int32_t *rem_parent, int32_t *rem_child)
{
    for (int64_t i = blockIdx.x * (int64_t) blockDim.x + threadIdx.x; i < t.E;
         i += (int64_t) gridDim.x * blockDim.x) {
        int32_t a = t.I[i], b = t.O[i];
        ins_left[i] = t.left[a];
        ins_parent[i] = t.parent[a];
        ins_child[i] = t.child[a];
        rem_right[i] = t.right[b];
        rem_parent[i] = t.parent[b];
        rem_child[i] = t.child[b];
    }
}

// Stable merge of the sorted lefts and rights into merged[1 .. 2E], with
// merged[0] = 0 and merged[2E + 1] = L.
__global__ void k_merge_coords(const double *lefts, const double *rights, int64_t E, double L,
    double *merged)
{
    for (int64_t i = blockIdx.x * (int64_t) blockDim.x + threadIdx.x; i < E;
         i += (int64_t) gridDim.x * blockDim.x) {
        double x = lefts[i];
        merged[1 + i + lower_bound(rights, E, x)] = x;
        double y = rights[i];
        merged[1 + i + upper_bound(lefts, E, y)] = y;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        merged[0] = 0.0;
        merged[2 * E + 1] = L;
    }
}

__global__ void k_flag_distinct(const double *a, int64_t n, int64_t *flags)
{
    for (int64_t i = blockIdx.x * (int64_t) blockDim.x + threadIdx.x; i < n;
         i += (int64_t) gridDim.x * blockDim.x) {
        flags[i] = (i == 0 || a[i] != a[i - 1]) ? 1 : 0;
    }
}

__global__ void k_compact_distinct(const double *a, const int64_t *pos, int64_t n, double *out)
{
    for (int64_t i = blockIdx.x * (int64_t) blockDim.x + threadIdx.x; i < n;
         i += (int64_t) gridDim.x * blockDim.x) {
        if (i == 0 || a[i] != a[i - 1]) {
            out[pos[i]] = a[i];
        }
    }
}

// each tree's length, as the window sums difference its ends
__global__ void k_tree_len(const double *bp, int64_t T, double *len)
{
    const int64_t t = blockIdx.x * (int64_t) blockDim.x + threadIdx.x;
    if (t < T) {
        len[t] = bp[t + 1] - bp[t];
    }
}

__global__ void k_tree_ranges(const double *bp, int64_t T, const double *ins_left,
    const double *rem_right, int64_t E, const double *site_pos, int64_t S, int32_t *tree_in,
    int32_t *tree_out, int32_t *tree_sites)
{
    for (int64_t t = blockIdx.x * (int64_t) blockDim.x + threadIdx.x; t <= T;
         t += (int64_t) gridDim.x * blockDim.x) {
        double b = bp[t];
        tree_in[t] = (int32_t) lower_bound(ins_left, E, b);
        tree_out[t] = (int32_t) lower_bound(rem_right, E, b);
        tree_sites[t] = (int32_t) (t == T ? S : lower_bound(site_pos, S, b));
    }
}

__global__ void k_site_mut(const int32_t *mut_site, int64_t M, int64_t S, int32_t *site_mut)
{
    for (int64_t s = blockIdx.x * (int64_t) blockDim.x + threadIdx.x; s <= S;
         s += (int64_t) gridDim.x * blockDim.x) {
        site_mut[s] = (int32_t) lower_bound(mut_site, M, (int32_t) s);
    }
}

__global__ void k_sample_flags(const uint32_t *flags, int64_t N, int64_t *is_sample)
{
    for (int64_t u = blockIdx.x * (int64_t) blockDim.x + threadIdx.x; u < N;
         u += (int64_t) gridDim.x * blockDim.x) {
        is_sample[u] = (flags[u] & 1u) ? 1 : 0;
    }
}

__global__ void k_sample_index(const uint32_t *flags, const int64_t *pos, int64_t N,
    int32_t *sample_index, int32_t *samples)
{
    for (int64_t u = blockIdx.x * (int64_t) blockDim.x + threadIdx.x; u < N;
         u += (int64_t) gridDim.x * blockDim.x) {
        if (flags[u] & 1u) {
            sample_index[u] = (int32_t) pos[u];
            samples[pos[u]] = (int32_t) u;
        } else {
            sample_index[u] = -1;
        }
    }
}

static int grid_for(int64_t n, int block = 256)
{
    int64_t g = (n + block - 1) / block;
    if (g < 1) {
        g = 1;
    }
    if (g > 65535LL * 8) {
        g = 65535LL * 8;
    }
    return (int) g;
}

template <typename T>
static int dev_alloc(tsg_treeseq_t *ts, T **p, int64_t count)
{
    if (count <= 0) {
        count = 1;
    }
    void *q = nullptr;
    TSG_CUDA(cudaMalloc(&q, (size_t) count * sizeof(T)));
    ts->owned.push_back(q);
    *p = (T *) q;
    return 0;
}

template <typename T>
static int upload(tsg_treeseq_t *ts, const T *host, int64_t count, const T **out)
{
    T *d = nullptr;
    int ret = dev_alloc(ts, &d, count);
    if (ret != 0) {
        return ret;
    }
    if (count > 0) {
        TSG_CUDA(cudaMemcpy(d, host, (size_t) count * sizeof(T), cudaMemcpyHostToDevice));
    }
    *out = d;
    return 0;
}

static int map_device_error(int32_t code)
{
    switch (code) {
        case DEV_OK:
            return 0;
        case DEV_NODE_OUT_OF_BOUNDS:
            return TSG_ERR_NODE_OUT_OF_BOUNDS;
        case DEV_BAD_TIME_ORDER:
            return TSG_ERR_BAD_NODE_TIME_ORDERING;
        case DEV_UNSORTED_INDEX:
            return TSG_ERR_TABLES_NOT_INDEXED;
        default:
            return TSG_ERR_BAD_TREE_SEQUENCE;
    }
}

}  // namespace tsg

using namespace tsg;

extern "C" {

const char *tsg_strerror(int err)
{
    switch (err) {
        case 0:
            return "Normal exit condition. This is not an error!";
        case TSG_ERR_GENERIC:
            return "Generic error";
        case TSG_ERR_NO_MEMORY:
            return "Out of memory";
        case TSG_ERR_IO:
            return errno != 0 ? strerror(errno) : "Generic IO error";
        case TSG_ERR_FILE_FORMAT:
            return "File format error. (TSK_ERR_FILE_FORMAT)";
        case TSG_ERR_FILE_VERSION_TOO_OLD:
            return "tskit file version too old. Please upgrade using the 'tskit upgrade' "
                   "command from tskit version<0.6.2. (TSK_ERR_FILE_VERSION_TOO_OLD)";
        case TSG_ERR_FILE_VERSION_TOO_NEW:
            return "tskit file version is too new for this instance. Please upgrade tskit to "
                   "the latest version. (TSK_ERR_FILE_VERSION_TOO_NEW)";
        case TSG_ERR_REQUIRED_COL_NOT_FOUND:
            return "A required column was not found in the file. "
                   "(TSK_ERR_REQUIRED_COL_NOT_FOUND)";
        case TSG_ERR_BOTH_COLUMNS_REQUIRED:
            return "Both columns in a related pair must be provided. "
                   "(TSK_ERR_BOTH_COLUMNS_REQUIRED)";
        case TSG_ERR_BAD_COLUMN_TYPE:
            return "An incompatible type for a column was found in the file. "
                   "(TSK_ERR_BAD_COLUMN_TYPE)";
        case TSG_ERR_BAD_OFFSET:
            return "Bad offset provided in input array. (TSK_ERR_BAD_OFFSET)";
        case TSG_ERR_TIME_NONFINITE:
            return "Times must be finite. (TSK_ERR_TIME_NONFINITE)";
        case TSG_ERR_BAD_PARAM_VALUE:
            return "Bad parameter value provided";
        case TSG_ERR_NODE_OUT_OF_BOUNDS:
            return "Node out of bounds";
        case TSG_ERR_BAD_NODE_TIME_ORDERING:
            return "time[parent] must be greater than time[child]";
        case TSG_ERR_DUPLICATE_SAMPLE:
            return "Duplicate sample value";
        case TSG_ERR_BAD_SAMPLES:
            return "The nodes provided are not samples";
        case TSG_ERR_TABLES_NOT_INDEXED:
            return "Table collection must be indexed";
        case TSG_ERR_BAD_NUM_WINDOWS:
            return "Must have at least one window, [0, L]";
        case TSG_ERR_BAD_WINDOWS:
            return "Windows must be increasing list [0, ..., L]";
        case TSG_ERR_MULTIPLE_STAT_MODES:
            return "Cannot specify more than one stats mode.";
        case TSG_ERR_BAD_STATE_DIMS:
            return "Must have state dimension >= 1";
        case TSG_ERR_BAD_RESULT_DIMS:
            return "Must have result dimension >= 1";
        case TSG_ERR_INSUFFICIENT_SAMPLE_SETS:
            return "Insufficient sample sets provided.";
        case TSG_ERR_INSUFFICIENT_INDEX_TUPLES:
            return "Insufficient sample set index tuples provided.";
        case TSG_ERR_BAD_SAMPLE_SET_INDEX:
            return "Sample set index out of bounds";
        case TSG_ERR_EMPTY_SAMPLE_SET:
            return "Samples cannot be empty";
        case TSG_ERR_UNSUPPORTED_STAT_MODE:
            return "Requested statistics mode not supported for this method.";
        case TSG_ERR_TIME_UNCALIBRATED:
            return "Statistics using branch lengths cannot be calculated when time_units "
                   "is 'uncalibrated'.";
        case TSG_ERR_STAT_POLARISED_UNSUPPORTED:
            return "The TSK_STAT_POLARISED option is not supported by this statistic. "
                   "(TSK_ERR_STAT_POLARISED_UNSUPPORTED)";
        case TSG_ERR_INSUFFICIENT_WEIGHTS:
            return "Insufficient weights provided (at least 1 required).";
        case TSG_ERR_BAD_TIME_WINDOWS_DIM:
            return "Must have at least one time window";
        case TSG_ERR_BAD_TIME_WINDOWS:
            return "Time windows must start at zero and be strictly increasing";
        case TSG_ERR_CUDA:
            return "CUDA error";
        case TSG_ERR_DEVICE_CHECK:
            return "A device-side consistency check failed";
        case TSG_ERR_TOO_MANY_SAMPLE_SETS:
            return "Too many sample sets for the device sweep (maximum 32)";
        case TSG_ERR_TOO_MANY_OUTPUTS:
            return "Too many summary outputs for the device sweep (maximum 64)";
        case TSG_ERR_BAD_TREE_SEQUENCE:
            return "Tables do not describe a valid tree sequence";
        case TSG_ERR_NOALLOC_TOO_LARGE:
            return "Query needs more scratch than the static no-allocation array holds (32 MiB)";
        case TSG_ERR_WORKSPACE_TOO_SMALL:
            return "Workspace too small for this query";
        default:
            return "Unknown error";
    }
}

int64_t tsg_launch_count(void) { return g_launches.load(); }

int tsg_treeseq_free(tsg_treeseq_t *ts)
{
    if (ts == nullptr) {
        return 0;
    }
    for (void *p : ts->owned) {
        cudaFree(p);
    }
    for (void *p : ts->compact_owned) {
        cudaFree(p);
    }
    if (ts->sync_ws != nullptr) {
        tsg_workspace_free(ts->sync_ws);
    }
    cudaFree(ts->stage);
    delete ts;
    return 0;
}

int64_t tsg_treeseq_get_num_trees(const tsg_treeseq_t *ts) { return ts->v.num_trees; }
int64_t tsg_treeseq_get_num_samples(const tsg_treeseq_t *ts) { return ts->v.num_samples; }
int64_t tsg_treeseq_get_num_spans(const tsg_treeseq_t *ts) { return ts->v.num_spans; }
int64_t tsg_treeseq_get_num_compact_spans(const tsg_treeseq_t *ts) { return ts->v.c_num_spans; }

int tsg_treeseq_get_plan_sizes(const tsg_treeseq_t *ts, int64_t *sizes)
{
    if (ts == nullptr || sizes == nullptr) {
        return TSG_ERR_BAD_PARAM_VALUE;
    }
    const bool c = ts->v.c_num_spans > 0;
    sizes[0] = ts->v.num_trees;
    sizes[1] = ts->v.num_spans;
    sizes[2] = ts->v.c_num_spans;
    sizes[3] = c ? ts->h_compact_nodes : 0;
    sizes[4] = c ? ts->h_compact_endpoints : 0;
    sizes[5] = ts->v.num_items;
    sizes[6] = ts->v.num_chunks;
    sizes[7] = c ? ts->v.c_num_anchors : 0;
    return 0;
}

int tsg_treeseq_set_compact_spans(tsg_treeseq_t *ts, int64_t num_spans)
{
    if (ts == nullptr || num_spans < -1) {
        return TSG_ERR_BAD_PARAM_VALUE;
    }
    std::lock_guard<std::mutex> lock(ts->sync_mutex);
    TSG_CUDA(cudaDeviceSynchronize());
    if (num_spans == 0 || ts->v.num_trees < 1) {
        ts->v.c_num_spans = 0;
        return 0;
    }
    if (num_spans < 0) {
        const tsg::HostTopology &h = ts->host;
        const int64_t T = ts->v.num_trees;
        num_spans = tsg::compact_default_spans(T,
            (int64_t) h.tree_in[(size_t) T] + (int64_t) h.tree_out[(size_t) T], ts->v.num_samples);
    }
    return tsg::build_compact_plan(ts, ts->host, std::min<int64_t>(num_spans, ts->v.num_trees));
}

int tsg_treeseq_get_breakpoints(const tsg_treeseq_t *ts, double *bp)
{
    std::memcpy(bp, ts->h_breakpoints.data(), ts->h_breakpoints.size() * sizeof(double));
    return 0;
}

int tsg_treeseq_init(tsg_treeseq_t **out, const tsg_tables_t *tables, int64_t num_spans,
    uint32_t options)
{
    int ret = 0;
    *out = nullptr;
    if (tables == nullptr || !(tables->sequence_length > 0) || tables->num_nodes < 0
        || tables->num_edges < 0 || tables->num_sites < 0 || tables->num_mutations < 0
        || tables->num_nodes > INT32_MAX || tables->num_edges > INT32_MAX / 2) {
        return TSG_ERR_BAD_PARAM_VALUE;
    }
    if (tables->num_edges > 0
        && (tables->edge_insertion_order == nullptr || tables->edge_removal_order == nullptr)) {
        return TSG_ERR_TABLES_NOT_INDEXED;
    }
    tsg_treeseq_t *ts = new tsg_treeseq_t();
    ts->options = options;
    const int64_t N = tables->num_nodes, E = tables->num_edges, S = tables->num_sites,
                  M = tables->num_mutations;
    const double L = tables->sequence_length;
    RawTables t{};
    t.N = N;
    t.E = E;
    t.S = S;
    t.M = M;
    t.L = L;
    int32_t *d_err = nullptr;
    int64_t *tmp = nullptr, *flags = nullptr;
    double *merged = nullptr;
    cudaStream_t st = 0;

    if (options & TSG_TABLES_ON_DEVICE) {
        t.node_time = tables->node_time;
        t.node_flags = tables->node_flags;
        t.left = tables->edge_left;
        t.right = tables->edge_right;
        t.parent = tables->edge_parent;
        t.child = tables->edge_child;
        t.I = tables->edge_insertion_order;
        t.O = tables->edge_removal_order;
        t.site_pos = tables->site_position;
        t.mut_site = tables->mutation_site;
        t.mut_node = tables->mutation_node;
        t.mut_allele = tables->mutation_allele;
        t.mut_alt = tables->mutation_alt_allele;
    } else {
        if ((ret = upload(ts, tables->node_time, N, &t.node_time))
            || (ret = upload(ts, tables->node_flags, N, &t.node_flags))
            || (ret = upload(ts, tables->edge_left, E, &t.left))
            || (ret = upload(ts, tables->edge_right, E, &t.right))
            || (ret = upload(ts, tables->edge_parent, E, &t.parent))
            || (ret = upload(ts, tables->edge_child, E, &t.child))
            || (ret = upload(ts, tables->edge_insertion_order, E, &t.I))
            || (ret = upload(ts, tables->edge_removal_order, E, &t.O))
            || (ret = upload(ts, tables->site_position, S, &t.site_pos))
            || (ret = upload(ts, tables->mutation_site, M, &t.mut_site))
            || (ret = upload(ts, tables->mutation_node, M, &t.mut_node))
            || (ret = upload(ts, tables->mutation_allele, M, &t.mut_allele))
            || (ret = upload(ts, tables->mutation_alt_allele, M, &t.mut_alt))) {
            goto fail;
        }
    }

    // ---- validation
    {
        const int64_t tmp_elems = std::max<int64_t>(2 * E + 2, N) + 64;
        if (cudaMalloc(&d_err, sizeof(int32_t)) != cudaSuccess
            || cudaMalloc(&flags, (size_t) tmp_elems * sizeof(int64_t)) != cudaSuccess
            || cudaMalloc(&tmp, (size_t) scan_tmp_elems(tmp_elems) * sizeof(int64_t))
                   != cudaSuccess
            || cudaMalloc(&merged, (size_t) (2 * E + 2) * sizeof(double)) != cudaSuccess) {
            ret = TSG_ERR_NO_MEMORY;
            goto fail;
        }
        TSG_CUDA(cudaMemsetAsync(d_err, 0, sizeof(int32_t), st));
        if (E > 0) {
            k_validate_edges<<<grid_for(E), 256, 0, st>>>(t, d_err);
            TSG_LAUNCHED();
        }
        if (S > 0 || M > 0) {
            k_validate_sites<<<grid_for(std::max(S, M)), 256, 0, st>>>(t, d_err);
            TSG_LAUNCHED();
        }
        int32_t h_err = 0;
        TSG_CUDA(cudaMemcpy(&h_err, d_err, sizeof(int32_t), cudaMemcpyDeviceToHost));
        if (h_err != 0) {
            ret = map_device_error(h_err);
            goto fail;
        }
    }

    // ---- samples
    {
        int32_t *sample_index = nullptr, *samples = nullptr;
        if ((ret = dev_alloc(ts, &sample_index, N))) {
            goto fail;
        }
        ts->h_node_flags.resize((size_t) N);
        if (N > 0) {
            TSG_CUDA(cudaMemcpy(ts->h_node_flags.data(), t.node_flags, (size_t) N * sizeof(uint32_t),
                cudaMemcpyDeviceToHost));
        }
        int64_t n = 0;
        ts->h_sample_index.assign((size_t) N, -1);
        for (int64_t u = 0; u < N; u++) {
            if (ts->h_node_flags[(size_t) u] & 1u) {
                ts->h_sample_index[(size_t) u] = (int32_t) n++;
            }
        }
        if ((ret = dev_alloc(ts, &samples, n))) {
            goto fail;
        }
        if (N > 0) {
            k_sample_flags<<<grid_for(N), 256, 0, st>>>(t.node_flags, N, flags);
            TSG_LAUNCHED();
            if ((ret = scan_exclusive_i64(flags, flags, N, tmp, st))) {
                goto fail;
            }
            k_sample_index<<<grid_for(N), 256, 0, st>>>(t.node_flags, flags, N, sample_index,
                samples);
            TSG_LAUNCHED();
        }
        ts->v.sample_index = sample_index;
        ts->v.samples = samples;
        ts->v.num_samples = n;
    }

    // ---- index-ordered edge columns and tree breakpoints
    {
        double *ins_left = nullptr, *rem_right = nullptr, *bp = nullptr;
        int32_t *ins_parent = nullptr, *ins_child = nullptr, *rem_parent = nullptr,
                *rem_child = nullptr;
        if ((ret = dev_alloc(ts, &ins_left, E)) || (ret = dev_alloc(ts, &rem_right, E))
            || (ret = dev_alloc(ts, &ins_parent, E)) || (ret = dev_alloc(ts, &ins_child, E))
            || (ret = dev_alloc(ts, &rem_parent, E)) || (ret = dev_alloc(ts, &rem_child, E))) {
            goto fail;
        }
        if (E > 0) {
            k_gather_index<<<grid_for(E), 256, 0, st>>>(t, ins_left, rem_right, ins_parent,
                ins_child, rem_parent, rem_child);
            TSG_LAUNCHED();
            k_merge_coords<<<grid_for(E), 256, 0, st>>>(ins_left, rem_right, E, L, merged);
            TSG_LAUNCHED();
        } else {
            double h2[2] = { 0.0, L };
            TSG_CUDA(cudaMemcpy(merged, h2, sizeof(h2), cudaMemcpyHostToDevice));
        }
        const int64_t nm = 2 * E + 2;
        k_flag_distinct<<<grid_for(nm), 256, 0, st>>>(merged, nm, flags);
        TSG_LAUNCHED();
        // number of distinct values = last exclusive prefix + last flag
        int64_t last_flag = 0;
        TSG_CUDA(cudaMemcpy(&last_flag, flags + nm - 1, sizeof(int64_t), cudaMemcpyDeviceToHost));
        if ((ret = scan_exclusive_i64(flags, flags, nm, tmp, st))) {
            goto fail;
        }
        int64_t last_pos = 0;
        TSG_CUDA(cudaMemcpy(&last_pos, flags + nm - 1, sizeof(int64_t), cudaMemcpyDeviceToHost));
        const int64_t nbp = last_pos + last_flag;
        const int64_t T = nbp - 1;
        if ((ret = dev_alloc(ts, &bp, nbp))) {
            goto fail;
        }
        k_compact_distinct<<<grid_for(nm), 256, 0, st>>>(merged, flags, nm, bp);
        TSG_LAUNCHED();
        ts->h_breakpoints.resize((size_t) nbp);
        TSG_CUDA(cudaMemcpy(ts->h_breakpoints.data(), bp, (size_t) nbp * sizeof(double),
            cudaMemcpyDeviceToHost));

        int32_t *tree_in = nullptr, *tree_out = nullptr, *tree_sites = nullptr,
                *site_mut = nullptr;
        double *tree_len = nullptr;
        if ((ret = dev_alloc(ts, &tree_in, T + 1)) || (ret = dev_alloc(ts, &tree_out, T + 1))
            || (ret = dev_alloc(ts, &tree_sites, T + 1))
            || (ret = dev_alloc(ts, &site_mut, S + 1))
            || (ret = dev_alloc(ts, &tree_len, T > 0 ? T : 1))) {
            goto fail;
        }
        if (T > 0) {
            k_tree_len<<<grid_for(T), 256, 0, st>>>(bp, T, tree_len);
            TSG_LAUNCHED();
        }
        k_tree_ranges<<<grid_for(T + 1), 256, 0, st>>>(bp, T, ins_left, rem_right, E, t.site_pos,
            S, tree_in, tree_out, tree_sites);
        TSG_LAUNCHED();
        k_site_mut<<<grid_for(S + 1), 256, 0, st>>>(t.mut_site, M, S, site_mut);
        TSG_LAUNCHED();

        ts->v.num_nodes = N;
        ts->v.num_edges = E;
        ts->v.num_sites = S;
        ts->v.num_mutations = M;
        ts->v.num_trees = T;
        ts->v.sequence_length = L;
        ts->v.node_time = t.node_time;
        ts->v.breakpoints = bp;
        ts->v.tree_len = tree_len;
        ts->v.tree_in = tree_in;
        ts->v.tree_out = tree_out;
        ts->v.tree_sites = tree_sites;
        ts->v.site_mut = site_mut;
        ts->v.ins_parent = ins_parent;
        ts->v.ins_left = ins_left;
        ts->v.ins_child = ins_child;
        ts->v.rem_parent = rem_parent;
        ts->v.rem_child = rem_child;
        ts->v.site_position = t.site_pos;
        ts->v.mutation_node = t.mut_node;
        ts->v.mutation_allele = t.mut_allele;
        ts->v.mutation_alt = t.mut_alt;

        // ---- span plan (host, deterministic)
        HostTopology h;
        auto d2h = [&](auto &vec, const auto *src, int64_t count) -> int {
            vec.resize((size_t) count);
            if (count > 0) {
                TSG_CUDA(cudaMemcpy(vec.data(), src, (size_t) count * sizeof(vec[0]),
                    cudaMemcpyDeviceToHost));
            }
            return 0;
        };
        if ((ret = d2h(h.left, t.left, E)) || (ret = d2h(h.right, t.right, E))
            || (ret = d2h(h.parent, t.parent, E)) || (ret = d2h(h.child, t.child, E))
            || (ret = d2h(h.ins_parent, ins_parent, E)) || (ret = d2h(h.ins_child, ins_child, E))
            || (ret = d2h(h.rem_parent, rem_parent, E)) || (ret = d2h(h.rem_child, rem_child, E))
            || (ret = d2h(h.ins_edge, t.I, E))
            || (ret = d2h(h.tree_in, tree_in, T + 1)) || (ret = d2h(h.tree_out, tree_out, T + 1))
            || (ret = d2h(h.tree_sites, tree_sites, T + 1))
            || (ret = d2h(h.site_mut, site_mut, S + 1)) || (ret = d2h(h.mut_node, t.mut_node, M))
            || (ret = d2h(h.mut_allele, t.mut_allele, M))
            || (ret = d2h(h.node_time, t.node_time, N))) {
            goto fail;
        }
        if (num_spans <= 0) {
            // default: one span per replay CTA (two per SM), all replayed in
            // one wave: a span's seek touches about two nodes per sample and
            // the spans carry equal edge-event work.  Large trees (more than
            // 30,000 alive edges: node state in global memory, seeks and
            // window outputs of O(samples) per span and weight-column block)
            // take one span per SM.
            const int64_t sms = std::max(device_count_sms(), 1);
            const int64_t alive0 = T > 0 ? (int64_t) (h.tree_in[1] - h.tree_in[0]) : 0;
            num_spans = alive0 > 30000 ? sms : 2 * sms;
            num_spans = std::min<int64_t>(T, num_spans);
        }
        if ((ret = build_span_plan(ts, h, num_spans)) != 0) {
            goto fail;
        }
        {
            const int64_t events = (int64_t) h.tree_in[(size_t) T] + (int64_t) h.tree_out[(size_t) T];
            const int64_t nc = compact_default_spans(T, events, ts->v.num_samples);
            if ((ret = build_compact_plan(ts, h, nc)) != 0) {
                goto fail;
            }
        }
        ts->host = std::move(h);
        if ((ret = d2h(ts->h_site_position, t.site_pos, S)) != 0) {
            goto fail;
        }
    }
    TSG_CUDA(cudaDeviceSynchronize());
    cudaFree(d_err);
    cudaFree(flags);
    cudaFree(tmp);
    cudaFree(merged);
    *out = ts;
    return 0;
fail:
    cudaFree(d_err);
    cudaFree(flags);
    cudaFree(tmp);
    cudaFree(merged);
    tsg_treeseq_free(ts);
    return ret;
}

}  // extern "C"
