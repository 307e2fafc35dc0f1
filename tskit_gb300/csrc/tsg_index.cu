// Edge orders on the device: the edge table's canonical sort order and the
// two edge indexes a tree sequence needs.
//
// Replaces the index build of tsk_table_collection_build_index
// (c/tskit/tables.c:11393-11450: insertion order by (left, time[parent],
// parent, child), removal order by (right, -time[parent], -parent, -child))
// and the edge order of tsk_table_collection_sort (by (time[parent], parent,
// child, left)).  Each order is a least-significant-first sequence of stable
// radix sorts (CUB) of (key, edge) pairs, one pass per key component, the
// keys mapped to unsigned integers that sort in the components' order
// (IEEE doubles: sign-flipped bits, -0 taken as +0; int32: offset by 2^31;
// descending: bit complement).  Ties keep edge-table order, as the
// reference's sorts do.
#include <cub/device/device_radix_sort.cuh>

#include "tsg_internal.cuh"

namespace tsg {

enum EdgeKey { KEY_LEFT, KEY_RIGHT, KEY_PARENT_TIME, KEY_PARENT, KEY_CHILD };

__device__ __forceinline__ uint64_t order_f64(double x)
{
    // -0 compares equal to +0
    const uint64_t b = (uint64_t) __double_as_longlong(x == 0.0 ? 0.0 : x);
    return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}

__global__ void k_iota(int32_t *p, int64_t n)
{
    for (int64_t i = blockIdx.x * (int64_t) blockDim.x + threadIdx.x; i < n;
         i += (int64_t) gridDim.x * blockDim.x) {
        p[i] = (int32_t) i;
    }
}

// the key component of each edge in the current order
__global__ void k_edge_keys(const int32_t *perm, int64_t n, int which, int desc,
    const double *left, const double *right, const int32_t *parent, const int32_t *child,
    const double *node_time, uint64_t *keys)
{
    for (int64_t i = blockIdx.x * (int64_t) blockDim.x + threadIdx.x; i < n;
         i += (int64_t) gridDim.x * blockDim.x) {
        const int32_t e = perm[i];
        uint64_t k;
        switch (which) {
            case KEY_LEFT: k = order_f64(left[e]); break;
            case KEY_RIGHT: k = order_f64(right[e]); break;
            case KEY_PARENT_TIME: k = order_f64(node_time[parent[e]]); break;
            case KEY_PARENT: k = (uint64_t) ((uint32_t) parent[e] ^ 0x80000000u); break;
            default: k = (uint64_t) ((uint32_t) child[e] ^ 0x80000000u); break;
        }
        if (desc) {
            k = (which == KEY_PARENT || which == KEY_CHILD) ? (~k & 0xffffffffull) : ~k;
        }
        keys[i] = k;
    }
}

}  // namespace tsg

using namespace tsg;

extern "C" int tsg_edge_orders(int64_t num_edges, const double *edge_left,
    const double *edge_right, const int32_t *edge_parent, const int32_t *edge_child,
    const double *node_time, int32_t *sort_order, int32_t *insertion_order,
    int32_t *removal_order, void *cuda_stream)
{
    const int64_t n = num_edges;
    if (n < 0 || n >= ((int64_t) 1 << 31)) {
        return TSG_ERR_BAD_PARAM_VALUE;
    }
    if (n == 0) {
        return 0;
    }
    cudaStream_t st = (cudaStream_t) cuda_stream;
    size_t temp = 0;
    cub::DeviceRadixSort::SortPairs(nullptr, temp, (const uint64_t *) nullptr,
        (uint64_t *) nullptr, (const int32_t *) nullptr, (int32_t *) nullptr, (int) n, 0, 64, st);
    void *buf = nullptr;
    const size_t kb = (size_t) n * 8, pb = (size_t) n * 4;
    const size_t tb = (temp + 255) / 256 * 256;
    if (cudaMalloc(&buf, tb + 2 * kb + 2 * pb) != cudaSuccess) {
        cudaGetLastError();
        return TSG_ERR_NO_MEMORY;
    }
    char *b = (char *) buf;
    void *dtemp = b;
    uint64_t *k0 = (uint64_t *) (b + tb), *k1 = (uint64_t *) (b + tb + kb);
    int32_t *p0 = (int32_t *) (b + tb + 2 * kb), *p1 = (int32_t *) (b + tb + 2 * kb + pb);
    const unsigned grid = (unsigned) std::min<int64_t>((n + 255) / 256, 65535);
    int ret = 0;
    // one order: passes from the least significant component to the most
    auto order = [&](const int *comps, const int *desc, int ncomp, int32_t *out) {
        k_iota<<<grid, 256, 0, st>>>(p0, n);
        g_launches.fetch_add(1, std::memory_order_relaxed);
        for (int c = 0; c < ncomp && ret == 0; c++) {
            k_edge_keys<<<grid, 256, 0, st>>>(p0, n, comps[c], desc[c], edge_left, edge_right,
                edge_parent, edge_child, node_time, k0);
            g_launches.fetch_add(1, std::memory_order_relaxed);
            const int bits = (comps[c] == KEY_PARENT || comps[c] == KEY_CHILD) ? 32 : 64;
            size_t t = temp;
            if (cub::DeviceRadixSort::SortPairs(dtemp, t, k0, k1, p0, p1, (int) n, 0, bits, st)
                != cudaSuccess) {
                ret = TSG_ERR_CUDA;
                break;
            }
            g_launches.fetch_add(1, std::memory_order_relaxed);
            std::swap(p0, p1);
        }
        if (ret == 0 && cudaMemcpyAsync(out, p0, pb, cudaMemcpyDeviceToDevice, st) != cudaSuccess) {
            ret = TSG_ERR_CUDA;
        }
    };
    if (sort_order != nullptr) {
        const int comps[4] = { KEY_LEFT, KEY_CHILD, KEY_PARENT, KEY_PARENT_TIME };
        const int desc[4] = { 0, 0, 0, 0 };
        order(comps, desc, 4, sort_order);
    }
    if (insertion_order != nullptr && ret == 0) {
        const int comps[4] = { KEY_CHILD, KEY_PARENT, KEY_PARENT_TIME, KEY_LEFT };
        const int desc[4] = { 0, 0, 0, 0 };
        order(comps, desc, 4, insertion_order);
    }
    if (removal_order != nullptr && ret == 0) {
        const int comps[4] = { KEY_CHILD, KEY_PARENT, KEY_PARENT_TIME, KEY_RIGHT };
        const int desc[4] = { 1, 1, 1, 0 };
        order(comps, desc, 4, removal_order);
    }
    if (ret == 0 && (cudaGetLastError() != cudaSuccess || cudaStreamSynchronize(st) != cudaSuccess)) {
        ret = TSG_ERR_CUDA;
    }
    cudaFree(buf);
    return ret;
}
