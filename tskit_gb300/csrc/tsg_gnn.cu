// Genealogical nearest neighbours on the GPU.
//
// Replaces tsk_treeseq_genealogical_nearest_neighbours (c/tskit/trees.c:
// 891-1074): for every focal node and tree, the smallest subtree above the
// focal node that holds a reference node other than itself; the reference
// sets' shares of that subtree (the focal node left out of its own set),
// weighted by the tree's span, averaged over the trees where such a subtree
// exists.
//
// One CTA per span of the tree sequence's span plan.  The CTA keeps the
// parent pointers and the per-set reference counts of every node in its own
// global slot: the span's first tree is built from its alive edges in edge
// order (a parent's time never precedes its child's, so adding each child's
// counts to its parent completes every subtree), later trees by the
// reference's root-path updates (one thread; a handful of events per tree).
// Per tree every thread takes focal nodes, walks up to the first ancestor
// whose union count exceeds the focal node's own membership and adds that
// node's counts times span / (count - own) to its per-span partial.  The
// partials are summed over spans in span order and divided by each focal
// node's total span (k_gnn_reduce), so the result is deterministic.
#include <algorithm>
#include <mutex>
#include <vector>

#include "tsg_internal.cuh"

namespace tsg {

// counts: N x K per CTA (K - 1 sets and their union); part: spans x F x
// (K - 1) partial sums and spans x F partial lengths
__global__ void __launch_bounds__(256) k_gnn_spans(TSView ts, int32_t K, const uint32_t *ref,
    const int16_t *set_of, const int32_t *focal, int32_t F, int32_t *gpar, uint32_t *gcnt,
    double *part, double *plen, int32_t *err)
{
    const int64_t N = ts.num_nodes;
    const int s = blockIdx.x;
    if (s >= ts.num_spans) {
        return;
    }
    int32_t *par = gpar + (int64_t) blockIdx.x * N;
    uint32_t *cnt = gcnt + (int64_t) blockIdx.x * N * K;
    const int tid = threadIdx.x, bd = blockDim.x;
    const int KS = K - 1;
    for (int64_t u = tid; u < N; u += bd) {
        par[u] = -1;
        for (int k = 0; k < K; k++) {
            cnt[u * K + k] = ref[u * K + k];
        }
    }
    double *A = part + (int64_t) s * F * KS;
    double *len = plen + (int64_t) s * F;
    for (int64_t i = tid; i < (int64_t) F * KS; i += bd) {
        A[i] = 0.0;
    }
    for (int64_t i = tid; i < F; i += bd) {
        len[i] = 0.0;
    }
    __syncthreads();
    const int32_t t0 = ts.span_tree[s], t1 = ts.span_tree[s + 1];
    // the first tree: alive edges in edge order, children complete before
    // their parents take them
    if (tid == 0) {
        for (int64_t i = ts.span_alive_off[s]; i < ts.span_alive_off[s + 1]; i++) {
            const int2 pc = ts.span_alive[i];
            par[pc.y] = pc.x;
            for (int k = 0; k < K; k++) {
                cnt[(int64_t) pc.x * K + k] += cnt[(int64_t) pc.y * K + k];
            }
        }
    }
    __syncthreads();
    for (int32_t t = t0; t < t1; t++) {
        if (t > t0 && tid == 0) {
            // removals, then insertions, each along the parent's root path
            // (c/tskit/trees.c:959-986)
            for (int pass = 0; pass < 2; pass++) {
                const int32_t a = pass == 0 ? ts.tree_out[t] : ts.tree_in[t];
                const int32_t b = pass == 0 ? ts.tree_out[t + 1] : ts.tree_in[t + 1];
                for (int32_t i = a; i < b; i++) {
                    const int32_t c = pass == 0 ? ts.rem_child[i] : ts.ins_child[i];
                    const int32_t p = pass == 0 ? ts.rem_parent[i] : ts.ins_parent[i];
                    par[c] = pass == 0 ? -1 : p;
                    int64_t steps = 0;
                    for (int32_t v = p; v >= 0; v = par[v]) {
                        if (++steps > N) {
                            dev_error(err, DEV_PATH_TOO_LONG);
                            break;
                        }
                        for (int k = 0; k < K; k++) {
                            if (pass == 0) {
                                cnt[(int64_t) v * K + k] -= cnt[(int64_t) c * K + k];
                            } else {
                                cnt[(int64_t) v * K + k] += cnt[(int64_t) c * K + k];
                            }
                        }
                    }
                }
            }
        }
        __syncthreads();
        const double tree_length = ts.breakpoints[t + 1] - ts.breakpoints[t];
        for (int32_t j = tid; j < F; j += bd) {
            const int32_t u = focal[j];
            const int16_t fs = set_of[u];
            const uint32_t delta = fs >= 0 ? 1u : 0u;
            int32_t p = u;
            uint32_t total = 0;
            int64_t steps = 0;
            while (p >= 0) {
                total = cnt[(int64_t) p * K + KS];
                if (total > delta) {
                    break;
                }
                p = par[p];
                if (++steps > N) {
                    dev_error(err, DEV_PATH_TOO_LONG);
                    p = -1;
                }
            }
            if (p >= 0) {
                len[j] += tree_length;
                const double scale = tree_length / (double) (total - delta);
                for (int k = 0; k < KS; k++) {
                    A[(int64_t) j * KS + k] += (double) cnt[(int64_t) p * K + k] * scale;
                }
                if (fs >= 0) {
                    A[(int64_t) j * KS + fs] -= scale;
                }
            }
        }
        __syncthreads();
    }
}

// the spans' partials summed in span order, divided by each focal node's
// total span (c/tskit/trees.c:1049-1058)
__global__ void k_gnn_reduce(const double *part, const double *plen, int64_t S, int32_t F,
    int32_t KS, double *out)
{
    for (int64_t i = blockIdx.x * (int64_t) blockDim.x + threadIdx.x; i < (int64_t) F * KS;
         i += (int64_t) gridDim.x * blockDim.x) {
        const int64_t j = i / KS;
        double a = 0.0, l = 0.0;
        for (int64_t s = 0; s < S; s++) {
            a += part[s * F * KS + i];
            l += plen[s * F + j];
        }
        out[i] = l > 0 ? a / l : a;
    }
}

}  // namespace tsg

using namespace tsg;

extern "C" int tsg_treeseq_genealogical_nearest_neighbours(const tsg_treeseq_t *self,
    const int32_t *focal, uint64_t num_focal, uint64_t num_sets, const uint64_t *set_sizes,
    const int32_t *sets, uint32_t options, double *result)
{
    (void) options;
    const TSView &v = self->v;
    const int64_t N = v.num_nodes, F = (int64_t) num_focal, S = v.num_spans;
    if (num_sets == 0 || num_sets > 32766) {
        return TSG_ERR_BAD_PARAM_VALUE;
    }
    const int32_t KS = (int32_t) num_sets, K = KS + 1;
    std::vector<uint32_t> ref((size_t) (N * K), 0u);
    std::vector<int16_t> set_of((size_t) std::max<int64_t>(N, 1), (int16_t) -1);
    for (uint64_t k = 0, j = 0; k < num_sets; k++) {
        for (uint64_t l = 0; l < set_sizes[k]; l++, j++) {
            const int32_t u = sets[j];
            if (u < 0 || u >= N) {
                return TSG_ERR_NODE_OUT_OF_BOUNDS;
            }
            if (set_of[(size_t) u] != -1) {
                return TSG_ERR_DUPLICATE_SAMPLE;
            }
            set_of[(size_t) u] = (int16_t) k;
            ref[(size_t) ((int64_t) u * K + (int64_t) k)] = 1u;
            ref[(size_t) ((int64_t) u * K + KS)] = 1u;
        }
    }
    for (int64_t j = 0; j < F; j++) {
        if (focal[j] < 0 || focal[j] >= N) {
            return TSG_ERR_NODE_OUT_OF_BOUNDS;
        }
    }
    if (F == 0) {
        return 0;
    }
    // one allocation: reference counts, set map, focal list, per-CTA parent
    // pointers and counts, span partials, result, error word
    int64_t off = 0;
    auto take = [&](int64_t bytes) {
        const int64_t o = off;
        off += (std::max<int64_t>(bytes, 8) + 255) / 256 * 256;
        return o;
    };
    const int64_t oR = take(N * K * 4), oM = take(N * 2), oF = take(F * 4);
    const int64_t oP = take(S * N * 4), oC = take(S * N * K * 4);
    const int64_t oA = take(S * F * KS * 8), oL = take(S * F * 8), oO = take(F * KS * 8);
    const int64_t oE = take(8);
    void *buf = nullptr;
    if (cudaMalloc(&buf, (size_t) off) != cudaSuccess) {
        cudaGetLastError();
        return TSG_ERR_NO_MEMORY;
    }
    char *b = (char *) buf;
    tsg_treeseq_t *mts = const_cast<tsg_treeseq_t *>(self);
    std::lock_guard<std::mutex> lock(mts->sync_mutex);
    cudaStream_t st = self->sync_stream;
    int ret = 0;
    int32_t herr = 0;
    if (cudaMemcpyAsync(b + oR, ref.data(), (size_t) (N * K * 4), cudaMemcpyHostToDevice, st)
            != cudaSuccess
        || cudaMemcpyAsync(b + oM, set_of.data(), (size_t) (N * 2), cudaMemcpyHostToDevice, st)
            != cudaSuccess
        || cudaMemcpyAsync(b + oF, focal, (size_t) (F * 4), cudaMemcpyHostToDevice, st)
            != cudaSuccess
        || cudaMemsetAsync(b + oE, 0, 8, st) != cudaSuccess) {
        ret = TSG_ERR_CUDA;
    }
    if (ret == 0) {
        k_gnn_spans<<<(unsigned) S, 256, 0, st>>>(v, K, (const uint32_t *) (b + oR),
            (const int16_t *) (b + oM), (const int32_t *) (b + oF), (int32_t) F,
            (int32_t *) (b + oP), (uint32_t *) (b + oC), (double *) (b + oA),
            (double *) (b + oL), (int32_t *) (b + oE));
        g_launches.fetch_add(1, std::memory_order_relaxed);
        const int64_t n = F * KS;
        k_gnn_reduce<<<(unsigned) std::min<int64_t>((n + 255) / 256, 65535), 256, 0, st>>>(
            (const double *) (b + oA), (const double *) (b + oL), S, (int32_t) F, KS,
            (double *) (b + oO));
        g_launches.fetch_add(1, std::memory_order_relaxed);
        if (cudaGetLastError() != cudaSuccess
            || cudaMemcpyAsync(result, b + oO, (size_t) (F * KS * 8), cudaMemcpyDeviceToHost, st)
                != cudaSuccess
            || cudaMemcpyAsync(&herr, b + oE, 4, cudaMemcpyDeviceToHost, st) != cudaSuccess
            || cudaStreamSynchronize(st) != cudaSuccess) {
            ret = TSG_ERR_CUDA;
        }
    }
    cudaFree(buf);
    if (ret == 0 && herr != 0) {
        ret = TSG_ERR_DEVICE_CHECK;
    }
    return ret;
}
