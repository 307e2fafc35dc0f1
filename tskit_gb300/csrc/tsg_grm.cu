// Site-mode divergence matrix and genetic relatedness matrix through an
// exact Gram matrix on the tensor cores (branch mode: k_divmat_branch, pair
// path lengths tree by tree).
//
// Replaces tsk_treeseq_divergence_matrix in site mode
// (c/tskit/trees.c:8753-8899, 8900-9001: D[u][v] counts, over the sites of a
// window, the sample pairs carrying different alleles) and the Python-level
// normalisation of genetic_relatedness_matrix (python/tskit/trees.py:
// 9072-9102).  For one sample per set, with X_any[s][j] = 1 when sample j
// carries a derived allele at site s and Y_a the indicator of allele a,
//   [g_j != g_k] = 1 - sum_a Y_a[j] Y_a[k], hence
//   D = r 1^T + 1 r^T - X_any^T X_any - Z^T Z,   r_j = sum_s X_any[s][j],
// where Z stacks the derived-allele indicators.  At biallelic sites
// Z = X_any, so D = r 1^T + 1 r^T - 2 Xb^T Xb - (X_any^T X_any + Z^T Z) over
// the multiallelic sites.  Both products run on tcgen05 (tsg_gram.cu) in exact
// integers; sets of several samples sum the per-sample entries.
//
// Genotypes: decoded on the device (k_decode_genotypes: one CTA per span,
// parent pointers replayed edge by edge, each sample's root path matched
// against the tree's mutation nodes; isolated samples take the ancestral
// allele, c/tskit/trees.c:8775-8818), written site-major, then transposed on
// the GPU into the K-contiguous E4M3 operands (128-column segments per
// window).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>
#include <thread>
#include <vector>

#include "tsg_internal.cuh"

namespace tsg {

int gram_tiles(int64_t n, std::vector<int32_t> &out);
int launch_gram(const uint8_t *G, int64_t n, int64_t ld, int64_t k0, int64_t kcols,
    const int32_t *tiles, int64_t num_tiles, int32_t multiplier, bool accumulate, int32_t *P,
    int64_t ldp, int32_t *err, cudaStream_t st);

static int64_t up128(int64_t v) { return (v + 127) / 128 * 128; }

#define TSG_DECODE_MUTS 256

// Genotypes on the device: allele codes of every sample (site-major rows of
// n bytes, in sample-index order) for the sites [s0, s1).  One CTA per span
// at a time: the parents of the span's stateful nodes and of the leaves live
// in a per-CTA global slot, rebuilt at the span start from its alive edges
// and updated edge by edge.  At every tree holding sites, each thread walks
// its samples' root paths against the tree's mutation nodes: a sample takes,
// per site, the allele of the last mutation (in the site's order) at the
// deepest of the site's mutation nodes on its path -- the decoding of
// c/tskit/genotypes.c and trees.c:8775-8818, where a later mutation below an
// earlier one overrides it -- and the ancestral allele 0 without one.
__global__ void __launch_bounds__(512) k_decode_genotypes(TSView ts, int64_t s0, int64_t s1,
    uint8_t *A, int32_t *slots, int64_t slot_words, int32_t *err)
{
    __shared__ int32_t s_enc[TSG_DECODE_MUTS];
    __shared__ int16_t s_site[TSG_DECODE_MUTS];
    __shared__ uint8_t s_allele[TSG_DECODE_MUTS];
    const int64_t n = ts.num_samples, nL = ts.num_leaves;
    const int tid = threadIdx.x, bd = blockDim.x;
    int32_t *par = slots + (int64_t) blockIdx.x * slot_words;  // max_local
    int32_t *lpar = par + ts.max_local;                         // leaves
    int32_t *gmap = lpar + nL;                                  // nodes
    for (int64_t s = blockIdx.x; s < ts.num_spans; s += gridDim.x) {
        const int32_t t0 = ts.span_tree[s], t1 = ts.span_tree[s + 1];
        if (ts.tree_sites[t1] <= s0 || ts.tree_sites[t0] >= s1) {
            continue;
        }
        const int64_t lo = ts.span_local_off[s];
        const int32_t Ls = (int32_t) (ts.span_local_off[s + 1] - lo);
        const int32_t *l2g = ts.span_l2g + lo;
        for (int32_t l = tid; l < Ls; l += bd) {
            par[l] = -1;
            gmap[l2g[l]] = l;
        }
        for (int64_t li = tid; li < nL; li += bd) {
            lpar[li] = -1;
        }
        __syncthreads();
        auto set_parent = [&](int32_t c, int32_t p) {
            if (c >= 0) {
                par[c] = p;
            } else {
                lpar[ts.leaf_index[-c - 1]] = p;
            }
        };
        for (int64_t i = ts.span_alive_off[s] + tid; i < ts.span_alive_off[s + 1]; i += bd) {
            const int2 pc = ts.span_alive_enc[i];
            set_parent(pc.y, pc.x);
        }
        __syncthreads();
        for (int32_t t = t0; t < t1; t++) {
            if (t > t0) {
                // removals, then insertions: one event per child in each
                for (int32_t i = ts.tree_out[t] + tid; i < ts.tree_out[t + 1]; i += bd) {
                    set_parent(ts.rem_enc[i].y, -1);
                }
                __syncthreads();
                for (int32_t i = ts.tree_in[t] + tid; i < ts.tree_in[t + 1]; i += bd) {
                    const int2 pc = ts.ins_enc[i];
                    set_parent(pc.y, pc.x);
                }
                __syncthreads();
            }
            int32_t sa = (int32_t) max((int64_t) ts.tree_sites[t], s0);
            const int32_t sb = (int32_t) min((int64_t) ts.tree_sites[t + 1], s1);
            while (sa < sb) {
                // a batch of at most 32 sites whose mutations fit the list
                const int32_t mb = ts.site_mut[sa];
                int32_t se = sa + 1;
                while (se < sb && se - sa < 32 && ts.site_mut[se + 1] - mb <= TSG_DECODE_MUTS) {
                    se++;
                }
                const int32_t nm = ts.site_mut[se] - mb;
                if (nm > TSG_DECODE_MUTS) {
                    if (tid == 0) {
                        dev_error(err, DEV_DECODE_MUTS);
                    }
                    break;
                }
                for (int32_t k = tid; k < nm; k += bd) {
                    const int32_t m = mb + k;
                    int32_t si = sa;
                    while (ts.site_mut[si + 1] <= m) {
                        si++;
                    }
                    s_enc[k] = ts.mut_enc[m];
                    s_site[k] = (int16_t) (si - sa);
                    s_allele[k] = (uint8_t) ts.mutation_allele[m];
                }
                __syncthreads();
                const int32_t nsb = se - sa;
                for (int64_t j = tid; j < n; j += bd) {
                    const int32_t g = ts.samples[j];
                    int32_t e = -(g + 1), p = -1;
                    const int32_t li = ts.leaf_index[g];
                    if (li >= 0) {
                        p = lpar[li];
                    } else {
                        const int32_t l = gmap[g];
                        if (l >= 0 && l < Ls && l2g[l] == g) {
                            e = l;
                            p = par[l];
                        }
                    }
                    uint32_t found = 0;
                    for (int32_t guard = 0;; guard++) {
                        uint32_t here = 0;
                        for (int32_t k = 0; k < nm; k++) {
                            const uint32_t bit = 1u << s_site[k];
                            if (s_enc[k] == e && !(found & bit)) {
                                A[(int64_t) (sa + s_site[k] - s0) * n + j] = s_allele[k];
                                here |= bit;
                            }
                        }
                        found |= here;
                        if (p < 0 || guard > Ls) {
                            break;
                        }
                        e = p;
                        p = par[p];
                    }
                    for (int32_t k = 0; k < nsb; k++) {
                        if (!((found >> k) & 1u)) {
                            A[(int64_t) (sa + k - s0) * n + j] = 0;
                        }
                    }
                }
                __syncthreads();
                sa = se;
            }
        }
        __syncthreads();
    }
}

// Run the device decoder for sites [s0, s1) into dA (ns x n bytes).
static int decode_genotypes_device(const tsg_treeseq_t *ts, int64_t s0, int64_t s1, uint8_t *dA,
    cudaStream_t st)
{
    const TSView &v = ts->v;
    if (s1 <= s0) {
        return 0;
    }
    const int64_t words = std::max<int64_t>(v.max_local, 1) + v.num_leaves + v.num_nodes;
    const int64_t grid = std::max<int64_t>(1, std::min<int64_t>(v.num_spans,
        2 * (int64_t) std::max(device_count_sms(), 1)));
    int32_t *slots = nullptr, *derr = nullptr;
    if (cudaMalloc(&slots, (size_t) (grid * words * 4)) != cudaSuccess
        || cudaMalloc(&derr, 4) != cudaSuccess) {
        cudaGetLastError();
        cudaFree(slots);
        return TSG_ERR_NO_MEMORY;
    }
    int ret = 0;
    int32_t herr = 0;
    if (cudaMemsetAsync(derr, 0, 4, st) != cudaSuccess) {
        ret = TSG_ERR_CUDA;
    } else {
        k_decode_genotypes<<<(unsigned) grid, 512, 0, st>>>(v, s0, s1, dA, slots, words, derr);
        g_launches.fetch_add(1, std::memory_order_relaxed);
        if (cudaGetLastError() != cudaSuccess
            || cudaMemcpyAsync(&herr, derr, 4, cudaMemcpyDeviceToHost, st) != cudaSuccess
            || cudaStreamSynchronize(st) != cudaSuccess) {
            ret = TSG_ERR_CUDA;
        } else if (herr != 0) {
            ret = TSG_ERR_DEVICE_CHECK;
        }
    }
    cudaFree(slots);
    cudaFree(derr);
    return ret;
}

// Largest allele code of the sites [s0, s1) (the decoder stores codes in a
// byte: larger ones are refused).
static int site_max_allele(const tsg_treeseq_t *ts, int64_t s0, int64_t s1, int *max_allele)
{
    const HostTopology &h = ts->host;
    int mx = 0;
    if (s1 > s0) {
        for (int32_t m = h.site_mut[(size_t) s0]; m < h.site_mut[(size_t) s1]; m++) {
            const int32_t a = h.mut_allele[(size_t) m];
            if (a < 0 || a > 255) {
                return TSG_ERR_BAD_PARAM_VALUE;
            }
            mx = std::max(mx, a);
        }
    }
    *max_allele = mx;
    return 0;
}

// Biallelic sites: Gb[j][kb[s]] = E4M3(1) where sample j carries the derived
// allele (32 x 32 tiles through shared memory; kb[s] < 0 skips the site).
__global__ void k_pack_biallelic(const uint8_t *A, int64_t S, int64_t n, const int64_t *kb,
    uint8_t *Gb, int64_t ldb)
{
    __shared__ uint8_t tile[32][33];
    const int64_t s0 = (int64_t) blockIdx.x * 32, j0 = (int64_t) blockIdx.y * 32;
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;  // 32 x 8 threads
    for (int r = ty; r < 32; r += 8) {
        const int64_t s = s0 + r, j = j0 + tx;
        tile[r][tx] = (s < S && j < n) ? A[s * n + j] : 0;
    }
    __syncthreads();
    for (int r = ty; r < 32; r += 8) {
        const int64_t j = j0 + r, s = s0 + tx;
        if (j < n && s < S) {
            const int64_t k = kb[s];
            if (k >= 0) {
                Gb[j * ldb + k] = tile[tx][r] != 0 ? (uint8_t) 0x38 : (uint8_t) 0;
            }
        }
    }
}

// Multiallelic sites: rows km[s] (derived at all) and km[s] + a (allele a).
__global__ void k_pack_multi(const uint8_t *A, int64_t n, const int32_t *msites,
    const int64_t *km, const int32_t *nall, int64_t nm, uint8_t *Gm, int64_t ldm)
{
    const int64_t idx = blockIdx.x * (int64_t) blockDim.x + threadIdx.x;
    if (idx >= nm * n) {
        return;
    }
    const int64_t i = idx / n, j = idx % n;
    const int32_t s = msites[i];
    const uint8_t x = A[(int64_t) s * n + j];
    uint8_t *row = Gm + j * ldm + km[i];
    row[0] = x != 0 ? (uint8_t) 0x38 : (uint8_t) 0;
    for (int a = 1; a <= nall[i]; a++) {
        row[a] = x == a ? (uint8_t) 0x38 : (uint8_t) 0;
    }
}

// r[w][j]: sites of window w where sample j carries a derived allele.
__global__ void k_derived_counts(const uint8_t *A, int64_t n, const int32_t *wsite, int32_t Wn,
    int32_t *r)
{
    const int64_t j = blockIdx.x * (int64_t) blockDim.x + threadIdx.x;
    if (j >= n) {
        return;
    }
    for (int w = 0; w < Wn; w++) {
        int32_t c = 0;
        for (int32_t s = wsite[w]; s < wsite[w + 1]; s++) {
            c += A[(int64_t) s * n + j] != 0;
        }
        r[(int64_t) w * n + j] = c;
    }
}

// One window: per-sample divergences summed over the sample sets, then the
// reference's normalisation (fill_lower_triangle_count_normalise,
// trees.c:8876-8898) and span normalisation.  Block per (I, J) set pair.
__global__ void __launch_bounds__(256) k_divmat_sets(const int32_t *P, int64_t ldp,
    const int32_t *r, const int32_t *set_off, const int32_t *set_samples, int32_t K,
    double span, int span_normalise, double *out)
{
    __shared__ double red[256];
    const int I = blockIdx.x / K, J = blockIdx.x % K;
    const int32_t a0 = set_off[I], a1 = set_off[I + 1], b0 = set_off[J], b1 = set_off[J + 1];
    const int64_t na = a1 - a0, nb = b1 - b0, total = na * nb;
    double s = 0;
    for (int64_t idx = threadIdx.x; idx < total; idx += blockDim.x) {
        const int32_t j = set_samples[a0 + idx / nb], k = set_samples[b0 + idx % nb];
        if (j != k) {
            const int32_t lo = j < k ? j : k, hi = j < k ? k : j;
            s += (double) (r[j] + r[k] - P[(int64_t) lo * ldp + hi]);
        }
    }
    red[threadIdx.x] = s;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if ((int) threadIdx.x < o) {
            red[threadIdx.x] += red[threadIdx.x + o];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        double v = red[0];
        const double den = I == J ? (double) na * (double) (na - 1) : (double) na * (double) nb;
        if (den != 0) {
            v /= den;
        }
        if (span_normalise) {
            v /= span;
        }
        out[(int64_t) I * K + J] = v;
    }
}

// One sample per set: D directly (block row per sample).
__global__ void __launch_bounds__(256) k_divmat_samples(const int32_t *P, int64_t ldp,
    const int32_t *r, const int32_t *samples_idx, int32_t K, double span, int span_normalise,
    double *out)
{
    const int I = blockIdx.x;
    const int32_t j = samples_idx[I];
    for (int J = threadIdx.x; J < K; J += blockDim.x) {
        const int32_t k = samples_idx[J];
        double v = 0;
        if (j != k) {
            const int32_t lo = j < k ? j : k, hi = j < k ? k : j;
            v = (double) (r[j] + r[k] - P[(int64_t) lo * ldp + hi]);
        }
        if (span_normalise) {
            v /= span;
        }
        out[(int64_t) I * K + J] = v;
    }
}

// genetic_relatedness_matrix's normalisation of one window's K x K matrix
// (python/tskit/trees.py:9086-9095): diagonal * (n - 1) / n, then
// K = ((B + mean(B)) - (y_i + y_j)) / -2 with y the column means.
__global__ void __launch_bounds__(256) k_grm_colmeans(double *B, int32_t K, const double *nsz,
    double *y)
{
    __shared__ double red[256];
    const int j = blockIdx.x;
    if (threadIdx.x == 0) {
        B[(int64_t) j * K + j] = B[(int64_t) j * K + j] * (nsz[j] - 1) / nsz[j];
    }
    __syncthreads();
    double s = 0;
    const int64_t chunk = (K + blockDim.x - 1) / blockDim.x;
    const int64_t b = (int64_t) threadIdx.x * chunk, e = b + chunk < K ? b + chunk : K;
    for (int64_t i = b; i < e; i++) {
        s += B[i * K + j];
    }
    red[threadIdx.x] = s;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if ((int) threadIdx.x < o) {
            red[threadIdx.x] += red[threadIdx.x + o];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        y[j] = red[0] / (double) K;
    }
}

__global__ void __launch_bounds__(256) k_grm_apply(double *B, int32_t K, const double *y)
{
    __shared__ double red[256];
    // overall mean: the column sums (K * y_j) in a fixed order
    double s = 0;
    for (int j = threadIdx.x; j < K; j += blockDim.x) {
        s += y[j];
    }
    red[threadIdx.x] = s;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if ((int) threadIdx.x < o) {
            red[threadIdx.x] += red[threadIdx.x + o];
        }
        __syncthreads();
    }
    const double mean = red[0] / (double) K;
    const int i = blockIdx.x;
    for (int j = threadIdx.x; j < K; j += blockDim.x) {
        double &v = B[(int64_t) i * K + j];
        v = ((v + mean) - (y[i] + y[j])) / -2.0;
    }
}

struct DivmatPlan {
    int64_t n, S, Wn;
    std::vector<int32_t> wsite;   // Wn + 1
    std::vector<int64_t> kb;      // per site: column in Gb or -1
    std::vector<int64_t> kb_seg;  // Wn + 1: window segment starts in Gb (multiples of 128)
    std::vector<int32_t> msites;  // multiallelic sites
    std::vector<int64_t> km;      // their first row in Gm
    std::vector<int32_t> nall;    // their largest allele code
    std::vector<int64_t> km_seg;  // Wn + 1
};

// The divergence-matrix pipeline for K sample sets given as sample indexes
// (set_off: K + 1 offsets).  relatedness: apply the relatedness-matrix
// normalisation to each window.  Result: Wn x K x K (host).
static int divmat_run(const tsg_treeseq_t *ts, int64_t K, const std::vector<int32_t> &set_off,
    const std::vector<int32_t> &set_samples, bool singletons, int64_t Wn, const double *windows,
    bool span_normalise, bool relatedness, const std::vector<double> &nsz, double *result)
{
    const int64_t n = ts->v.num_samples, S = ts->v.num_sites;
    const auto &pos = ts->h_site_position;
    DivmatPlan pl;
    pl.n = n;
    pl.S = S;
    pl.Wn = Wn;
    pl.wsite.resize((size_t) Wn + 1);
    for (int64_t w = 0; w <= Wn; w++) {
        pl.wsite[(size_t) w] =
            (int32_t) (std::lower_bound(pos.begin(), pos.end(), windows[w]) - pos.begin());
    }
    const int64_t s_lo = pl.wsite[0], s_hi = pl.wsite[(size_t) Wn];
    // the sites the windows cover (decoded on the device below)
    const int64_t ns = s_hi - s_lo;
    int max_allele = 0, ret;
    if ((ret = site_max_allele(ts, s_lo, s_hi, &max_allele)) != 0) {
        return ret;
    }
    // per site: biallelic (largest code <= 1) or multiallelic
    const HostTopology &h = ts->host;
    pl.kb.assign((size_t) ns, -1);
    pl.kb_seg.assign((size_t) Wn + 1, 0);
    pl.km_seg.assign((size_t) Wn + 1, 0);
    int64_t colb = 0, rowm = 0;
    for (int64_t w = 0; w < Wn; w++) {
        pl.kb_seg[(size_t) w] = colb;
        pl.km_seg[(size_t) w] = rowm;
        for (int64_t s = pl.wsite[(size_t) w]; s < pl.wsite[(size_t) w + 1]; s++) {
            int32_t mx = 0;
            for (int32_t m = h.site_mut[(size_t) s]; m < h.site_mut[(size_t) s + 1]; m++) {
                mx = std::max(mx, h.mut_allele[(size_t) m]);
            }
            if (mx <= 1) {
                pl.kb[(size_t) (s - s_lo)] = colb++;
            } else {
                pl.msites.push_back((int32_t) (s - s_lo));
                pl.km.push_back(rowm);
                pl.nall.push_back(mx);
                rowm += 1 + mx;
            }
        }
        colb = up128(colb);
        rowm = up128(rowm);
    }
    pl.kb_seg[(size_t) Wn] = colb;
    pl.km_seg[(size_t) Wn] = rowm;
    const int64_t ldb = std::max<int64_t>(colb, 128), ldm = std::max<int64_t>(rowm, 128);
    const int64_t nrows = n;

    cudaStream_t st = ts->sync_stream;
    std::vector<int32_t> tiles;
    gram_tiles(n, tiles);
    const int64_t num_tiles = (int64_t) tiles.size() / 2;
    // device buffers
    uint8_t *dA = nullptr, *dGb = nullptr, *dGm = nullptr;
    int64_t *dkb = nullptr, *dkm = nullptr;
    int32_t *dms = nullptr, *dnall = nullptr, *dtiles = nullptr, *dP = nullptr, *dr = nullptr,
            *dws = nullptr, *derr = nullptr, *dsoff = nullptr, *dss = nullptr;
    double *dout = nullptr, *dy = nullptr, *dnsz = nullptr;
    auto cleanup = [&]() {
        cudaFree(dA);
        cudaFree(dGb);
        cudaFree(dGm);
        cudaFree(dkb);
        cudaFree(dkm);
        cudaFree(dms);
        cudaFree(dnall);
        cudaFree(dtiles);
        cudaFree(dP);
        cudaFree(dr);
        cudaFree(dws);
        cudaFree(derr);
        cudaFree(dsoff);
        cudaFree(dss);
        cudaFree(dout);
        cudaFree(dy);
        cudaFree(dnsz);
    };
    auto alloc = [&](void **p, int64_t bytes) {
        return cudaMalloc(p, (size_t) std::max<int64_t>(bytes, 256)) == cudaSuccess;
    };
    if (!alloc((void **) &dA, ns * n) || !alloc((void **) &dGb, nrows * ldb)
        || !alloc((void **) &dGm, pl.msites.empty() ? 0 : nrows * ldm)
        || !alloc((void **) &dkb, ns * 8) || !alloc((void **) &dkm, (int64_t) pl.km.size() * 8)
        || !alloc((void **) &dms, (int64_t) pl.msites.size() * 4)
        || !alloc((void **) &dnall, (int64_t) pl.nall.size() * 4)
        || !alloc((void **) &dtiles, (int64_t) tiles.size() * 4)
        || !alloc((void **) &dP, n * n * 4) || !alloc((void **) &dr, Wn * n * 4)
        || !alloc((void **) &dws, (Wn + 1) * 4) || !alloc((void **) &derr, 4)
        || !alloc((void **) &dsoff, (K + 1) * 4)
        || !alloc((void **) &dss, (int64_t) set_samples.size() * 4)
        || !alloc((void **) &dout, K * K * 8) || !alloc((void **) &dy, K * 8)
        || !alloc((void **) &dnsz, K * 8)) {
        cudaGetLastError();
        cleanup();
        return TSG_ERR_NO_MEMORY;
    }
    std::vector<int32_t> wsite_rel((size_t) Wn + 1);
    for (int64_t w = 0; w <= Wn; w++) {
        wsite_rel[(size_t) w] = (int32_t) (pl.wsite[(size_t) w] - s_lo);
    }
    auto h2d = [&](void *d, const void *hsrc, int64_t bytes) {
        return bytes == 0 || cudaMemcpyAsync(d, hsrc, (size_t) bytes, cudaMemcpyHostToDevice, st)
            == cudaSuccess;
    };
    if ((ret = decode_genotypes_device(ts, s_lo, s_hi, dA, st)) != 0) {
        cleanup();
        return ret;
    }
    if (!h2d(dkb, pl.kb.data(), ns * 8)
        || !h2d(dkm, pl.km.data(), (int64_t) pl.km.size() * 8)
        || !h2d(dms, pl.msites.data(), (int64_t) pl.msites.size() * 4)
        || !h2d(dnall, pl.nall.data(), (int64_t) pl.nall.size() * 4)
        || !h2d(dtiles, tiles.data(), (int64_t) tiles.size() * 4)
        || !h2d(dws, wsite_rel.data(), (Wn + 1) * 4)
        || !h2d(dsoff, set_off.data(), (K + 1) * 4)
        || !h2d(dss, set_samples.data(), (int64_t) set_samples.size() * 4)
        || !h2d(dnsz, nsz.data(), K * 8)
        || cudaMemsetAsync(dGb, 0, (size_t) (nrows * ldb), st) != cudaSuccess
        || (!pl.msites.empty() && cudaMemsetAsync(dGm, 0, (size_t) (nrows * ldm), st) != cudaSuccess)
        || cudaMemsetAsync(derr, 0, 4, st) != cudaSuccess) {
        cleanup();
        return TSG_ERR_CUDA;
    }
    auto launched = [&]() {
        g_launches.fetch_add(1, std::memory_order_relaxed);
        return cudaGetLastError() == cudaSuccess;
    };
    bool ok = true;
    if (ns > 0) {
        dim3 grid((unsigned) ((ns + 31) / 32), (unsigned) ((n + 31) / 32));
        k_pack_biallelic<<<grid, 256, 0, st>>>(dA, ns, n, dkb, dGb, ldb);
        ok = ok && launched();
        if (!pl.msites.empty()) {
            const int64_t tot = (int64_t) pl.msites.size() * n;
            k_pack_multi<<<(unsigned) ((tot + 255) / 256), 256, 0, st>>>(dA, n, dms, dkm, dnall,
                (int64_t) pl.msites.size(), dGm, ldm);
            ok = ok && launched();
        }
        k_derived_counts<<<(unsigned) ((n + 255) / 256), 256, 0, st>>>(dA, n, dws, (int32_t) Wn, dr);
        ok = ok && launched();
    } else {
        ok = ok && cudaMemsetAsync(dr, 0, (size_t) (Wn * n * 4), st) == cudaSuccess;
    }
    if (!ok) {
        cleanup();
        return TSG_ERR_CUDA;
    }
    const int64_t chunk = (int64_t) 1 << 24;
    for (int64_t w = 0; w < Wn && ok; w++) {
        bool acc = false;
        // P = 2 Xb^T Xb (biallelic) + (X_any^T X_any + Z^T Z) (multiallelic)
        for (int pass = 0; pass < 2 && ok; pass++) {
            const uint8_t *G = pass == 0 ? dGb : dGm;
            const int64_t ld = pass == 0 ? ldb : ldm;
            const int64_t a = pass == 0 ? pl.kb_seg[(size_t) w] : pl.km_seg[(size_t) w];
            const int64_t b = pass == 0 ? pl.kb_seg[(size_t) w + 1] : pl.km_seg[(size_t) w + 1];
            for (int64_t k0 = a; k0 < b; k0 += chunk) {
                const int64_t kc = std::min(chunk, b - k0);
                if ((ret = launch_gram(G, n, ld, k0, kc, dtiles, num_tiles, pass == 0 ? 2 : 1,
                         acc, dP, n, derr, st))
                    != 0) {
                    ok = false;
                    break;
                }
                acc = true;
            }
        }
        if (!ok) {
            break;
        }
        if (!acc) {
            ok = cudaMemsetAsync(dP, 0, (size_t) (n * n * 4), st) == cudaSuccess;
        }
        const double span = windows[w + 1] - windows[w];
        if (singletons) {
            k_divmat_samples<<<(unsigned) K, 256, 0, st>>>(dP, n, dr + w * n, dss, (int32_t) K,
                span, span_normalise ? 1 : 0, dout);
        } else {
            k_divmat_sets<<<(unsigned) (K * K), 256, 0, st>>>(dP, n, dr + w * n, dsoff, dss,
                (int32_t) K, span, span_normalise ? 1 : 0, dout);
        }
        ok = ok && launched();
        if (relatedness && K > 0) {
            k_grm_colmeans<<<(unsigned) K, 256, 0, st>>>(dout, (int32_t) K, dnsz, dy);
            ok = ok && launched();
            k_grm_apply<<<(unsigned) K, 256, 0, st>>>(dout, (int32_t) K, dy);
            ok = ok && launched();
        }
        ok = ok
            && cudaMemcpyAsync(result + w * K * K, dout, (size_t) (K * K * 8),
                   cudaMemcpyDeviceToHost, st) == cudaSuccess;
    }
    int32_t herr = 0;
    if (ok) {
        ok = cudaMemcpyAsync(&herr, derr, 4, cudaMemcpyDeviceToHost, st) == cudaSuccess
            && cudaStreamSynchronize(st) == cudaSuccess;
    }
    cleanup();
    if (!ok) {
        return ret != 0 ? ret : TSG_ERR_CUDA;
    }
    return herr != 0 ? TSG_ERR_DEVICE_CHECK : 0;
}

// get_sample_set_index_map (trees.c:8828-8874) in sample indexes; NULL sets
// mean every sample alone.
static int divmat_sets(const tsg_treeseq_t *ts, uint64_t K, const uint64_t *sizes,
    const int32_t *sets, std::vector<int32_t> &off, std::vector<int32_t> &samples, bool &singletons,
    std::vector<double> &nsz, int64_t &nsets)
{
    const int64_t n = ts->v.num_samples, N = ts->v.num_nodes;
    singletons = true;
    if (sets == nullptr) {
        nsets = sizes == nullptr ? n : (int64_t) K;
        off.resize((size_t) nsets + 1);
        samples.resize((size_t) n);
        for (int64_t i = 0; i < n; i++) {
            samples[(size_t) i] = (int32_t) i;
        }
        off[0] = 0;
        for (int64_t k = 0; k < nsets; k++) {
            const int64_t sz = sizes == nullptr ? 1 : (int64_t) sizes[k];
            off[(size_t) k + 1] = off[(size_t) k] + (int32_t) sz;
            singletons = singletons && sz == 1;
        }
        if (off[(size_t) nsets] > n) {
            return TSG_ERR_BAD_PARAM_VALUE;
        }
    } else {
        nsets = (int64_t) K;
        off.assign((size_t) nsets + 1, 0);
        std::vector<char> seen((size_t) N, 0);
        int64_t j = 0;
        for (int64_t k = 0; k < nsets; k++) {
            const int64_t sz = sizes == nullptr ? 1 : (int64_t) sizes[k];
            for (int64_t l = 0; l < sz; l++) {
                const int32_t u = sets[j++];
                if (u < 0 || u >= N) {
                    return TSG_ERR_NODE_OUT_OF_BOUNDS;
                }
                const int32_t si = ts->h_sample_index[(size_t) u];
                if (si < 0) {
                    return TSG_ERR_BAD_SAMPLES;
                }
                if (seen[(size_t) u]) {
                    return TSG_ERR_DUPLICATE_SAMPLE;
                }
                seen[(size_t) u] = 1;
                samples.push_back(si);
            }
            off[(size_t) k + 1] = off[(size_t) k] + (int32_t) sz;
            singletons = singletons && sz == 1;
        }
    }
    nsz.resize((size_t) nsets);
    for (int64_t k = 0; k < nsets; k++) {
        nsz[(size_t) k] = (double) (off[(size_t) k + 1] - off[(size_t) k]);
    }
    return 0;
}

// Branch mode (tsk_treeseq_divergence_matrix_branch, c/tskit/trees.c:
// 8578-8672): for every tree and pair of samples, (t_w - t_u) + (t_w - t_v)
// times the tree's overlap with the window, w the pair's MRCA, or each
// sample's own root for samples in different subtrees.  One CTA per 32 x 32
// tile of sample pairs replays the whole sequence (parent pointers, the
// events of each transition applied in parallel, one child each); per tree,
// each tile sample's depth and root come from one walk, and each thread
// finds its pair's MRCA by lifting the deeper sample and walking both up.
// Each pair's window sum is added tree by tree, in the reference's order
// and arithmetic.  out: Wn x m x m (upper triangle, zero elsewhere).
#define TSG_DIVB_TILE 32
__global__ void __launch_bounds__(TSG_DIVB_TILE * TSG_DIVB_TILE) k_divmat_branch(TSView ts,
    const int32_t *focal, int32_t m, const int32_t *tiles, int32_t Wn, const double *windows,
    int32_t *gpar, int par_in_smem, double *out, int32_t *err)
{
    extern __shared__ int32_t smem_par[];
    __shared__ int32_t s_node[2 * TSG_DIVB_TILE], s_depth[2 * TSG_DIVB_TILE],
        s_root[2 * TSG_DIVB_TILE];
    const int64_t N = ts.num_nodes;
    int32_t *par = par_in_smem ? smem_par : gpar + (int64_t) blockIdx.x * N;
    const int tid = threadIdx.x, bd = blockDim.x;
    const int32_t bi = tiles[2 * blockIdx.x], bj = tiles[2 * blockIdx.x + 1];
    // tile samples: rows bi*32 + r, columns bj*32 + c
    if (tid < 2 * TSG_DIVB_TILE) {
        const int32_t k = tid < TSG_DIVB_TILE ? bi * TSG_DIVB_TILE + tid
                                               : bj * TSG_DIVB_TILE + (tid - TSG_DIVB_TILE);
        s_node[tid] = k < m ? focal[k] : -1;
    }
    for (int64_t u = tid; u < N; u += bd) {
        par[u] = -1;
    }
    __syncthreads();
    const int r = tid / TSG_DIVB_TILE, c = tid % TSG_DIVB_TILE;
    const int32_t gi = bi * TSG_DIVB_TILE + r, gj = bj * TSG_DIVB_TILE + c;
    const bool mine = gi < m && gj < m && gi < gj;
    const int32_t u = s_node[r], v = s_node[TSG_DIVB_TILE + c];
    const double tu0 = mine ? ts.node_time[u] : 0.0, tv0 = mine ? ts.node_time[v] : 0.0;
    int32_t w = 0;
    double acc = 0.0;
    auto flush = [&]() {
        if (mine) {
            out[((int64_t) w * m + gi) * m + gj] = acc;
        }
        acc = 0.0;
        w++;
    };
    for (int32_t t = 0; t < (int32_t) ts.num_trees && w < Wn; t++) {
        for (int32_t i = ts.tree_out[t] + tid; i < ts.tree_out[t + 1]; i += bd) {
            par[ts.rem_child[i]] = -1;
        }
        __syncthreads();
        for (int32_t i = ts.tree_in[t] + tid; i < ts.tree_in[t + 1]; i += bd) {
            par[ts.ins_child[i]] = ts.ins_parent[i];
        }
        __syncthreads();
        const double left = ts.breakpoints[t], right = ts.breakpoints[t + 1];
        if (right <= windows[w]) {
            continue;  // before the current window
        }
        // depth and root of each tile sample
        if (tid < 2 * TSG_DIVB_TILE) {
            int32_t x = s_node[tid], depth = 0, root = x;
            if (x >= 0) {
                for (int32_t y = par[x]; y >= 0; y = par[y]) {
                    root = y;
                    if (++depth > N) {
                        dev_error(err, DEV_PATH_TOO_LONG);
                        break;
                    }
                }
            }
            s_depth[tid] = depth;
            s_root[tid] = root;
        }
        __syncthreads();
        double d = 0.0;
        if (mine) {
            int32_t a = u, b = v, da = s_depth[r], db = s_depth[TSG_DIVB_TILE + c];
            int32_t top_u, top_v;
            if (s_root[r] != s_root[TSG_DIVB_TILE + c]) {
                top_u = s_root[r];
                top_v = s_root[TSG_DIVB_TILE + c];
            } else {
                for (; da > db; da--) {
                    a = par[a];
                }
                for (; db > da; db--) {
                    b = par[b];
                }
                // at equal depths below one root the walks meet (at most
                // depth steps; node times increase along parents)
                for (int32_t steps = 0; a != b && a >= 0 && b >= 0; steps++) {
                    if (steps > da) {
                        dev_error(err, DEV_PATH_TOO_LONG);
                        a = b = -1;
                        break;
                    }
                    a = par[a];
                    b = par[b];
                }
                top_u = top_v = a;
            }
            if (top_u >= 0 && top_v >= 0) {
                d = (ts.node_time[top_u] - tu0) + (ts.node_time[top_v] - tv0);
            }
        }
        // the tree's overlap with each window it meets
        for (int32_t ww = w; ww < Wn && windows[ww] < right; ww++) {
            const double a = left > windows[ww] ? left : windows[ww];
            const double b = right < windows[ww + 1] ? right : windows[ww + 1];
            if (b <= a) {
                continue;
            }
            while (w < ww) {
                flush();
            }
            acc += d * (b - a);
        }
        while (w < Wn && windows[w + 1] <= right) {
            flush();
        }
        __syncthreads();
    }
    while (w < Wn) {
        flush();
    }
}

static int divmat_branch(const tsg_treeseq_t *ts, int64_t K, const std::vector<int32_t> &off,
    const std::vector<int32_t> &samples, int64_t Wn, const double *windows, uint32_t options,
    bool relatedness, const std::vector<double> &nsz, double *result)
{
    const int64_t n = ts->v.num_samples, m = (int64_t) samples.size(), N = ts->v.num_nodes;
    std::vector<int32_t> node_of((size_t) std::max<int64_t>(n, 1));
    for (int64_t u = 0; u < N; u++) {
        const int32_t si = ts->h_sample_index[(size_t) u];
        if (si >= 0) {
            node_of[(size_t) si] = (int32_t) u;
        }
    }
    std::vector<int32_t> focal((size_t) std::max<int64_t>(m, 1));
    for (int64_t j = 0; j < m; j++) {
        focal[(size_t) j] = node_of[(size_t) samples[(size_t) j]];
    }
    const int64_t nb = (m + TSG_DIVB_TILE - 1) / TSG_DIVB_TILE;
    std::vector<int32_t> tiles;
    for (int64_t a = 0; a < nb; a++) {
        for (int64_t b = a; b < nb; b++) {
            tiles.push_back((int32_t) a);
            tiles.push_back((int32_t) b);
        }
    }
    const int64_t ntiles = (int64_t) tiles.size() / 2;
    const size_t smem_bytes = (size_t) std::max<int64_t>(N, 1) * 4;
    const bool in_smem = smem_bytes <= 160 * 1024;
    tsg_treeseq_t *mts = const_cast<tsg_treeseq_t *>(ts);
    std::lock_guard<std::mutex> lock(mts->sync_mutex);
    cudaStream_t st = ts->sync_stream;
    std::vector<double> D((size_t) (Wn * m * m));
    double *dD = nullptr, *dwin = nullptr, *dout = nullptr, *dy = nullptr, *dnsz = nullptr;
    int32_t *dfocal = nullptr, *dtiles = nullptr, *dpar = nullptr, *derr = nullptr;
    auto cleanup = [&]() {
        cudaFree(dD);
        cudaFree(dwin);
        cudaFree(dout);
        cudaFree(dy);
        cudaFree(dnsz);
        cudaFree(dfocal);
        cudaFree(dtiles);
        cudaFree(dpar);
        cudaFree(derr);
    };
    auto alloc = [&](void **p, int64_t bytes) {
        return cudaMalloc(p, (size_t) std::max<int64_t>(bytes, 256)) == cudaSuccess;
    };
    if (!alloc((void **) &dD, Wn * m * m * 8) || !alloc((void **) &dwin, (Wn + 1) * 8)
        || !alloc((void **) &dfocal, m * 4) || !alloc((void **) &dtiles, ntiles * 8)
        || !alloc((void **) &derr, 4)
        || (!in_smem && !alloc((void **) &dpar, ntiles * N * 4))
        || !alloc((void **) &dout, K * K * 8) || !alloc((void **) &dy, K * 8)
        || !alloc((void **) &dnsz, K * 8)) {
        cudaGetLastError();
        cleanup();
        return TSG_ERR_NO_MEMORY;
    }
    int ret = 0;
    if (cudaMemsetAsync(dD, 0, (size_t) (Wn * m * m * 8), st) != cudaSuccess
        || cudaMemsetAsync(derr, 0, 4, st) != cudaSuccess
        || cudaMemcpyAsync(dwin, windows, (size_t) ((Wn + 1) * 8), cudaMemcpyHostToDevice, st)
            != cudaSuccess
        || (m > 0 && cudaMemcpyAsync(dfocal, focal.data(), (size_t) (m * 4),
                         cudaMemcpyHostToDevice, st) != cudaSuccess)
        || (ntiles > 0 && cudaMemcpyAsync(dtiles, tiles.data(), (size_t) (ntiles * 8),
                              cudaMemcpyHostToDevice, st) != cudaSuccess)
        || cudaMemcpyAsync(dnsz, nsz.data(), (size_t) (K * 8), cudaMemcpyHostToDevice, st)
            != cudaSuccess) {
        ret = TSG_ERR_CUDA;
    }
    if (ret == 0 && ntiles > 0) {
        if (in_smem && smem_bytes > 48 * 1024
            && cudaFuncSetAttribute(k_divmat_branch, cudaFuncAttributeMaxDynamicSharedMemorySize,
                   (int) smem_bytes) != cudaSuccess) {
            ret = TSG_ERR_CUDA;
        } else {
            k_divmat_branch<<<(unsigned) ntiles, TSG_DIVB_TILE * TSG_DIVB_TILE,
                in_smem ? smem_bytes : 0, st>>>(ts->v, dfocal, (int32_t) m, dtiles, (int32_t) Wn,
                dwin, dpar, in_smem ? 1 : 0, dD, derr);
            g_launches.fetch_add(1, std::memory_order_relaxed);
            if (cudaGetLastError() != cudaSuccess) {
                ret = TSG_ERR_CUDA;
            }
        }
    }
    int32_t herr = 0;
    if (ret == 0
        && (cudaMemcpyAsync(D.data(), dD, (size_t) (Wn * m * m * 8), cudaMemcpyDeviceToHost, st)
                != cudaSuccess
            || cudaMemcpyAsync(&herr, derr, 4, cudaMemcpyDeviceToHost, st) != cudaSuccess
            || cudaStreamSynchronize(st) != cudaSuccess)) {
        ret = TSG_ERR_CUDA;
    }
    if (ret == 0 && herr != 0) {
        ret = TSG_ERR_DEVICE_CHECK;
    }
    // sets: sums over their pairs, normalised as fill_lower_triangle_count_normalise
    // (trees.c:8876-8899), then by the window's span
    std::vector<double> out((size_t) (Wn * K * K), 0.0);
    for (int64_t w = 0; ret == 0 && w < Wn; w++) {
        const double *Dw = D.data() + w * m * m;
        auto pair = [&](int64_t i, int64_t j) {
            return i < j ? Dw[i * m + j] : Dw[j * m + i];
        };
        for (int64_t a = 0; a < K; a++) {
            for (int64_t b = a; b < K; b++) {
                double sum = 0.0;
                for (int32_t i = off[(size_t) a]; i < off[(size_t) a + 1]; i++) {
                    for (int32_t j = off[(size_t) b]; j < off[(size_t) b + 1]; j++) {
                        if (i != j) {
                            sum += pair(i, j);
                        }
                    }
                }
                const double na = nsz[(size_t) a], nb2 = nsz[(size_t) b];
                const double denom = a == b ? na * (na - 1) : na * nb2;
                if (denom != 0) {
                    sum /= denom;
                }
                if (options & TSG_STAT_SPAN_NORMALISE) {
                    sum /= windows[w + 1] - windows[w];
                }
                out[(size_t) (w * K * K + a * K + b)] = sum;
                out[(size_t) (w * K * K + b * K + a)] = sum;
            }
        }
    }
    for (int64_t w = 0; ret == 0 && w < Wn; w++) {
        if (!relatedness || K == 0) {
            std::copy(out.begin() + w * K * K, out.begin() + (w + 1) * K * K, result + w * K * K);
            continue;
        }
        if (cudaMemcpyAsync(dout, out.data() + w * K * K, (size_t) (K * K * 8),
                cudaMemcpyHostToDevice, st) != cudaSuccess) {
            ret = TSG_ERR_CUDA;
            break;
        }
        k_grm_colmeans<<<(unsigned) K, 256, 0, st>>>(dout, (int32_t) K, dnsz, dy);
        g_launches.fetch_add(1, std::memory_order_relaxed);
        k_grm_apply<<<(unsigned) K, 256, 0, st>>>(dout, (int32_t) K, dy);
        g_launches.fetch_add(1, std::memory_order_relaxed);
        if (cudaGetLastError() != cudaSuccess
            || cudaMemcpyAsync(result + w * K * K, dout, (size_t) (K * K * 8),
                   cudaMemcpyDeviceToHost, st) != cudaSuccess) {
            ret = TSG_ERR_CUDA;
        }
    }
    if (ret == 0 && cudaStreamSynchronize(st) != cudaSuccess) {
        ret = TSG_ERR_CUDA;
    }
    cleanup();
    return ret;
}

static int divmat_entry(const tsg_treeseq_t *ts, uint64_t K, const uint64_t *sizes,
    const int32_t *sets, uint64_t Wn, const double *windows, uint32_t options, bool relatedness,
    double *result)
{
    if (options & TSG_STAT_NODE) {
        return TSG_ERR_UNSUPPORTED_STAT_MODE;
    }
    bool site = options & TSG_STAT_SITE, branch = options & TSG_STAT_BRANCH;
    if (!site && !branch) {
        site = true;
    }
    if (site && branch) {
        return TSG_ERR_MULTIPLE_STAT_MODES;
    }
    if (options & TSG_STAT_POLARISED) {
        return TSG_ERR_STAT_POLARISED_UNSUPPORTED;
    }
    // c/tskit/trees.c:8628-8631
    if (branch && (ts->options & TSG_TIME_UNCALIBRATED)
        && !(options & TSG_STAT_ALLOW_TIME_UNCALIBRATED)) {
        return TSG_ERR_TIME_UNCALIBRATED;
    }
    const double L = ts->v.sequence_length;
    double default_windows[2] = { 0, L };
    if (windows == nullptr) {
        Wn = 1;
        windows = default_windows;
    } else {
        if (Wn < 1) {
            return TSG_ERR_BAD_NUM_WINDOWS;
        }
        if (windows[0] < 0 || windows[Wn] > L) {
            return TSG_ERR_BAD_WINDOWS;
        }
        for (uint64_t j = 0; j < Wn; j++) {
            if (windows[j] >= windows[j + 1]) {
                return TSG_ERR_BAD_WINDOWS;
            }
        }
    }
    std::vector<int32_t> off, samples;
    std::vector<double> nsz;
    bool singletons;
    int64_t nsets;
    int ret = divmat_sets(ts, K, sizes, sets, off, samples, singletons, nsz, nsets);
    if (ret != 0) {
        return ret;
    }
    if (branch) {
        return divmat_branch(ts, nsets, off, samples, (int64_t) Wn, windows, options,
            relatedness, nsz, result);
    }
    tsg_treeseq_t *mts = const_cast<tsg_treeseq_t *>(ts);
    std::lock_guard<std::mutex> lock(mts->sync_mutex);
    return divmat_run(ts, nsets, off, samples, singletons, (int64_t) Wn, windows,
        (options & TSG_STAT_SPAN_NORMALISE) != 0, relatedness, nsz, result);
}

}  // namespace tsg

using namespace tsg;

extern "C" {

int tsg_treeseq_divergence_matrix(const tsg_treeseq_t *self, uint64_t num_sample_sets,
    const uint64_t *sample_set_sizes, const int32_t *sample_sets, uint64_t num_windows,
    const double *windows, uint32_t options, double *result)
{
    return divmat_entry(self, num_sample_sets, sample_set_sizes, sample_sets, num_windows, windows,
        options, false, result);
}

int tsg_treeseq_genetic_relatedness_matrix(const tsg_treeseq_t *self, uint64_t num_sample_sets,
    const uint64_t *sample_set_sizes, const int32_t *sample_sets, uint64_t num_windows,
    const double *windows, uint32_t options, double *result)
{
    return divmat_entry(self, num_sample_sets, sample_set_sizes, sample_sets, num_windows, windows,
        options, true, result);
}

int tsg_treeseq_genotype_operand(const tsg_treeseq_t *self, int64_t site_start,
    int64_t site_stop, uint8_t *G, int64_t ld, void *cuda_stream)
{
    const int64_t n = self->v.num_samples;
    if (site_start < 0 || site_stop > self->v.num_sites || site_stop < site_start
        || ld < site_stop - site_start) {
        return TSG_ERR_BAD_PARAM_VALUE;
    }
    const int64_t ns = site_stop - site_start;
    int max_allele = 0;
    int ret = site_max_allele(self, site_start, site_stop, &max_allele);
    if (ret != 0 || ns == 0) {
        return ret;
    }
    cudaStream_t st = (cudaStream_t) cuda_stream;
    uint8_t *dA = nullptr;
    int64_t *dkb = nullptr;
    std::vector<int64_t> kb((size_t) ns);
    for (int64_t s = 0; s < ns; s++) {
        kb[(size_t) s] = s;
    }
    if (cudaMalloc(&dA, (size_t) (ns * n)) != cudaSuccess || cudaMalloc(&dkb, (size_t) ns * 8) != cudaSuccess) {
        cudaGetLastError();
        cudaFree(dA);
        return TSG_ERR_NO_MEMORY;
    }
    if ((ret = decode_genotypes_device(self, site_start, site_stop, dA, st)) != 0) {
        cudaFree(dA);
        cudaFree(dkb);
        return ret;
    }
    if (cudaMemcpyAsync(dkb, kb.data(), (size_t) ns * 8, cudaMemcpyHostToDevice, st) != cudaSuccess) {
        ret = TSG_ERR_CUDA;
    } else {
        dim3 grid((unsigned) ((ns + 31) / 32), (unsigned) ((n + 31) / 32));
        k_pack_biallelic<<<grid, 256, 0, st>>>(dA, ns, n, dkb, G, ld);
        g_launches.fetch_add(1, std::memory_order_relaxed);
        if (cudaGetLastError() != cudaSuccess || cudaStreamSynchronize(st) != cudaSuccess) {
            ret = TSG_ERR_CUDA;
        }
    }
    cudaFree(dA);
    cudaFree(dkb);
    return ret;
}

int tsg_gram_e4m3(const uint8_t *G, int64_t n, int64_t ld, int64_t k, int32_t *P, int64_t ldp,
    void *cuda_stream)
{
    NvtxRange nvtx("tsg.gram");
    cudaStream_t st = (cudaStream_t) cuda_stream;
    std::vector<int32_t> tiles;
    gram_tiles(n, tiles);
    int32_t *dtiles = nullptr, *derr = nullptr;
    if (cudaMalloc(&dtiles, std::max<size_t>(tiles.size() * 4, 4)) != cudaSuccess
        || cudaMalloc(&derr, 4) != cudaSuccess) {
        cudaGetLastError();
        cudaFree(dtiles);
        return TSG_ERR_NO_MEMORY;
    }
    int ret = 0;
    if (cudaMemcpyAsync(dtiles, tiles.data(), tiles.size() * 4, cudaMemcpyHostToDevice, st)
            != cudaSuccess
        || cudaMemsetAsync(derr, 0, 4, st) != cudaSuccess) {
        ret = TSG_ERR_CUDA;
    }
    const int64_t chunk = (int64_t) 1 << 24;
    bool acc = false;
    for (int64_t k0 = 0; ret == 0 && k0 < k; k0 += chunk) {
        ret = launch_gram(G, n, ld, k0, std::min(chunk, k - k0), dtiles,
            (int64_t) tiles.size() / 2, 1, acc, P, ldp, derr, st);
        acc = true;
    }
    int32_t herr = 0;
    if (ret == 0 && (cudaMemcpyAsync(&herr, derr, 4, cudaMemcpyDeviceToHost, st) != cudaSuccess
                        || cudaStreamSynchronize(st) != cudaSuccess)) {
        ret = TSG_ERR_CUDA;
    }
    cudaFree(dtiles);
    cudaFree(derr);
    if (ret == 0 && herr != 0) {
        ret = TSG_ERR_DEVICE_CHECK;
    }
    return ret;
}

}  // extern "C"
