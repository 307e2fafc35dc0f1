// Site-mode divergence matrix and genetic relatedness matrix through an
// exact Gram matrix on the tensor cores.
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
// Genotypes: decoded on the host (native threads, one tree range each, a
// tree with child/sibling lists as the reference's variant decoder keeps;
// isolated samples take the ancestral allele, c/tskit/trees.c:8775-8818),
// written site-major, uploaded once, then transposed on the GPU into the
// K-contiguous E4M3 operands (128-column segments per window).
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

// Site-major allele codes of every sample (row s: n bytes), for sites
// [s0, s1).  Returns the largest allele code seen (255 max).
static int decode_genotypes(const tsg_treeseq_t *ts, int64_t s0, int64_t s1, uint8_t *out,
    int *max_allele)
{
    const HostTopology &h = ts->host;
    const int64_t N = ts->v.num_nodes, T = ts->v.num_trees, n = ts->v.num_samples;
    const auto &bp = ts->h_breakpoints;
    const auto &sidx = ts->h_sample_index;
    if (s1 <= s0) {
        *max_allele = 0;
        return 0;
    }
    // trees holding the sites, split over threads
    const int64_t t_first = std::upper_bound(h.tree_sites.begin(), h.tree_sites.end(), (int32_t) s0)
        - h.tree_sites.begin() - 1;
    const int64_t t_last = std::upper_bound(h.tree_sites.begin(), h.tree_sites.end(), (int32_t) (s1 - 1))
        - h.tree_sites.begin() - 1;
    const int64_t ntrees = t_last - t_first + 1;
    unsigned nth = std::max(1u, std::min(64u, std::thread::hardware_concurrency()));
    nth = (unsigned) std::max<int64_t>(1, std::min<int64_t>(nth, ntrees));
    std::vector<int> maxa(nth, 0), bad(nth, 0);
    std::vector<std::thread> pool;
    for (unsigned tid = 0; tid < nth; tid++) {
        pool.emplace_back([&, tid]() {
            const int64_t ta = t_first + ntrees * tid / nth;
            const int64_t tb = t_first + ntrees * (tid + 1) / nth;
            std::vector<int32_t> parent((size_t) N, -1), lc((size_t) N, -1), rc((size_t) N, -1),
                ls((size_t) N, -1), rs((size_t) N, -1), stack;
            auto insert = [&](int32_t p, int32_t c) {
                parent[(size_t) c] = p;
                rs[(size_t) c] = -1;
                ls[(size_t) c] = rc[(size_t) p];
                if (rc[(size_t) p] != -1) {
                    rs[(size_t) rc[(size_t) p]] = c;
                } else {
                    lc[(size_t) p] = c;
                }
                rc[(size_t) p] = c;
            };
            auto remove = [&](int32_t p, int32_t c) {
                const int32_t l = ls[(size_t) c], r = rs[(size_t) c];
                if (l != -1) {
                    rs[(size_t) l] = r;
                } else {
                    lc[(size_t) p] = r;
                }
                if (r != -1) {
                    ls[(size_t) r] = l;
                } else {
                    rc[(size_t) p] = l;
                }
                parent[(size_t) c] = ls[(size_t) c] = rs[(size_t) c] = -1;
            };
            // seek: the edges alive at the first tree, in insertion order
            const double x0 = bp[(size_t) ta];
            for (int32_t i = 0; i < h.tree_in[(size_t) ta + 1]; i++) {
                const int32_t e = h.ins_edge[(size_t) i];
                if (h.right[(size_t) e] > x0) {
                    insert(h.ins_parent[(size_t) i], h.ins_child[(size_t) i]);
                }
            }
            for (int64_t t = ta; t < tb; t++) {
                if (t > ta) {
                    for (int32_t i = h.tree_out[(size_t) t]; i < h.tree_out[(size_t) t + 1]; i++) {
                        remove(h.rem_parent[(size_t) i], h.rem_child[(size_t) i]);
                    }
                    for (int32_t i = h.tree_in[(size_t) t]; i < h.tree_in[(size_t) t + 1]; i++) {
                        insert(h.ins_parent[(size_t) i], h.ins_child[(size_t) i]);
                    }
                }
                const int64_t sa = std::max<int64_t>(s0, h.tree_sites[(size_t) t]);
                const int64_t sb = std::min<int64_t>(s1, h.tree_sites[(size_t) t + 1]);
                for (int64_t s = sa; s < sb; s++) {
                    uint8_t *row = out + (s - s0) * n;
                    std::memset(row, 0, (size_t) n);
                    // mutations in order: a later (lower) mutation overrides
                    for (int32_t m = h.site_mut[(size_t) s]; m < h.site_mut[(size_t) s + 1]; m++) {
                        const int32_t a = h.mut_allele[(size_t) m];
                        if (a > 255 || a < 0) {
                            bad[tid] = 1;
                            continue;
                        }
                        maxa[tid] = std::max(maxa[tid], a);
                        stack.clear();
                        stack.push_back(h.mut_node[(size_t) m]);
                        while (!stack.empty()) {
                            const int32_t u = stack.back();
                            stack.pop_back();
                            const int32_t si = sidx[(size_t) u];
                            if (si >= 0) {
                                row[si] = (uint8_t) a;
                            }
                            for (int32_t c = lc[(size_t) u]; c != -1; c = rs[(size_t) c]) {
                                stack.push_back(c);
                            }
                        }
                    }
                }
            }
        });
    }
    for (auto &th : pool) {
        th.join();
    }
    int mx = 0;
    for (unsigned tid = 0; tid < nth; tid++) {
        if (bad[tid]) {
            return TSG_ERR_BAD_PARAM_VALUE;
        }
        mx = std::max(mx, maxa[tid]);
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
    // decode the sites the windows cover
    const int64_t ns = s_hi - s_lo;
    std::unique_ptr<uint8_t[]> A(new (std::nothrow) uint8_t[(size_t) std::max<int64_t>(ns * n, 1)]);
    if (!A) {
        return TSG_ERR_NO_MEMORY;
    }
    int max_allele = 0, ret;
    if ((ret = decode_genotypes(ts, s_lo, s_hi, A.get(), &max_allele)) != 0) {
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
    if (!h2d(dA, A.get(), ns * n) || !h2d(dkb, pl.kb.data(), ns * 8)
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
    if (branch) {
        return TSG_ERR_UNSUPPORTED_STAT_MODE;  // branch mode: not on this path
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
    std::unique_ptr<uint8_t[]> A(new (std::nothrow) uint8_t[(size_t) std::max<int64_t>(ns * n, 1)]);
    if (!A) {
        return TSG_ERR_NO_MEMORY;
    }
    int max_allele = 0;
    int ret;
    {
        tsg_treeseq_t *mts = const_cast<tsg_treeseq_t *>(self);
        std::lock_guard<std::mutex> lock(mts->sync_mutex);
        ret = decode_genotypes(self, site_start, site_stop, A.get(), &max_allele);
    }
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
    ret = 0;
    if (cudaMemcpyAsync(dA, A.get(), (size_t) (ns * n), cudaMemcpyHostToDevice, st) != cudaSuccess
        || cudaMemcpyAsync(dkb, kb.data(), (size_t) ns * 8, cudaMemcpyHostToDevice, st) != cudaSuccess) {
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
