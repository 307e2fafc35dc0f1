/*
 * CPU oracle for the tree-sequence statistics path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file restates, in plain C99 and double
 * precision, the reference tskit algorithms that the GPU kernels replace; it
 * is the checker for the parity tests and the timed CPU baseline ("port") on
 * machines where the reference cannot be built.  The product never links or
 * calls it.  Parity of this restatement is pinned against the reference
 * library itself (oracle/Makefile builds it) and against golden vectors
 * generated from it (tests/golden/).
 *
 * Restated reference functions (paths inside the tskit project):
 *   branch sweep       c/tskit/trees.c:1352-1523  tsk_treeseq_branch_general_stat
 *   node sweep         c/tskit/trees.c:1788-1918  tsk_treeseq_node_general_stat
 *   site sweep         c/tskit/trees.c:1654-1776  tsk_treeseq_site_general_stat
 *   allele weights     c/tskit/trees.c:1525-1652  get_allele_weights / site result
 *   unpolarised f      c/tskit/trees.c:1944-1972
 *   span normalise     c/tskit/trees.c:1920-1934
 *   summary functions  c/tskit/trees.c:3934 (diversity), 4221 (segsites),
 *                      4248 (Y1), 4690 (divergence), 4729/4755 (relatedness),
 *                      4899 (Y2), 4938 (f2), 5177 (Y3), 5219 (f3), 5266 (f4)
 *   AFS                c/tskit/trees.c:3469-3928
 *   relatedness matvec c/tskit/trees.c:10402-10816
 *   divergence matrix  c/tskit/trees.c:8684-8899 (site mode), 8578-8672 (branch)
 *
 * A compensated (double-double) restatement of the branch sweep for integer
 * summaries, orc_branch_count_stat_dd, attributes FP64 disagreements.
 *
 * Integer allele codes per mutation replace the reference's derived-state
 * string comparisons; they are computed on the host with the same numbering
 * (tskit_gb300/tables.py: Tables.allele_codes).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define ORC_STAT_SITE (1u << 0)
#define ORC_STAT_BRANCH (1u << 1)
#define ORC_STAT_NODE (1u << 2)
#define ORC_STAT_POLARISED (1u << 10)
#define ORC_STAT_SPAN_NORMALISE (1u << 11)
#define ORC_STAT_NONCENTRED (1u << 14)

#define ORC_ERR_NO_MEMORY (-2)
#define ORC_ERR_BAD_PARAM (-4)

enum {
    ORC_DIVERSITY = 1,
    ORC_SEGSITES = 2,
    ORC_Y1 = 3,
    ORC_DIVERGENCE = 4,
    ORC_Y2 = 5,
    ORC_F2 = 6,
    ORC_Y3 = 7,
    ORC_F3 = 8,
    ORC_F4 = 9,
    ORC_RELATEDNESS = 10,
    ORC_RELATEDNESS_NONCENTRED = 11,
};

typedef struct {
    int32_t num_nodes, num_edges, num_sites, num_mutations, num_samples;
    double sequence_length;
    const double *node_time;
    const int32_t *samples; /* sample node ids in increasing id order */
    const double *edge_left, *edge_right;
    const int32_t *edge_parent, *edge_child;
    const int32_t *ins, *rem;
    const double *site_position;
    const int32_t *mutation_site, *mutation_node, *mutation_allele, *mutation_alt;
} orc_ts_t;

typedef struct {
    int32_t type;
    int32_t idx[4];
} orc_output_t;

/* --------------------------------------------------------- summary funcs */
static void eval_summary(int32_t K, const double *x, const double *n, int32_t R,
    const orc_output_t *outs, double *y)
{
    double meanx = 0;
    int need_mean = 0;
    for (int32_t r = 0; r < R; r++) {
        if (outs[r].type == ORC_RELATEDNESS) {
            need_mean = 1;
        }
    }
    if (need_mean) {
        double s = 0;
        for (int32_t k = 0; k < K; k++) {
            s += x[k] / n[k];
        }
        meanx = s / (double) K;
    }
    for (int32_t r = 0; r < R; r++) {
        const int32_t *ix = outs[r].idx;
        const int32_t i = ix[0], j = ix[1], k = ix[2], l = ix[3];
        double v = 0;
        switch (outs[r].type) {
            case ORC_DIVERSITY:
                v = x[i] * (n[i] - x[i]) / (n[i] * (n[i] - 1));
                break;
            case ORC_SEGSITES:
                v = (x[i] > 0) * (1 - x[i] / n[i]);
                break;
            case ORC_Y1:
                v = x[i] * (n[i] - x[i]) * (n[i] - x[i] - 1)
                    / (n[i] * (n[i] - 1) * (n[i] - 2));
                break;
            case ORC_DIVERGENCE:
                v = x[i] * (n[j] - x[j]) / (n[i] * (n[j] - (i == j)));
                break;
            case ORC_Y2:
                v = x[i] * (n[j] - x[j]) * (n[j] - x[j] - 1) / (n[i] * n[j] * (n[j] - 1));
                break;
            case ORC_F2:
                v = (x[i] * (x[i] - 1) * (n[j] - x[j]) * (n[j] - x[j] - 1)
                        - x[i] * (n[i] - x[i]) * (n[j] - x[j]) * x[j])
                    / (n[i] * (n[i] - 1) * n[j] * (n[j] - 1));
                break;
            case ORC_Y3:
                v = x[i] * (n[j] - x[j]) * (n[k] - x[k]) / (n[i] * n[j] * n[k]);
                break;
            case ORC_F3:
                v = (x[i] * (x[i] - 1) * (n[j] - x[j]) * (n[k] - x[k])
                        - x[i] * (n[i] - x[i]) * (n[j] - x[j]) * x[k])
                    / (n[i] * (n[i] - 1) * n[j] * n[k]);
                break;
            case ORC_F4:
                v = (x[i] * x[k] * (n[j] - x[j]) * (n[l] - x[l])
                        - x[i] * x[l] * (n[j] - x[j]) * (n[k] - x[k]))
                    / (n[i] * n[j] * n[k] * n[l]);
                break;
            case ORC_RELATEDNESS:
                v = (x[i] / n[i] - meanx) * (x[j] / n[j] - meanx);
                break;
            case ORC_RELATEDNESS_NONCENTRED:
                v = x[i] * x[j] / (n[i] * n[j]);
                break;
            default:
                v = NAN;
        }
        y[r] = v;
    }
}

typedef struct {
    int32_t K, R;
    const double *n;
    const orc_output_t *outs;
    int polarised;
    const double *total;
    double *tmp_x, *tmp_y;
} summary_ctx_t;

/* f, or f(x) + f(total - x) when unpolarised (trees.c:1944-1972) */
static void summary(summary_ctx_t *c, const double *x, double *y, int unpolarised_wrap)
{
    eval_summary(c->K, x, c->n, c->R, c->outs, y);
    if (unpolarised_wrap) {
        for (int32_t k = 0; k < c->K; k++) {
            c->tmp_x[k] = c->total[k] - x[k];
        }
        eval_summary(c->K, c->tmp_x, c->n, c->R, c->outs, c->tmp_y);
        for (int32_t r = 0; r < c->R; r++) {
            y[r] += c->tmp_y[r];
        }
    }
}

static void span_normalise(int32_t Wn, const double *windows, int64_t row, double *a)
{
    for (int32_t w = 0; w < Wn; w++) {
        double span = windows[w + 1] - windows[w];
        for (int64_t k = 0; k < row; k++) {
            a[w * row + k] /= span;
        }
    }
}

/* --------------------------------------------------------- branch sweep */
static int branch_stat(const orc_ts_t *ts, summary_ctx_t *c, const double *W,
    int32_t Wn, const double *windows, double *result)
{
    const int32_t N = ts->num_nodes, E = ts->num_edges, K = c->K, R = c->R;
    const int unpol = !c->polarised;
    int32_t *parent = malloc((size_t) N * sizeof(int32_t));
    double *bl = calloc((size_t) N, sizeof(double));
    double *x = calloc((size_t) N * K, sizeof(double));
    double *s = calloc((size_t) N * R, sizeof(double));
    double *run = calloc((size_t) R, sizeof(double));
    double *zero = calloc((size_t) K, sizeof(double));
    double *fz = calloc((size_t) R, sizeof(double));
    int ret = ORC_ERR_NO_MEMORY;
    if (!parent || !bl || !x || !s || !run || !zero || !fz) {
        goto out;
    }
    for (int32_t u = 0; u < N; u++) {
        parent[u] = -1;
    }
    summary(c, zero, fz, unpol);
    for (int32_t u = 0; u < N; u++) {
        memcpy(s + (int64_t) u * R, fz, (size_t) R * sizeof(double));
    }
    for (int32_t j = 0; j < ts->num_samples; j++) {
        int32_t u = ts->samples[j];
        memcpy(x + (int64_t) u * K, W + (int64_t) j * K, (size_t) K * sizeof(double));
        summary(c, x + (int64_t) u * K, s + (int64_t) u * R, unpol);
    }
    memset(result, 0, (size_t) Wn * R * sizeof(double));
    int32_t tj = 0, tk = 0, w = 0;
    double left = 0, L = ts->sequence_length;
    while (tj < E || left < L) {
        while (tk < E && ts->edge_right[ts->rem[tk]] == left) {
            int32_t e = ts->rem[tk++];
            int32_t ch = ts->edge_child[e];
            for (int32_t r = 0; r < R; r++) {
                run[r] -= bl[ch] * s[(int64_t) ch * R + r];
            }
            parent[ch] = -1;
            bl[ch] = 0;
            for (int32_t u = ts->edge_parent[e]; u != -1; u = parent[u]) {
                double *su = s + (int64_t) u * R;
                for (int32_t r = 0; r < R; r++) {
                    run[r] -= bl[u] * su[r];
                }
                for (int32_t k = 0; k < K; k++) {
                    x[(int64_t) u * K + k] -= x[(int64_t) ch * K + k];
                }
                summary(c, x + (int64_t) u * K, su, unpol);
                for (int32_t r = 0; r < R; r++) {
                    run[r] += bl[u] * su[r];
                }
            }
        }
        while (tj < E && ts->edge_left[ts->ins[tj]] == left) {
            int32_t e = ts->ins[tj++];
            int32_t ch = ts->edge_child[e], p = ts->edge_parent[e];
            parent[ch] = p;
            bl[ch] = ts->node_time[p] - ts->node_time[ch];
            for (int32_t r = 0; r < R; r++) {
                run[r] += bl[ch] * s[(int64_t) ch * R + r];
            }
            for (int32_t u = p; u != -1; u = parent[u]) {
                double *su = s + (int64_t) u * R;
                for (int32_t r = 0; r < R; r++) {
                    run[r] -= bl[u] * su[r];
                }
                for (int32_t k = 0; k < K; k++) {
                    x[(int64_t) u * K + k] += x[(int64_t) ch * K + k];
                }
                summary(c, x + (int64_t) u * K, su, unpol);
                for (int32_t r = 0; r < R; r++) {
                    run[r] += bl[u] * su[r];
                }
            }
        }
        double right = L;
        if (tj < E && ts->edge_left[ts->ins[tj]] < right) {
            right = ts->edge_left[ts->ins[tj]];
        }
        if (tk < E && ts->edge_right[ts->rem[tk]] < right) {
            right = ts->edge_right[ts->rem[tk]];
        }
        while (w < Wn && windows[w] < right) {
            double a = left > windows[w] ? left : windows[w];
            double b = right < windows[w + 1] ? right : windows[w + 1];
            for (int32_t r = 0; r < R; r++) {
                result[(int64_t) w * R + r] += run[r] * (b - a);
            }
            if (windows[w + 1] <= right) {
                w++;
            } else {
                break;
            }
        }
        left = right;
    }
    ret = 0;
out:
    free(parent);
    free(bl);
    free(x);
    free(s);
    free(run);
    free(zero);
    free(fz);
    return ret;
}

/* -------------------------------------------- compensated branch sweep */
/*
 * A higher-precision restatement of the branch sweep (trees.c:1352-1523) for
 * sample-count statistics whose summary is an integer polynomial over a
 * product of set sizes (every built-in summary but the centred relatedness),
 * used to attribute disagreements between FP64 implementations at the 1e-12
 * level.  Same edge order and root-path updates as branch_stat, but:
 *   - counts are integers and each node's summary is kept as its exact
 *     integer numerator N(x) (f(x) = N(x) / D, D the term's denominator);
 *   - branch lengths are exact double-double differences of node times;
 *   - the running sum of bl * N and the window sums are double-double
 *     (Dekker/Knuth error-free transforms, no FMA needed), divided by D and
 *     rounded to double once at the end.
 * The running sum of the FP64 form drifts by about sqrt(updates) * 2^-53 of
 * its terms; this form's drift is below 2^-100 relative.
 */
typedef struct {
    double hi, lo;
} orc_dd;

static orc_dd dd_two_sum(double a, double b)
{
    double s = a + b;
    double bb = s - a;
    orc_dd r;
    r.hi = s;
    r.lo = (a - (s - bb)) + (b - bb);
    return r;
}

static orc_dd dd_quick(double a, double b)
{
    double s = a + b;
    orc_dd r;
    r.hi = s;
    r.lo = b - (s - a);
    return r;
}

static void dd_split(double a, double *hi, double *lo)
{
    double t = 134217729.0 * a; /* 2^27 + 1 */
    *hi = t - (t - a);
    *lo = a - *hi;
}

static orc_dd dd_two_prod(double a, double b)
{
    double ah, al, bh, bl;
    double p = a * b;
    dd_split(a, &ah, &al);
    dd_split(b, &bh, &bl);
    orc_dd r;
    r.hi = p;
    r.lo = ((ah * bh - p) + ah * bl + al * bh) + al * bl;
    return r;
}

static orc_dd dd_add(orc_dd a, orc_dd b)
{
    orc_dd s = dd_two_sum(a.hi, b.hi);
    orc_dd t = dd_two_sum(a.lo, b.lo);
    s.lo += t.hi;
    s = dd_quick(s.hi, s.lo);
    s.lo += t.lo;
    return dd_quick(s.hi, s.lo);
}

static orc_dd dd_neg(orc_dd a)
{
    a.hi = -a.hi;
    a.lo = -a.lo;
    return a;
}

static orc_dd dd_mul(orc_dd a, orc_dd b)
{
    orc_dd p = dd_two_prod(a.hi, b.hi);
    p.lo += a.hi * b.lo + a.lo * b.hi;
    return dd_quick(p.hi, p.lo);
}

static orc_dd dd_from_i64(int64_t v)
{
    orc_dd r;
    r.hi = (double) v;
    r.lo = (double) (v - (int64_t) r.hi);
    return r;
}

/* a / b to double-double accuracy (long division, three quotient digits) */
static orc_dd dd_div(orc_dd a, orc_dd b)
{
    double q1 = a.hi / b.hi;
    orc_dd r = dd_add(a, dd_neg(dd_mul(b, dd_two_sum(q1, 0.0))));
    double q2 = r.hi / b.hi;
    r = dd_add(r, dd_neg(dd_mul(b, dd_two_sum(q2, 0.0))));
    double q3 = r.hi / b.hi;
    orc_dd q = dd_quick(q1, q2);
    return dd_add(q, dd_two_sum(q3, 0.0));
}

/* the summary's integer numerator and denominator (trees.c summary funcs) */
static int64_t summary_num(int32_t type, const int64_t *x, const int64_t *n, const int32_t *ix)
{
    const int64_t xi = x[ix[0]], xj = x[ix[1]], xk = x[ix[2]], xl = x[ix[3]];
    const int64_t ni = n[ix[0]], nj = n[ix[1]], nk = n[ix[2]], nl = n[ix[3]];
    switch (type) {
        case ORC_DIVERSITY:
            return xi * (ni - xi);
        case ORC_SEGSITES:
            return xi > 0 ? ni - xi : 0;
        case ORC_Y1:
            return xi * (ni - xi) * (ni - xi - 1);
        case ORC_DIVERGENCE:
            return xi * (nj - xj);
        case ORC_Y2:
            return xi * (nj - xj) * (nj - xj - 1);
        case ORC_F2:
            return xi * (xi - 1) * (nj - xj) * (nj - xj - 1) - xi * (ni - xi) * (nj - xj) * xj;
        case ORC_Y3:
            return xi * (nj - xj) * (nk - xk);
        case ORC_F3:
            return xi * (xi - 1) * (nj - xj) * (nk - xk) - xi * (ni - xi) * (nj - xj) * xk;
        case ORC_F4:
            return xi * xk * (nj - xj) * (nl - xl) - xi * xl * (nj - xj) * (nk - xk);
        case ORC_RELATEDNESS_NONCENTRED:
            return xi * xj;
        default:
            return 0;
    }
}

static int64_t summary_den(int32_t type, const int64_t *n, const int32_t *ix)
{
    const int64_t ni = n[ix[0]], nj = n[ix[1]], nk = n[ix[2]], nl = n[ix[3]];
    switch (type) {
        case ORC_DIVERSITY:
            return ni * (ni - 1);
        case ORC_SEGSITES:
            return ni;
        case ORC_Y1:
            return ni * (ni - 1) * (ni - 2);
        case ORC_DIVERGENCE:
            return ni * (nj - (ix[0] == ix[1]));
        case ORC_Y2:
            return ni * nj * (nj - 1);
        case ORC_F2:
            return ni * (ni - 1) * nj * (nj - 1);
        case ORC_Y3:
            return ni * nj * nk;
        case ORC_F3:
            return ni * (ni - 1) * nj * nk;
        case ORC_F4:
            return ni * nj * nk * nl;
        case ORC_RELATEDNESS_NONCENTRED:
            return ni * nj;
        default:
            return 1;
    }
}

/* N(x), plus N(n - x) when unpolarised, for every output */
static void summary_nums(int32_t K, int32_t R, const orc_output_t *outs, const int64_t *n,
    const int64_t *x, int unpol, int64_t *xc, int64_t *y)
{
    for (int32_t r = 0; r < R; r++) {
        y[r] = summary_num(outs[r].type, x, n, outs[r].idx);
    }
    if (unpol) {
        for (int32_t k = 0; k < K; k++) {
            xc[k] = n[k] - x[k];
        }
        for (int32_t r = 0; r < R; r++) {
            y[r] += summary_num(outs[r].type, xc, n, outs[r].idx);
        }
    }
}

/*
 * member: num_samples x K 0/1 set membership (sample order); n: set sizes,
 * each below 2^15.  result: Wn x R, span-normalised when asked.  Returns
 * ORC_ERR_BAD_PARAM for a centred relatedness term or a set of 2^15 or more.
 */
int orc_branch_count_stat_dd(const orc_ts_t *ts, int32_t K, const uint8_t *member,
    const int64_t *n, int32_t R, const orc_output_t *outs, int32_t Wn,
    const double *windows, uint32_t options, double *result)
{
    const int32_t N = ts->num_nodes, E = ts->num_edges;
    const int unpol = !(options & ORC_STAT_POLARISED);
    for (int32_t k = 0; k < K; k++) {
        if (n[k] < 1 || n[k] >= (1 << 15)) {
            return ORC_ERR_BAD_PARAM;
        }
    }
    for (int32_t r = 0; r < R; r++) {
        if (outs[r].type < ORC_DIVERSITY || outs[r].type > ORC_RELATEDNESS_NONCENTRED
                || outs[r].type == ORC_RELATEDNESS) {
            return ORC_ERR_BAD_PARAM;
        }
    }
    int32_t *parent = malloc((size_t) N * sizeof(int32_t));
    orc_dd *bl = calloc((size_t) N, sizeof(orc_dd));
    int64_t *x = calloc((size_t) N * K, sizeof(int64_t));
    int64_t *s = calloc((size_t) N * R, sizeof(int64_t));
    orc_dd *run = calloc((size_t) R, sizeof(orc_dd));
    orc_dd *acc = calloc((size_t) Wn * R, sizeof(orc_dd));
    int64_t *zero = calloc((size_t) K, sizeof(int64_t));
    int64_t *xc = calloc((size_t) K, sizeof(int64_t));
    int64_t *fz = calloc((size_t) R, sizeof(int64_t));
    uint8_t *wtouched = calloc((size_t) Wn + 1, 1);
    int ret = ORC_ERR_NO_MEMORY;
    if (!parent || !bl || !x || !s || !run || !acc || !zero || !xc || !fz || !wtouched) {
        goto out;
    }
    for (int32_t u = 0; u < N; u++) {
        parent[u] = -1;
    }
    summary_nums(K, R, outs, n, zero, unpol, xc, fz);
    for (int32_t u = 0; u < N; u++) {
        memcpy(s + (int64_t) u * R, fz, (size_t) R * sizeof(int64_t));
    }
    for (int32_t j = 0; j < ts->num_samples; j++) {
        int32_t u = ts->samples[j];
        for (int32_t k = 0; k < K; k++) {
            x[(int64_t) u * K + k] = member[(int64_t) j * K + k] ? 1 : 0;
        }
        summary_nums(K, R, outs, n, x + (int64_t) u * K, unpol, xc, s + (int64_t) u * R);
    }
    int32_t tj = 0, tk = 0, w = 0;
    double left = 0, L = ts->sequence_length;
    /* a term whose denominator is zero (a set too small for it) is NaN in the
     * reference wherever its running sum has taken any node's value */
    int touched = 0;
#define ORC_DD_ADD_NODE(u, sign)                                                         \
    touched = 1;                                                                         \
    for (int32_t r = 0; r < R; r++) {                                                    \
        orc_dd v = dd_mul(bl[u], dd_from_i64(s[(int64_t) (u) * R + r]));                 \
        run[r] = dd_add(run[r], (sign) > 0 ? v : dd_neg(v));                             \
    }
    while (tj < E || left < L) {
        while (tk < E && ts->edge_right[ts->rem[tk]] == left) {
            int32_t e = ts->rem[tk++];
            int32_t ch = ts->edge_child[e];
            ORC_DD_ADD_NODE(ch, -1)
            parent[ch] = -1;
            bl[ch].hi = bl[ch].lo = 0;
            for (int32_t u = ts->edge_parent[e]; u != -1; u = parent[u]) {
                ORC_DD_ADD_NODE(u, -1)
                for (int32_t k = 0; k < K; k++) {
                    x[(int64_t) u * K + k] -= x[(int64_t) ch * K + k];
                }
                summary_nums(K, R, outs, n, x + (int64_t) u * K, unpol, xc, s + (int64_t) u * R);
                ORC_DD_ADD_NODE(u, +1)
            }
        }
        while (tj < E && ts->edge_left[ts->ins[tj]] == left) {
            int32_t e = ts->ins[tj++];
            int32_t ch = ts->edge_child[e], p = ts->edge_parent[e];
            parent[ch] = p;
            bl[ch] = dd_two_sum(ts->node_time[p], -ts->node_time[ch]);
            ORC_DD_ADD_NODE(ch, +1)
            for (int32_t u = p; u != -1; u = parent[u]) {
                ORC_DD_ADD_NODE(u, -1)
                for (int32_t k = 0; k < K; k++) {
                    x[(int64_t) u * K + k] += x[(int64_t) ch * K + k];
                }
                summary_nums(K, R, outs, n, x + (int64_t) u * K, unpol, xc, s + (int64_t) u * R);
                ORC_DD_ADD_NODE(u, +1)
            }
        }
        double right = L;
        if (tj < E && ts->edge_left[ts->ins[tj]] < right) {
            right = ts->edge_left[ts->ins[tj]];
        }
        if (tk < E && ts->edge_right[ts->rem[tk]] < right) {
            right = ts->edge_right[ts->rem[tk]];
        }
        while (w < Wn && windows[w] < right) {
            double a = left > windows[w] ? left : windows[w];
            double b = right < windows[w + 1] ? right : windows[w + 1];
            orc_dd len = dd_two_sum(b, -a);
            wtouched[w] |= (uint8_t) touched;
            for (int32_t r = 0; r < R; r++) {
                acc[(int64_t) w * R + r] = dd_add(acc[(int64_t) w * R + r], dd_mul(run[r], len));
            }
            if (windows[w + 1] <= right) {
                w++;
            } else {
                break;
            }
        }
        left = right;
    }
#undef ORC_DD_ADD_NODE
    for (int32_t wi = 0; wi < Wn; wi++) {
        orc_dd span = dd_two_sum(windows[wi + 1], -windows[wi]);
        for (int32_t r = 0; r < R; r++) {
            const int64_t d = summary_den(outs[r].type, n, outs[r].idx);
            if (d == 0) {
                result[(int64_t) wi * R + r] = wtouched[wi] ? NAN : 0.0;
                continue;
            }
            orc_dd den = dd_from_i64(d);
            if (options & ORC_STAT_SPAN_NORMALISE) {
                den = dd_mul(den, span);
            }
            orc_dd v = dd_div(acc[(int64_t) wi * R + r], den);
            result[(int64_t) wi * R + r] = v.hi + v.lo;
        }
    }
    ret = 0;
out:
    free(parent);
    free(bl);
    free(x);
    free(s);
    free(run);
    free(acc);
    free(zero);
    free(xc);
    free(fz);
    free(wtouched);
    return ret;
}

/* ----------------------------------------------------------- node sweep */
/*
 * Node mode (trees.c:1788-1918): for every node, the integral along each
 * window of f at the node's state.  Whenever a root-path walk changes a
 * node's state, the interval since the node's last update is added with the
 * old summary; at each window's end every node is flushed.
 * result: Wn x N x R.
 */
static int node_stat(const orc_ts_t *ts, summary_ctx_t *c, const double *W, int32_t Wn,
    const double *windows, double *result)
{
    const int32_t N = ts->num_nodes, E = ts->num_edges, K = c->K, R = c->R;
    const int unpol = !c->polarised;
    int32_t *parent = malloc((size_t) (N > 0 ? N : 1) * sizeof(int32_t));
    double *x = calloc((size_t) (N > 0 ? N : 1) * K, sizeof(double));
    double *s = calloc((size_t) (N > 0 ? N : 1) * R, sizeof(double));
    double *last = calloc((size_t) (N > 0 ? N : 1), sizeof(double));
    int ret = ORC_ERR_NO_MEMORY;
    if (!parent || !x || !s || !last) {
        goto out;
    }
    for (int32_t u = 0; u < N; u++) {
        parent[u] = -1;
    }
    for (int32_t j = 0; j < ts->num_samples; j++) {
        memcpy(x + (int64_t) ts->samples[j] * K, W + (int64_t) j * K, (size_t) K * sizeof(double));
    }
    for (int32_t u = 0; u < N; u++) {
        summary(c, x + (int64_t) u * K, s + (int64_t) u * R, unpol);
    }
    memset(result, 0, (size_t) Wn * N * R * sizeof(double));
    int32_t tj = 0, tk = 0, w = 0;
    double left = 0, L = ts->sequence_length;
    while (tj < E || left < L) {
        for (int pass = 0; pass < 2; pass++) {
            for (;;) {
                int32_t e;
                if (pass == 0) {
                    if (!(tk < E && ts->edge_right[ts->rem[tk]] == left)) {
                        break;
                    }
                    e = ts->rem[tk++];
                } else {
                    if (!(tj < E && ts->edge_left[ts->ins[tj]] == left)) {
                        break;
                    }
                    e = ts->ins[tj++];
                    parent[ts->edge_child[e]] = ts->edge_parent[e];
                }
                const int32_t ch = ts->edge_child[e];
                const double sign = pass == 0 ? -1.0 : 1.0;
                for (int32_t u = ts->edge_parent[e]; u != -1; u = parent[u]) {
                    double *out = result + ((int64_t) w * N + u) * R;
                    double *su = s + (int64_t) u * R;
                    for (int32_t r = 0; r < R; r++) {
                        out[r] += (left - last[u]) * su[r];
                    }
                    last[u] = left;
                    for (int32_t k = 0; k < K; k++) {
                        x[(int64_t) u * K + k] += sign * x[(int64_t) ch * K + k];
                    }
                    summary(c, x + (int64_t) u * K, su, unpol);
                }
                if (pass == 0) {
                    parent[ch] = -1;
                }
            }
        }
        double right = L;
        if (tj < E && ts->edge_left[ts->ins[tj]] < right) {
            right = ts->edge_left[ts->ins[tj]];
        }
        if (tk < E && ts->edge_right[ts->rem[tk]] < right) {
            right = ts->edge_right[ts->rem[tk]];
        }
        while (w < Wn && windows[w + 1] <= right) {
            const double wr = windows[w + 1];
            for (int32_t u = 0; u < N; u++) {
                double *out = result + ((int64_t) w * N + u) * R;
                for (int32_t r = 0; r < R; r++) {
                    out[r] += (wr - last[u]) * s[(int64_t) u * R + r];
                }
                last[u] = wr;
            }
            w++;
        }
        left = right;
    }
    ret = 0;
out:
    free(parent);
    free(x);
    free(s);
    free(last);
    return ret;
}

/* ------------------------------------------- branch divergence matrix */
/*
 * Branch divergence matrix with every sample its own set
 * (tsk_treeseq_divergence_matrix_branch, trees.c:8578-8672): for every tree
 * and pair of samples, the span-weighted path length between them,
 * (t_mrca - t_u) + (t_mrca - t_v), with each sample's root in place of the
 * MRCA for samples in different subtrees.  result: Wn x n x n, symmetric
 * with a zero diagonal, not span-normalised.
 */
int orc_divergence_matrix_branch(const orc_ts_t *ts, int32_t Wn, const double *windows,
    double *result)
{
    const int32_t N = ts->num_nodes, E = ts->num_edges, n = ts->num_samples;
    int32_t *parent = malloc((size_t) (N > 0 ? N : 1) * sizeof(int32_t));
    int64_t *stamp = calloc((size_t) (N > 0 ? N : 1), sizeof(int64_t));
    int64_t mark = 0;
    if (!parent || !stamp) {
        free(parent);
        free(stamp);
        return ORC_ERR_NO_MEMORY;
    }
    for (int32_t u = 0; u < N; u++) {
        parent[u] = -1;
    }
    memset(result, 0, (size_t) Wn * n * n * sizeof(double));
    int32_t tj = 0, tk = 0, w = 0;
    double left = 0, L = ts->sequence_length;
    while (tj < E || left < L) {
        while (tk < E && ts->edge_right[ts->rem[tk]] == left) {
            parent[ts->edge_child[ts->rem[tk++]]] = -1;
        }
        while (tj < E && ts->edge_left[ts->ins[tj]] == left) {
            const int32_t e = ts->ins[tj++];
            parent[ts->edge_child[e]] = ts->edge_parent[e];
        }
        double right = L;
        if (tj < E && ts->edge_left[ts->ins[tj]] < right) {
            right = ts->edge_left[ts->ins[tj]];
        }
        if (tk < E && ts->edge_right[ts->rem[tk]] < right) {
            right = ts->edge_right[ts->rem[tk]];
        }
        for (int32_t wi = w; wi < Wn && windows[wi] < right; wi++) {
            const double a = left > windows[wi] ? left : windows[wi];
            const double b = right < windows[wi + 1] ? right : windows[wi + 1];
            if (b <= a) {
                continue;
            }
            double *D = result + (int64_t) wi * n * n;
            for (int32_t j = 0; j < n; j++) {
                const int32_t u = ts->samples[j];
                mark++;
                int32_t ru = u;
                for (int32_t x = u; x != -1; x = parent[x]) {
                    stamp[x] = mark;
                    ru = x;
                }
                for (int32_t k = j + 1; k < n; k++) {
                    const int32_t v = ts->samples[k];
                    int32_t y = v, rv = v, top = -1;
                    for (; y != -1; y = parent[y]) {
                        if (stamp[y] == mark) {
                            top = y;
                            break;
                        }
                        rv = y;
                    }
                    const int32_t tu_node = top != -1 ? top : ru;
                    const int32_t tv_node = top != -1 ? top : rv;
                    const double d = ((ts->node_time[tu_node] - ts->node_time[u])
                                         + (ts->node_time[tv_node] - ts->node_time[v]))
                        * (b - a);
                    D[(int64_t) j * n + k] += d;
                }
            }
        }
        while (w < Wn && windows[w + 1] <= right) {
            w++;
        }
        left = right;
    }
    for (int32_t wi = 0; wi < Wn; wi++) {
        double *D = result + (int64_t) wi * n * n;
        for (int32_t j = 0; j < n; j++) {
            for (int32_t k = j + 1; k < n; k++) {
                D[(int64_t) k * n + j] = D[(int64_t) j * n + k];
            }
        }
    }
    free(parent);
    free(stamp);
    return 0;
}

/* ----------------------------------------------------------- site sweep */
/* allele states for one site: states[a*K + k] (trees.c:1525-1612) */
static int32_t site_allele_states(const orc_ts_t *ts, int32_t m0, int32_t m1,
    const double *x, int32_t K, const double *total, double *states)
{
    int32_t A = 1;
    for (int32_t m = m0; m < m1; m++) {
        if (ts->mutation_allele[m] + 1 > A) {
            A = ts->mutation_allele[m] + 1;
        }
    }
    memset(states, 0, (size_t) A * K * sizeof(double));
    memcpy(states, total, (size_t) K * sizeof(double));
    for (int32_t m = m0; m < m1; m++) {
        const double *xm = x + (int64_t) ts->mutation_node[m] * K;
        double *sa = states + (int64_t) ts->mutation_allele[m] * K;
        double *sb = states + (int64_t) ts->mutation_alt[m] * K;
        for (int32_t k = 0; k < K; k++) {
            sa[k] += xm[k];
        }
        for (int32_t k = 0; k < K; k++) {
            sb[k] -= xm[k];
        }
    }
    return A;
}

typedef void (*site_visit_fn)(void *ctx, int32_t site, int32_t m0, int32_t m1,
    const double *x, const int32_t *parent);

/* Shared tree sweep that keeps x up to date and visits each site. */
static int site_sweep(const orc_ts_t *ts, int32_t K, const double *Wnode_init,
    site_visit_fn visit, void *ctx)
{
    const int32_t N = ts->num_nodes, E = ts->num_edges;
    int32_t *parent = malloc((size_t) N * sizeof(int32_t));
    double *x = calloc((size_t) N * K, sizeof(double));
    if (!parent || !x) {
        free(parent);
        free(x);
        return ORC_ERR_NO_MEMORY;
    }
    for (int32_t u = 0; u < N; u++) {
        parent[u] = -1;
    }
    for (int32_t j = 0; j < ts->num_samples; j++) {
        memcpy(x + (int64_t) ts->samples[j] * K, Wnode_init + (int64_t) j * K,
            (size_t) K * sizeof(double));
    }
    int32_t tj = 0, tk = 0, site = 0, mut = 0;
    double left = 0, L = ts->sequence_length;
    while (tj < E || left < L) {
        while (tk < E && ts->edge_right[ts->rem[tk]] == left) {
            int32_t e = ts->rem[tk++];
            int32_t ch = ts->edge_child[e];
            for (int32_t u = ts->edge_parent[e]; u != -1; u = parent[u]) {
                for (int32_t k = 0; k < K; k++) {
                    x[(int64_t) u * K + k] -= x[(int64_t) ch * K + k];
                }
            }
            parent[ch] = -1;
        }
        while (tj < E && ts->edge_left[ts->ins[tj]] == left) {
            int32_t e = ts->ins[tj++];
            int32_t ch = ts->edge_child[e];
            parent[ch] = ts->edge_parent[e];
            for (int32_t u = parent[ch]; u != -1; u = parent[u]) {
                for (int32_t k = 0; k < K; k++) {
                    x[(int64_t) u * K + k] += x[(int64_t) ch * K + k];
                }
            }
        }
        double right = L;
        if (tj < E && ts->edge_left[ts->ins[tj]] < right) {
            right = ts->edge_left[ts->ins[tj]];
        }
        if (tk < E && ts->edge_right[ts->rem[tk]] < right) {
            right = ts->edge_right[ts->rem[tk]];
        }
        while (site < ts->num_sites && ts->site_position[site] < right) {
            int32_t m0 = mut;
            while (mut < ts->num_mutations && ts->mutation_site[mut] == site) {
                mut++;
            }
            visit(ctx, site, m0, mut, x, parent);
            site++;
        }
        left = right;
    }
    free(parent);
    free(x);
    return 0;
}

typedef struct {
    const orc_ts_t *ts;
    summary_ctx_t *c;
    const double *windows;
    int32_t Wn, w;
    double *result, *states, *y;
} site_stat_ctx_t;

static void site_stat_visit(void *vctx, int32_t site, int32_t m0, int32_t m1,
    const double *x, const int32_t *parent)
{
    (void) parent;
    site_stat_ctx_t *s = (site_stat_ctx_t *) vctx;
    summary_ctx_t *c = s->c;
    const double pos = s->ts->site_position[site];
    int32_t A = site_allele_states(s->ts, m0, m1, x, c->K, c->total, s->states);
    while (s->windows[s->w + 1] <= pos) {
        s->w++;
    }
    double *row = s->result + (int64_t) s->w * c->R;
    /* accumulate the per-site result first, as trees.c:1614-1652 does */
    double *acc = s->y + c->R;
    memset(acc, 0, (size_t) c->R * sizeof(double));
    for (int32_t a = c->polarised ? 1 : 0; a < A; a++) {
        eval_summary(c->K, s->states + (int64_t) a * c->K, c->n, c->R, c->outs, s->y);
        for (int32_t r = 0; r < c->R; r++) {
            acc[r] += s->y[r];
        }
    }
    for (int32_t r = 0; r < c->R; r++) {
        row[r] += acc[r];
    }
}

/*
 * Sample-count statistic (tsk_treeseq_sample_count_stat + general_stat).
 * W: num_samples x K weights indexed by sample order; n: K set sizes.
 * windows: Wn+1 breakpoints.  result: Wn x R (node mode: Wn x N x R).
 */
int orc_sample_count_stat(const orc_ts_t *ts, int32_t K, const double *W,
    const double *n, int32_t R, const orc_output_t *outs, int32_t Wn,
    const double *windows, uint32_t options, double *result)
{
    int ret;
    summary_ctx_t c;
    double *total = calloc((size_t) K, sizeof(double));
    double *tmp = calloc((size_t) (K + 2 * R + 8), sizeof(double));
    if (!total || !tmp) {
        free(total);
        free(tmp);
        return ORC_ERR_NO_MEMORY;
    }
    for (int32_t j = 0; j < ts->num_samples; j++) {
        for (int32_t k = 0; k < K; k++) {
            total[k] += W[(int64_t) j * K + k];
        }
    }
    c.K = K;
    c.R = R;
    c.n = n;
    c.outs = outs;
    c.polarised = !!(options & ORC_STAT_POLARISED);
    c.total = total;
    c.tmp_x = tmp;
    c.tmp_y = tmp + K;
    int64_t row = R;
    if (options & ORC_STAT_NODE) {
        ret = node_stat(ts, &c, W, Wn, windows, result);
        row = (int64_t) ts->num_nodes * R;
    } else if (options & ORC_STAT_BRANCH) {
        ret = branch_stat(ts, &c, W, Wn, windows, result);
    } else {
        site_stat_ctx_t s;
        int32_t max_alleles = 2;
        for (int32_t m = 0; m < ts->num_mutations; m++) {
            if (ts->mutation_allele[m] + 1 > max_alleles) {
                max_alleles = ts->mutation_allele[m] + 1;
            }
        }
        s.ts = ts;
        s.c = &c;
        s.windows = windows;
        s.Wn = Wn;
        s.w = 0;
        s.result = result;
        s.states = calloc((size_t) max_alleles * K, sizeof(double));
        s.y = calloc((size_t) 2 * R, sizeof(double));
        memset(result, 0, (size_t) Wn * R * sizeof(double));
        ret = (!s.states || !s.y) ? ORC_ERR_NO_MEMORY
                                  : site_sweep(ts, K, W, site_stat_visit, &s);
        free(s.states);
        free(s.y);
    }
    if (ret == 0 && (options & ORC_STAT_SPAN_NORMALISE)) {
        span_normalise(Wn, windows, row, result);
    }
    free(total);
    free(tmp);
    return ret;
}

/* ------------------------------------------------------------------ AFS */
/* fold a coordinate (trees.c:3469-3496) */
static void afs_fold(int64_t *coord, const int64_t *dims, int32_t K)
{
    double n = 0;
    int64_t s = 0;
    for (int32_t k = 0; k < K; k++) {
        n += (double) dims[k] - 1;
        s += coord[k];
    }
    n /= 2;
    int32_t k = K;
    while ((double) s == n && k > 0) {
        k--;
        n -= ((double) (dims[k] - 1)) / 2;
        s -= coord[k];
    }
    if ((double) s > n) {
        for (k = 0; k < K; k++) {
            coord[k] = dims[k] - 1 - coord[k];
        }
    }
}

static int64_t afs_index(const int64_t *coord, const int64_t *dims, int32_t K)
{
    int64_t idx = 0;
    for (int32_t k = 0; k < K; k++) {
        idx = idx * dims[k] + coord[k];
    }
    return idx;
}

typedef struct {
    const orc_ts_t *ts;
    int32_t K; /* number of sample sets; state has K+1 columns */
    const int64_t *dims;
    int64_t afs_size;
    const double *windows;
    int32_t Wn, w;
    int polarised;
    double *result, *states, *total;
    int64_t *coord;
} site_afs_ctx_t;

static void site_afs_visit(void *vctx, int32_t site, int32_t m0, int32_t m1,
    const double *x, const int32_t *parent)
{
    (void) parent;
    site_afs_ctx_t *s = (site_afs_ctx_t *) vctx;
    const int32_t K1 = s->K + 1;
    const double pos = s->ts->site_position[site];
    while (s->windows[s->w + 1] <= pos) {
        s->w++;
    }
    int32_t A = site_allele_states(s->ts, m0, m1, x, K1, s->total, s->states);
    double inc = s->polarised ? 1.0 : 0.5;
    double *afs = s->result + (int64_t) s->w * s->afs_size;
    for (int32_t a = s->polarised ? 1 : 0; a < A; a++) {
        const double *st = s->states + (int64_t) a * K1;
        int64_t all = (int64_t) st[s->K];
        if (all > 0 && all < s->ts->num_samples) {
            for (int32_t k = 0; k < s->K; k++) {
                s->coord[k] = (int64_t) st[k];
            }
            if (!s->polarised) {
                afs_fold(s->coord, s->dims, s->K);
            }
            afs[afs_index(s->coord, s->dims, s->K)] += inc;
        }
    }
}

/* lazy per-node flush of branch AFS (trees.c:3650-3694) */
static void branch_afs_flush(const orc_ts_t *ts, int32_t u, double right,
    double *last, const int32_t *parent, const double *x, int32_t K,
    const int64_t *dims, int64_t afs_size, int32_t TW, const double *tw, int32_t w,
    int polarised, int64_t *coord, double *result)
{
    const double *row = x + (int64_t) u * (K + 1);
    int64_t all = (int64_t) row[K];
    if (parent[u] != -1 && all > 0 && all < ts->num_samples) {
        double tu = ts->node_time[u], tv = ts->node_time[parent[u]];
        for (int32_t t = 0; t < TW && tw[t] < tv; t++) {
            for (int32_t k = 0; k < K; k++) {
                coord[k] = (int64_t) row[k];
            }
            if (!polarised) {
                afs_fold(coord, dims, K);
            }
            double hi = tw[t + 1] < tv ? tw[t + 1] : tv;
            double lo = tw[t] > tu ? tw[t] : tu;
            double bl = hi - lo > 0 ? hi - lo : 0;
            result[((int64_t) w * TW + t) * afs_size + afs_index(coord, dims, K)]
                += (right - last[u]) * bl;
        }
    }
    last[u] = right;
}

/*
 * Allele frequency spectrum.  sets: concatenated sample node ids with
 * set_sizes[K].  Result: Wn x TW x prod(set_sizes + 1).
 */
int orc_afs(const orc_ts_t *ts, int32_t K, const int64_t *set_sizes,
    const int32_t *sets, int32_t Wn, const double *windows, int32_t TW,
    const double *time_windows, uint32_t options, double *result)
{
    const int32_t N = ts->num_nodes, E = ts->num_edges, K1 = K + 1;
    const int polarised = !!(options & ORC_STAT_POLARISED);
    int64_t *dims = malloc((size_t) K * sizeof(int64_t));
    int64_t *coord = malloc((size_t) K * sizeof(int64_t));
    double *x = calloc((size_t) N * K1, sizeof(double));
    int ret = ORC_ERR_NO_MEMORY;
    int64_t afs_size = 1;
    if (!dims || !coord || !x) {
        goto out;
    }
    {
        int64_t j = 0;
        for (int32_t k = 0; k < K; k++) {
            dims[k] = set_sizes[k] + 1;
            afs_size *= dims[k];
            for (int64_t l = 0; l < set_sizes[k]; l++) {
                x[(int64_t) sets[j++] * K1 + k] = 1;
            }
        }
    }
    for (int32_t j = 0; j < ts->num_samples; j++) {
        x[(int64_t) ts->samples[j] * K1 + K] = 1;
    }
    memset(result, 0, (size_t) Wn * TW * afs_size * sizeof(double));
    if (options & ORC_STAT_BRANCH) {
        int32_t *parent = malloc((size_t) N * sizeof(int32_t));
        double *last = calloc((size_t) N, sizeof(double));
        if (!parent || !last) {
            free(parent);
            free(last);
            goto out;
        }
        for (int32_t u = 0; u < N; u++) {
            parent[u] = -1;
        }
        int32_t tj = 0, tk = 0, w = 0;
        double left = 0, L = ts->sequence_length;
        while (tj < E || left < L) {
            while (tk < E && ts->edge_right[ts->rem[tk]] == left) {
                int32_t e = ts->rem[tk++];
                int32_t ch = ts->edge_child[e];
                branch_afs_flush(ts, ch, left, last, parent, x, K, dims, afs_size, TW,
                    time_windows, w, polarised, coord, result);
                for (int32_t v = ts->edge_parent[e]; v != -1; v = parent[v]) {
                    branch_afs_flush(ts, v, left, last, parent, x, K, dims, afs_size,
                        TW, time_windows, w, polarised, coord, result);
                    for (int32_t k = 0; k < K1; k++) {
                        x[(int64_t) v * K1 + k] -= x[(int64_t) ch * K1 + k];
                    }
                }
                parent[ch] = -1;
            }
            while (tj < E && ts->edge_left[ts->ins[tj]] == left) {
                int32_t e = ts->ins[tj++];
                int32_t ch = ts->edge_child[e];
                parent[ch] = ts->edge_parent[e];
                for (int32_t v = parent[ch]; v != -1; v = parent[v]) {
                    branch_afs_flush(ts, v, left, last, parent, x, K, dims, afs_size,
                        TW, time_windows, w, polarised, coord, result);
                    for (int32_t k = 0; k < K1; k++) {
                        x[(int64_t) v * K1 + k] += x[(int64_t) ch * K1 + k];
                    }
                }
            }
            double right = L;
            if (tj < E && ts->edge_left[ts->ins[tj]] < right) {
                right = ts->edge_left[ts->ins[tj]];
            }
            if (tk < E && ts->edge_right[ts->rem[tk]] < right) {
                right = ts->edge_right[ts->rem[tk]];
            }
            while (w < Wn && windows[w + 1] <= right) {
                for (int32_t u = 0; u < N; u++) {
                    branch_afs_flush(ts, u, windows[w + 1], last, parent, x, K, dims,
                        afs_size, TW, time_windows, w, polarised, coord, result);
                }
                w++;
            }
            left = right;
        }
        free(parent);
        free(last);
        ret = 0;
    } else {
        site_afs_ctx_t s;
        int32_t max_alleles = 2;
        for (int32_t m = 0; m < ts->num_mutations; m++) {
            if (ts->mutation_allele[m] + 1 > max_alleles) {
                max_alleles = ts->mutation_allele[m] + 1;
            }
        }
        s.ts = ts;
        s.K = K;
        s.dims = dims;
        s.afs_size = afs_size;
        s.windows = windows;
        s.Wn = Wn;
        s.w = 0;
        s.polarised = polarised;
        s.result = result;
        s.states = calloc((size_t) max_alleles * K1, sizeof(double));
        s.total = calloc((size_t) K1, sizeof(double));
        s.coord = coord;
        if (!s.states || !s.total) {
            free(s.states);
            free(s.total);
            goto out;
        }
        for (int32_t k = 0; k < K; k++) {
            s.total[k] = (double) set_sizes[k];
        }
        s.total[K] = (double) ts->num_samples;
        /* the sweep wants weights by sample order: gather them from x */
        double *Wsamp = malloc((size_t) ts->num_samples * K1 * sizeof(double));
        if (!Wsamp) {
            free(s.states);
            free(s.total);
            goto out;
        }
        for (int32_t j = 0; j < ts->num_samples; j++) {
            memcpy(Wsamp + (int64_t) j * K1, x + (int64_t) ts->samples[j] * K1,
                (size_t) K1 * sizeof(double));
        }
        ret = site_sweep(ts, K1, Wsamp, site_afs_visit, &s);
        free(Wsamp);
        free(s.states);
        free(s.total);
    }
    if (ret == 0 && (options & ORC_STAT_SPAN_NORMALISE)) {
        span_normalise(Wn, windows, afs_size * TW, result);
    }
out:
    free(dims);
    free(coord);
    free(x);
    return ret;
}

/* ------------------------------------------------- relatedness matvec */
/*
 * Branch-mode genetic relatedness times a weight matrix
 * (tsk_treeseq_genetic_relatedness_vector, trees.c:10402-10816), restated
 * with the same lazy per-node accumulation.  W: num_samples x nw.
 * focal: num_focal node ids.  result: Wn x num_focal x nw.
 */
int orc_relatedness_vector(const orc_ts_t *ts, int32_t nw, const double *W, int32_t Wn,
    const double *windows, int32_t num_focal, const int32_t *focal, uint32_t options,
    double *result)
{
    const int32_t N = ts->num_nodes, E = ts->num_edges, n = ts->num_samples;
    const double *t = ts->node_time;
    int32_t *parent = malloc((size_t) N * sizeof(int32_t));
    double *xl = calloc((size_t) N, sizeof(double));
    double *v = calloc((size_t) N * nw, sizeof(double));
    double *w = calloc((size_t) N * nw, sizeof(double));
    double *mean = calloc((size_t) nw, sizeof(double));
    int ret = ORC_ERR_NO_MEMORY;
    if (!parent || !xl || !v || !w || !mean) {
        goto out;
    }
    for (int32_t u = 0; u < N; u++) {
        parent[u] = -1;
    }
    memset(result, 0, (size_t) Wn * num_focal * nw * sizeof(double));
    if (!(options & ORC_STAT_NONCENTRED)) {
        for (int32_t j = 0; j < n; j++) {
            for (int32_t k = 0; k < nw; k++) {
                mean[k] += W[(int64_t) j * nw + k];
            }
        }
        for (int32_t k = 0; k < nw; k++) {
            mean[k] /= (double) n;
        }
    }
    for (int32_t j = 0; j < n; j++) {
        for (int32_t k = 0; k < nw; k++) {
            w[(int64_t) ts->samples[j] * nw + k] = W[(int64_t) j * nw + k] - mean[k];
        }
    }
    double pos = windows[0];
#define ADD_Z(u)                                                                        \
    do {                                                                                \
        int32_t _u = (u);                                                               \
        if (parent[_u] != -1) {                                                         \
            double _f = (t[parent[_u]] - t[_u]) * (pos - xl[_u]);                       \
            for (int32_t k = 0; k < nw; k++) {                                          \
                v[(int64_t) _u * nw + k] += _f * w[(int64_t) _u * nw + k];              \
            }                                                                           \
        }                                                                               \
        xl[_u] = pos;                                                                   \
    } while (0)
#define ADJUST_UP(p0, c0, sign)                                                          \
    do {                                                                                \
        for (int32_t _p = (p0); _p != -1; _p = parent[_p]) {                            \
            ADD_Z(_p);                                                                  \
            for (int32_t k = 0; k < nw; k++) {                                          \
                v[(int64_t) (c0) *nw + k] -= (sign) *v[(int64_t) _p * nw + k];          \
                w[(int64_t) _p * nw + k] += (sign) *w[(int64_t) (c0) *nw + k];          \
            }                                                                           \
        }                                                                               \
    } while (0)
    /* position the tree at windows[0]: apply all edges covering it */
    int32_t tj = 0, tk = 0;
    while (tj < E && ts->edge_left[ts->ins[tj]] <= pos) {
        int32_t e = ts->ins[tj++];
        if (pos < ts->edge_right[e]) {
            int32_t p = ts->edge_parent[e], c = ts->edge_child[e];
            ADJUST_UP(p, c, +1.0);
            xl[c] = pos;
            parent[c] = p;
        }
    }
    while (tk < E && ts->edge_right[ts->rem[tk]] <= pos) {
        tk++;
    }
    for (int32_t m = 0; m < Wn;) {
        /* apply removals and insertions at pos */
        while (tk < E && ts->edge_right[ts->rem[tk]] == pos) {
            int32_t e = ts->rem[tk++];
            int32_t p = ts->edge_parent[e], c = ts->edge_child[e];
            ADD_Z(c);
            parent[c] = -1;
            ADJUST_UP(p, c, -1.0);
        }
        while (tj < E && ts->edge_left[ts->ins[tj]] == pos) {
            int32_t e = ts->ins[tj++];
            int32_t p = ts->edge_parent[e], c = ts->edge_child[e];
            ADJUST_UP(p, c, +1.0);
            xl[c] = pos;
            parent[c] = p;
        }
        double next = windows[m + 1];
        if (tj < E && ts->edge_left[ts->ins[tj]] < next) {
            next = ts->edge_left[ts->ins[tj]];
        }
        if (tk < E && ts->edge_right[ts->rem[tk]] < next) {
            next = ts->edge_right[ts->rem[tk]];
        }
        pos = next;
        if (pos == windows[m + 1]) {
            double *y = result + (int64_t) m * num_focal * nw;
            for (int32_t j = 0; j < num_focal; j++) {
                for (int32_t u = focal[j]; u != -1; u = parent[u]) {
                    if (xl[u] != pos) {
                        ADD_Z(u);
                    }
                    for (int32_t k = 0; k < nw; k++) {
                        y[(int64_t) j * nw + k] += v[(int64_t) u * nw + k];
                    }
                }
            }
            if (!(options & ORC_STAT_NONCENTRED)) {
                for (int32_t k = 0; k < nw; k++) {
                    double s = 0;
                    for (int32_t j = 0; j < num_focal; j++) {
                        s += y[(int64_t) j * nw + k];
                    }
                    s /= (double) num_focal;
                    for (int32_t j = 0; j < num_focal; j++) {
                        y[(int64_t) j * nw + k] -= s;
                    }
                }
            }
            memset(v, 0, (size_t) N * nw * sizeof(double));
            m++;
        }
    }
#undef ADD_Z
#undef ADJUST_UP
    if (options & ORC_STAT_SPAN_NORMALISE) {
        span_normalise(Wn, windows, (int64_t) num_focal * nw, result);
    }
    ret = 0;
out:
    free(parent);
    free(xl);
    free(v);
    free(w);
    free(mean);
    return ret;
}

/* ------------------------------------------------------ genotype matrix */
typedef struct {
    const orc_ts_t *ts;
    int32_t s0, s1;        /* decoded site range */
    int32_t *mut_at_node;
    int8_t *G;             /* (s1 - s0) x num_samples */
} geno_ctx_t;

static void geno_visit(void *vctx, int32_t site, int32_t m0, int32_t m1,
    const double *x, const int32_t *parent)
{
    (void) x;
    geno_ctx_t *g = (geno_ctx_t *) vctx;
    const orc_ts_t *ts = g->ts;
    if (site < g->s0 || site >= g->s1) {
        return;
    }
    for (int32_t m = m0; m < m1; m++) {
        g->mut_at_node[ts->mutation_node[m]] = m;
    }
    for (int32_t j = 0; j < ts->num_samples; j++) {
        int32_t a = 0;
        for (int32_t u = ts->samples[j]; u != -1; u = parent[u]) {
            if (g->mut_at_node[u] >= m0 && g->mut_at_node[u] < m1) {
                a = ts->mutation_allele[g->mut_at_node[u]];
                break;
            }
        }
        g->G[(int64_t) (site - g->s0) * ts->num_samples + j] = (int8_t) a;
    }
    for (int32_t m = m0; m < m1; m++) {
        g->mut_at_node[ts->mutation_node[m]] = -1;
    }
}

/*
 * Allele index per (site, sample) for sites [s0, s1): the allele of the
 * nearest mutation above the sample at the site (later mutations on the same
 * node win), 0 if none (c/tskit/genotypes.c, decoding with isolated samples
 * not missing).
 */
int orc_genotype_rows(const orc_ts_t *ts, int32_t s0, int32_t s1, int8_t *G)
{
    geno_ctx_t g;
    if (s0 < 0 || s1 > ts->num_sites || s1 < s0) {
        return ORC_ERR_BAD_PARAM;
    }
    int32_t *mut_at_node = malloc((size_t) ts->num_nodes * sizeof(int32_t));
    double *Wz = calloc((size_t) ts->num_samples, sizeof(double));
    int ret;
    if (!mut_at_node || !Wz) {
        free(mut_at_node);
        free(Wz);
        return ORC_ERR_NO_MEMORY;
    }
    for (int32_t u = 0; u < ts->num_nodes; u++) {
        mut_at_node[u] = -1;
    }
    g.ts = ts;
    g.s0 = s0;
    g.s1 = s1;
    g.mut_at_node = mut_at_node;
    g.G = G;
    ret = site_sweep(ts, 1, Wz, geno_visit, &g);
    free(mut_at_node);
    free(Wz);
    return ret;
}

int orc_genotype_matrix(const orc_ts_t *ts, int8_t *G)
{
    return orc_genotype_rows(ts, 0, ts->num_sites, G);
}

/*
 * Site-mode divergence matrix with every sample its own set, over sites
 * [s0, s1) in one window, unnormalised: the reference's loop
 * (c/tskit/trees.c:8685-8716 update_site_divergence, driven by
 * 8753-8826): per site the samples are grouped by allele and every pair of
 * samples carrying different alleles adds 1 to D[u][v], u < v (upper
 * triangle only, row-major num_samples x num_samples).  D is not cleared.
 */
int orc_divergence_matrix_site_range(const orc_ts_t *ts, int32_t s0, int32_t s1, double *D)
{
    const int64_t n = ts->num_samples;
    const int32_t chunk = 64;
    int8_t *G = malloc((size_t) chunk * (size_t) n);
    int32_t *A = malloc((size_t) n * sizeof(int32_t));
    int64_t *off = NULL;
    int32_t max_allele = 0;
    int ret = 0;
    if (!G || !A) {
        ret = ORC_ERR_NO_MEMORY;
        goto out;
    }
    for (int32_t c0 = s0; c0 < s1 && ret == 0; c0 += chunk) {
        const int32_t c1 = c0 + chunk < s1 ? c0 + chunk : s1;
        if ((ret = orc_genotype_rows(ts, c0, c1, G)) != 0) {
            break;
        }
        for (int32_t s = c0; s < c1; s++) {
            const int8_t *g = G + (int64_t) (s - c0) * n;
            int32_t na = 0;
            for (int64_t j = 0; j < n; j++) {
                na = g[j] + 1 > na ? g[j] + 1 : na;
            }
            if (na > max_allele) {
                free(off);
                off = malloc((size_t) (na + 1) * sizeof(int64_t));
                if (!off) {
                    ret = ORC_ERR_NO_MEMORY;
                    goto out;
                }
                max_allele = na;
            }
            /* group the samples by allele, in sample order within a group */
            for (int32_t a = 0; a <= na; a++) {
                off[a] = 0;
            }
            for (int64_t j = 0; j < n; j++) {
                off[g[j] + 1]++;
            }
            for (int32_t a = 0; a < na; a++) {
                off[a + 1] += off[a];
            }
            for (int64_t j = 0; j < n; j++) {
                A[off[g[j]]++] = (int32_t) j;
            }
            for (int32_t a = na; a > 0; a--) {
                off[a] = off[a - 1];
            }
            off[0] = 0;
            for (int32_t a = 0; a < na; a++) {
                for (int32_t b = a + 1; b < na; b++) {
                    for (int64_t j = off[a]; j < off[a + 1]; j++) {
                        for (int64_t k = off[b]; k < off[b + 1]; k++) {
                            int64_t u = A[j], v = A[k];
                            if (u > v) {
                                int64_t t = u;
                                u = v;
                                v = t;
                            }
                            D[u * n + v] += 1.0;
                        }
                    }
                }
            }
        }
    }
out:
    free(G);
    free(A);
    free(off);
    return ret;
}

/*
 * Exact per-sample sums over the mutations above each sample: for sample
 * index j,
 *   out[j][0]     = #{mutations m with j below node(m) in m's tree}
 *   out[j][1 + k] = sum over those m of x_k(node(m)),
 * x_k(u) the number of set-k samples below u in that tree (member is
 * num_samples x K, 0/1).  For infinite-sites biallelic data (one mutation per
 * site, no parent mutation) out[j][0] is sample j's derived-allele count and
 * out[j][1 + k] the number of (site, set-k sample) pairs sharing j's derived
 * allele; with set k = {i} that is the shared-derived count G[i][j].
 *
 * One tree sweep with lazy path sums, O(edges x depth x K): acc[u] holds
 * increments for every sample below u, so a sample's total is the sum of acc
 * over its root path.  Removing edge (c, p) pushes the path sum above c into
 * acc[c]; inserting one subtracts the new path sum above c; at the end every
 * edge is removed and a sample's total is its own acc.
 */
int orc_site_path_sums(const orc_ts_t *ts, int32_t K, const uint8_t *member, int64_t *out)
{
    const int32_t N = ts->num_nodes, E = ts->num_edges, A = K + 1;
    int32_t *parent = malloc((size_t) N * sizeof(int32_t));
    int64_t *x = calloc((size_t) N * (size_t) (K > 0 ? K : 1), sizeof(int64_t));
    int64_t *acc = calloc((size_t) N * (size_t) A, sizeof(int64_t));
    int64_t *sum = calloc((size_t) A, sizeof(int64_t));
    if (!parent || !x || !acc || !sum) {
        free(parent);
        free(x);
        free(acc);
        free(sum);
        return ORC_ERR_NO_MEMORY;
    }
    for (int32_t u = 0; u < N; u++) {
        parent[u] = -1;
    }
    for (int32_t j = 0; j < ts->num_samples; j++) {
        for (int32_t k = 0; k < K; k++) {
            x[(int64_t) ts->samples[j] * K + k] = member[(int64_t) j * K + k];
        }
    }
    int32_t tj = 0, tk = 0, mut = 0;
    double left = 0, L = ts->sequence_length;
    for (;;) {
        const int done = !(tj < E || left < L);
        while (tk < E && (done || ts->edge_right[ts->rem[tk]] == left)) {
            int32_t e = ts->rem[tk++];
            int32_t ch = ts->edge_child[e];
            memset(sum, 0, (size_t) A * sizeof(int64_t));
            for (int32_t u = ts->edge_parent[e]; u != -1; u = parent[u]) {
                for (int32_t a = 0; a < A; a++) {
                    sum[a] += acc[(int64_t) u * A + a];
                }
                for (int32_t k = 0; k < K; k++) {
                    x[(int64_t) u * K + k] -= x[(int64_t) ch * K + k];
                }
            }
            for (int32_t a = 0; a < A; a++) {
                acc[(int64_t) ch * A + a] += sum[a];
            }
            parent[ch] = -1;
        }
        if (done) {
            break;
        }
        while (tj < E && ts->edge_left[ts->ins[tj]] == left) {
            int32_t e = ts->ins[tj++];
            int32_t ch = ts->edge_child[e];
            parent[ch] = ts->edge_parent[e];
            memset(sum, 0, (size_t) A * sizeof(int64_t));
            for (int32_t u = parent[ch]; u != -1; u = parent[u]) {
                for (int32_t a = 0; a < A; a++) {
                    sum[a] += acc[(int64_t) u * A + a];
                }
                for (int32_t k = 0; k < K; k++) {
                    x[(int64_t) u * K + k] += x[(int64_t) ch * K + k];
                }
            }
            for (int32_t a = 0; a < A; a++) {
                acc[(int64_t) ch * A + a] -= sum[a];
            }
        }
        double right = L;
        if (tj < E && ts->edge_left[ts->ins[tj]] < right) {
            right = ts->edge_left[ts->ins[tj]];
        }
        if (tk < E && ts->edge_right[ts->rem[tk]] < right) {
            right = ts->edge_right[ts->rem[tk]];
        }
        while (mut < ts->num_mutations
               && ts->site_position[ts->mutation_site[mut]] < right) {
            const int32_t u = ts->mutation_node[mut++];
            acc[(int64_t) u * A] += 1;
            for (int32_t k = 0; k < K; k++) {
                acc[(int64_t) u * A + 1 + k] += x[(int64_t) u * K + k];
            }
        }
        left = right;
    }
    for (int32_t j = 0; j < ts->num_samples; j++) {
        memcpy(out + (int64_t) j * A, acc + (int64_t) ts->samples[j] * A,
            (size_t) A * sizeof(int64_t));
    }
    free(parent);
    free(x);
    free(acc);
    free(sum);
    return 0;
}
