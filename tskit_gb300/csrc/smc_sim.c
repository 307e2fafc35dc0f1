/*
 * Seeded SMC-style generator of synthetic tree sequences.
 *
 * This is the input generator for the benchmarks and the large parity cases
 * (the reference measures its statistics on no public data set).  Model:
 *
 *   1. A Kingman coalescent tree of n haploid samples at time 0: with k
 *      lineages the waiting time is Exp(k(k-1)/2) and a uniformly random pair
 *      merges.  Node times are float64.
 *   2. B recombination breakpoints uniform on [0, L).  At each one a branch
 *      is chosen with probability proportional to its length, cut at a
 *      uniform time on it, and the detached lineage re-coalesces above that
 *      time with the remaining tree at rate equal to the number of remaining
 *      lineages, onto a uniformly chosen lineage (subtree prune and regraft).
 *   3. Infinite-sites biallelic mutations: for each marginal tree, a Poisson
 *      number of sites with mean mu * span * total_branch_length, positions
 *      uniform on the tree's interval, each with one mutation on a branch
 *      chosen proportional to length.  mu is chosen so that the expected
 *      number of sites equals the requested target.
 *
 * Every tree is binary and every node is ancestral to samples, so the output
 * is already simplified; node 0..n-1 are the samples.  Random numbers come
 * from xoshiro256** seeded through splitmix64.
 *
 * Data structures (all O(log N) per operation):
 *   - a segment tree over node ids holding branch lengths (length-biased
 *     branch choice for cuts and mutations),
 *   - a treap over internal nodes keyed by (time, id) with subtree counts and
 *     time sums, used to invert the re-coalescence hazard
 *     H(T) = int_t^T k(tau) dtau with k(tau) = 1 + #{internal nodes above tau},
 *     and for order statistics when drawing a lineage by rejection.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------ rng */
typedef struct {
    uint64_t s[4];
} rng_t;

static uint64_t splitmix64(uint64_t *x)
{
    uint64_t z = (*x += 0x9e3779b97f4a7c15ULL);
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
    return z ^ (z >> 31);
}

static inline uint64_t rotl64(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }

static inline uint64_t rng_next(rng_t *r)
{
    uint64_t *s = r->s;
    const uint64_t result = rotl64(s[1] * 5, 7) * 9;
    const uint64_t t = s[1] << 17;
    s[2] ^= s[0];
    s[3] ^= s[1];
    s[1] ^= s[2];
    s[0] ^= s[3];
    s[2] ^= t;
    s[3] = rotl64(s[3], 45);
    return result;
}

static void rng_seed(rng_t *r, uint64_t seed)
{
    uint64_t x = seed;
    for (int j = 0; j < 4; j++) {
        r->s[j] = splitmix64(&x);
    }
}

/* uniform on [0, 1) */
static inline double rng_unif(rng_t *r) { return (double) (rng_next(r) >> 11) * 0x1.0p-53; }

/* uniform integer on [0, m) */
static inline int64_t rng_int(rng_t *r, int64_t m)
{
    return (int64_t) (rng_unif(r) * (double) m) % m;
}

static inline double rng_exp(rng_t *r) { return -log1p(-rng_unif(r)); }

static int64_t rng_poisson(rng_t *r, double lambda)
{
    /* Poisson additivity: sum of Knuth draws with mean <= 16 each. */
    int64_t total = 0;
    while (lambda > 0) {
        double l = lambda > 16.0 ? 16.0 : lambda;
        double L = exp(-l), p = 1.0;
        int64_t k = 0;
        do {
            k++;
            p *= rng_unif(r);
        } while (p > L);
        total += k - 1;
        lambda -= l;
    }
    return total;
}

/* ----------------------------------------------------------- segment tree */
typedef struct {
    int64_t size; /* power of two */
    double *sum;  /* 2*size */
} segtree_t;

static int seg_init(segtree_t *t, int64_t n)
{
    t->size = 1;
    while (t->size < n) {
        t->size <<= 1;
    }
    t->sum = calloc((size_t) (2 * t->size), sizeof(double));
    return t->sum == NULL ? -1 : 0;
}

static void seg_set(segtree_t *t, int64_t i, double w)
{
    int64_t j = t->size + i;
    t->sum[j] = w;
    for (j >>= 1; j >= 1; j >>= 1) {
        t->sum[j] = t->sum[2 * j] + t->sum[2 * j + 1];
    }
}

static int64_t seg_sample(segtree_t *t, rng_t *r)
{
    for (;;) {
        double x = rng_unif(r) * t->sum[1];
        int64_t j = 1;
        while (j < t->size) {
            if (x < t->sum[2 * j] || t->sum[2 * j + 1] <= 0) {
                j = 2 * j;
            } else {
                x -= t->sum[2 * j];
                j = 2 * j + 1;
            }
        }
        if (t->sum[j] > 0) {
            return j - t->size;
        }
    }
}

/* ------------------------------------------------------------------ treap */
typedef struct {
    int32_t *l, *r;
    uint32_t *prio;
    int32_t *cnt;
    double *tsum;
    const double *time;
    int32_t root;
} treap_t;

static inline int treap_less(const treap_t *T, int32_t a, int32_t b)
{
    return T->time[a] < T->time[b] || (T->time[a] == T->time[b] && a < b);
}

static inline void treap_pull(treap_t *T, int32_t x)
{
    int32_t a = T->l[x], b = T->r[x];
    T->cnt[x] = 1 + (a >= 0 ? T->cnt[a] : 0) + (b >= 0 ? T->cnt[b] : 0);
    T->tsum[x] = T->time[x] + (a >= 0 ? T->tsum[a] : 0) + (b >= 0 ? T->tsum[b] : 0);
}

/* split into keys < k and keys >= k, where k is node id `key` */
static void treap_split(treap_t *T, int32_t x, int32_t key, int32_t *a, int32_t *b)
{
    if (x < 0) {
        *a = *b = -1;
        return;
    }
    if (treap_less(T, x, key)) {
        treap_split(T, T->r[x], key, &T->r[x], b);
        *a = x;
    } else {
        treap_split(T, T->l[x], key, a, &T->l[x]);
        *b = x;
    }
    treap_pull(T, x);
}

static int32_t treap_merge(treap_t *T, int32_t a, int32_t b)
{
    if (a < 0) {
        return b;
    }
    if (b < 0) {
        return a;
    }
    if (T->prio[a] > T->prio[b]) {
        T->r[a] = treap_merge(T, T->r[a], b);
        treap_pull(T, a);
        return a;
    }
    T->l[b] = treap_merge(T, a, T->l[b]);
    treap_pull(T, b);
    return b;
}

static void treap_insert(treap_t *T, int32_t x)
{
    int32_t a, b;
    T->l[x] = T->r[x] = -1;
    treap_pull(T, x);
    treap_split(T, T->root, x, &a, &b);
    T->root = treap_merge(T, treap_merge(T, a, x), b);
}

/* split into keys <= k and keys > k */
static void treap_split_le(treap_t *T, int32_t x, int32_t key, int32_t *a, int32_t *b)
{
    if (x < 0) {
        *a = *b = -1;
        return;
    }
    if (!treap_less(T, key, x)) {
        treap_split_le(T, T->r[x], key, &T->r[x], b);
        *a = x;
    } else {
        treap_split_le(T, T->l[x], key, a, &T->l[x]);
        *b = x;
    }
    treap_pull(T, x);
}

static void treap_erase(treap_t *T, int32_t x)
{
    int32_t a, b, mid, c;
    treap_split(T, T->root, x, &a, &b);      /* a: < x, b: >= x */
    treap_split_le(T, b, x, &mid, &c);       /* mid: == x, c: > x */
    T->root = treap_merge(T, a, c);
}

/* count and time-sum of nodes with time <= t (all ids) */
static void treap_prefix(const treap_t *T, double t, int64_t *cnt, double *sum)
{
    int32_t x = T->root;
    int64_t c = 0;
    double s = 0;
    while (x >= 0) {
        if (T->time[x] <= t) {
            int32_t a = T->l[x];
            c += 1 + (a >= 0 ? T->cnt[a] : 0);
            s += T->time[x] + (a >= 0 ? T->tsum[a] : 0);
            x = T->r[x];
        } else {
            x = T->l[x];
        }
    }
    *cnt = c;
    *sum = s;
}

/* j-th smallest (0-based) */
static int32_t treap_select(const treap_t *T, int64_t j)
{
    int32_t x = T->root;
    while (x >= 0) {
        int32_t a = T->l[x];
        int64_t ca = a >= 0 ? T->cnt[a] : 0;
        if (j < ca) {
            x = a;
        } else if (j == ca) {
            return x;
        } else {
            j -= ca + 1;
            x = T->r[x];
        }
    }
    return -1;
}

/*
 * Invert the hazard: given start time t and target E, return T with
 * H(T) = (T - t)(1 + #{u: t_u > T}) + sum_{t < t_u <= T} (t_u - t) = E,
 * where u ranges over the treap's nodes.
 */
static double treap_hazard_invert(const treap_t *T, double t, double E)
{
    int64_t c0, total;
    double s0;
    treap_prefix(T, t, &c0, &s0);
    total = T->root >= 0 ? T->cnt[T->root] : 0;
    const int64_t nA = total - c0;
    double best_tau = t, best_H = 0;
    int64_t best_gt = nA;
    int32_t x = T->root;
    int64_t acc_c = 0;
    double acc_s = 0;
    while (x >= 0) {
        int32_t a = T->l[x];
        int64_t cle = acc_c + (a >= 0 ? T->cnt[a] : 0) + 1;
        double sle = acc_s + (a >= 0 ? T->tsum[a] : 0) + T->time[x];
        if (T->time[x] <= t) {
            acc_c = cle;
            acc_s = sle;
            x = T->r[x];
            continue;
        }
        int64_t cA = cle - c0;
        double sA = sle - s0;
        int64_t gt = nA - cA;
        double tau = T->time[x];
        double H = (tau - t) * (double) (1 + gt) + (sA - t * (double) cA);
        if (H <= E) {
            best_tau = tau;
            best_H = H;
            best_gt = gt;
            acc_c = cle;
            acc_s = sle;
            x = T->r[x];
        } else {
            x = T->l[x];
        }
    }
    return best_tau + (E - best_H) / (double) (1 + best_gt);
}

/* ------------------------------------------------------------ generator */
typedef struct {
    int64_t n, cap_nodes;
    int64_t num_nodes;
    double *time;
    int32_t *parent, *c0, *c1;
    double *edge_start;
    /* output edges */
    int64_t num_edges, cap_edges;
    double *el, *er;
    int32_t *ep, *ec;
    /* output sites */
    int64_t num_sites, cap_sites;
    double *site_pos;
    int32_t *mut_node;
    int32_t root;
} smc_state_t;

typedef struct {
    int64_t num_nodes, num_edges, num_sites, num_samples;
    double *node_time;
    double *edge_left, *edge_right;
    int32_t *edge_parent, *edge_child;
    double *site_position;
    int32_t *mutation_node;
} smc_result_t;

static int grow_edges(smc_state_t *S)
{
    if (S->num_edges < S->cap_edges) {
        return 0;
    }
    int64_t cap = S->cap_edges * 2 + 1024;
    double *el = realloc(S->el, (size_t) cap * sizeof(double));
    double *er = realloc(S->er, (size_t) cap * sizeof(double));
    int32_t *ep = realloc(S->ep, (size_t) cap * sizeof(int32_t));
    int32_t *ec = realloc(S->ec, (size_t) cap * sizeof(int32_t));
    if (!el || !er || !ep || !ec) {
        return -1;
    }
    S->el = el;
    S->er = er;
    S->ep = ep;
    S->ec = ec;
    S->cap_edges = cap;
    return 0;
}

static int grow_sites(smc_state_t *S, int64_t extra)
{
    if (S->num_sites + extra <= S->cap_sites) {
        return 0;
    }
    int64_t cap = (S->cap_sites + extra) * 2 + 1024;
    double *p = realloc(S->site_pos, (size_t) cap * sizeof(double));
    int32_t *m = realloc(S->mut_node, (size_t) cap * sizeof(int32_t));
    if (!p || !m) {
        return -1;
    }
    S->site_pos = p;
    S->mut_node = m;
    S->cap_sites = cap;
    return 0;
}

/* close the edge above u at position x */
static int end_edge(smc_state_t *S, int32_t u, double x)
{
    if (S->parent[u] >= 0 && x > S->edge_start[u]) {
        if (grow_edges(S) != 0) {
            return -1;
        }
        S->el[S->num_edges] = S->edge_start[u];
        S->er[S->num_edges] = x;
        S->ep[S->num_edges] = S->parent[u];
        S->ec[S->num_edges] = u;
        S->num_edges++;
    }
    return 0;
}

static inline void set_branch(smc_state_t *S, segtree_t *seg, int32_t u)
{
    double w = S->parent[u] >= 0 ? S->time[S->parent[u]] - S->time[u] : 0.0;
    seg_set(seg, u, w);
}

static int cmp_double(const void *a, const void *b)
{
    double x = *(const double *) a, y = *(const double *) b;
    return (x > y) - (x < y);
}

static int add_sites(smc_state_t *S, segtree_t *seg, rng_t *r, double a, double b,
    double mu, double *scratch_pos, int64_t scratch_cap)
{
    double lam = mu * (b - a) * seg->sum[1];
    int64_t k = rng_poisson(r, lam);
    if (k == 0) {
        return 0;
    }
    if (k > scratch_cap) {
        k = scratch_cap;
    }
    for (int64_t j = 0; j < k; j++) {
        scratch_pos[j] = a + rng_unif(r) * (b - a);
    }
    qsort(scratch_pos, (size_t) k, sizeof(double), cmp_double);
    if (grow_sites(S, k) != 0) {
        return -1;
    }
    for (int64_t j = 0; j < k; j++) {
        double x = scratch_pos[j];
        int32_t u = (int32_t) seg_sample(seg, r);
        if (S->num_sites > 0 && x <= S->site_pos[S->num_sites - 1]) {
            continue; /* keep positions strictly increasing */
        }
        S->site_pos[S->num_sites] = x;
        S->mut_node[S->num_sites] = u;
        S->num_sites++;
    }
    return 0;
}

static void free_state(smc_state_t *S)
{
    free(S->time);
    free(S->parent);
    free(S->c0);
    free(S->c1);
    free(S->edge_start);
    free(S->el);
    free(S->er);
    free(S->ep);
    free(S->ec);
    free(S->site_pos);
    free(S->mut_node);
}

/*
 * Run the generator.  Returns 0 on success and fills *out (free with
 * smc_free_result).  sites_target is the expected number of sites.
 */
int smc_simulate(int64_t n, double L, int64_t num_breakpoints, double sites_target,
    uint64_t seed, smc_result_t *out)
{
    int ret = -1;
    rng_t rng;
    smc_state_t S;
    segtree_t seg = { 0, NULL };
    treap_t T;
    double *bps = NULL, *scratch = NULL;
    int32_t *cand = NULL, *stack = NULL, *lineages = NULL;
    int64_t scratch_cap = 1 << 16;

    memset(&S, 0, sizeof(S));
    memset(&T, 0, sizeof(T));
    memset(out, 0, sizeof(*out));
    if (n < 2 || L <= 0 || num_breakpoints < 0) {
        return -2;
    }
    rng_seed(&rng, seed);
    S.n = n;
    S.cap_nodes = 2 * n + num_breakpoints + 8;
    S.time = calloc((size_t) S.cap_nodes, sizeof(double));
    S.parent = malloc((size_t) S.cap_nodes * sizeof(int32_t));
    S.c0 = malloc((size_t) S.cap_nodes * sizeof(int32_t));
    S.c1 = malloc((size_t) S.cap_nodes * sizeof(int32_t));
    S.edge_start = calloc((size_t) S.cap_nodes, sizeof(double));
    T.l = malloc((size_t) S.cap_nodes * sizeof(int32_t));
    T.r = malloc((size_t) S.cap_nodes * sizeof(int32_t));
    T.prio = malloc((size_t) S.cap_nodes * sizeof(uint32_t));
    T.cnt = malloc((size_t) S.cap_nodes * sizeof(int32_t));
    T.tsum = malloc((size_t) S.cap_nodes * sizeof(double));
    T.time = S.time;
    T.root = -1;
    bps = malloc((size_t) (num_breakpoints + 1) * sizeof(double));
    scratch = malloc((size_t) scratch_cap * sizeof(double));
    lineages = malloc((size_t) n * sizeof(int32_t));
    stack = malloc((size_t) S.cap_nodes * sizeof(int32_t));
    cand = malloc((size_t) S.cap_nodes * sizeof(int32_t));
    if (!S.time || !S.parent || !S.c0 || !S.c1 || !S.edge_start || !T.l || !T.r
        || !T.prio || !T.cnt || !T.tsum || !bps || !scratch || !lineages || !stack
        || !cand || seg_init(&seg, S.cap_nodes) != 0) {
        goto out;
    }
    for (int64_t j = 0; j < S.cap_nodes; j++) {
        S.parent[j] = S.c0[j] = S.c1[j] = -1;
        T.prio[j] = (uint32_t) (rng_next(&rng) >> 32);
    }

    /* 1. Kingman tree */
    for (int64_t j = 0; j < n; j++) {
        lineages[j] = (int32_t) j;
        S.time[j] = 0.0;
    }
    S.num_nodes = n;
    {
        double t = 0;
        int64_t k = n;
        while (k > 1) {
            t += rng_exp(&rng) / ((double) k * (double) (k - 1) / 2.0);
            int64_t a = rng_int(&rng, k);
            int64_t b = rng_int(&rng, k - 1);
            if (b >= a) {
                b++;
            }
            int32_t u = (int32_t) S.num_nodes++;
            S.time[u] = t;
            S.c0[u] = lineages[a];
            S.c1[u] = lineages[b];
            S.parent[lineages[a]] = u;
            S.parent[lineages[b]] = u;
            S.edge_start[lineages[a]] = 0;
            S.edge_start[lineages[b]] = 0;
            /* remove a and b, add u */
            if (a < b) {
                int64_t tmp = a;
                a = b;
                b = tmp;
            }
            lineages[a] = lineages[k - 1];
            lineages[b] = u;
            k--;
            treap_insert(&T, u);
        }
        S.root = lineages[0];
    }
    for (int64_t u = 0; u < S.num_nodes; u++) {
        set_branch(&S, &seg, (int32_t) u);
    }

    /* mutation rate giving the requested expected number of sites */
    double harmonic = 0;
    for (int64_t k = 1; k < n; k++) {
        harmonic += 1.0 / (double) k;
    }
    const double mu = sites_target / (L * 2.0 * harmonic);

    /* 2. breakpoints */
    for (int64_t j = 0; j < num_breakpoints; j++) {
        bps[j] = rng_unif(&rng) * L;
    }
    qsort(bps, (size_t) num_breakpoints, sizeof(double), cmp_double);

    double last_x = 0;
    const int64_t K0 = (int64_t) sqrt(2.0 * (double) n) + 8;
    for (int64_t bi = 0; bi < num_breakpoints; bi++) {
        double x = bps[bi];
        if (x <= last_x) {
            continue;
        }
        if (add_sites(&S, &seg, &rng, last_x, x, mu, scratch, scratch_cap) != 0) {
            goto out;
        }
        last_x = x;

        /* choose the branch to cut */
        int32_t c = (int32_t) seg_sample(&seg, &rng);
        int32_t p = S.parent[c];
        int32_t s = S.c0[p] == c ? S.c1[p] : S.c0[p];
        int32_t gp = S.parent[p];
        double tcut = S.time[c] + rng_unif(&rng) * (S.time[p] - S.time[c]);

        /* detach c and dissolve p */
        if (end_edge(&S, c, x) || end_edge(&S, s, x) || end_edge(&S, p, x)) {
            goto out;
        }
        S.parent[c] = -1;
        S.parent[p] = -1;
        S.c0[p] = S.c1[p] = -1;
        treap_erase(&T, p);
        if (gp >= 0) {
            if (S.c0[gp] == p) {
                S.c0[gp] = s;
            } else {
                S.c1[gp] = s;
            }
            S.parent[s] = gp;
            S.edge_start[s] = x;
        } else {
            S.parent[s] = -1;
            S.root = s;
        }
        seg_set(&seg, c, 0);
        seg_set(&seg, p, 0);
        set_branch(&S, &seg, s);

        /* re-coalescence time */
        double Tn = treap_hazard_invert(&T, tcut, rng_exp(&rng));
        int64_t cle;
        double sle;
        treap_prefix(&T, Tn, &cle, &sle);
        int64_t total_int = T.root >= 0 ? T.cnt[T.root] : 0;
        int64_t k = 1 + (total_int - cle);

        /* choose a lineage of the remaining tree at time Tn */
        int32_t d = -1;
        if (k <= K0) {
            int64_t ns = 0, nc = 0;
            stack[ns++] = S.root;
            while (ns > 0) {
                int32_t u = stack[--ns];
                if (S.time[u] <= Tn) {
                    cand[nc++] = u;
                } else {
                    stack[ns++] = S.c0[u];
                    stack[ns++] = S.c1[u];
                }
            }
            d = cand[rng_int(&rng, nc)];
        } else {
            for (;;) {
                int64_t j = rng_int(&rng, n + cle);
                int32_t u = j < n ? (int32_t) j : treap_select(&T, j - n);
                if (u == c) {
                    continue;
                }
                if (S.parent[u] >= 0) {
                    if (S.time[S.parent[u]] > Tn) {
                        d = u;
                        break;
                    }
                } else if (u == S.root) {
                    d = u;
                    break;
                }
            }
        }

        /* new node q above d and c */
        int32_t q = (int32_t) S.num_nodes++;
        int32_t pd = S.parent[d];
        S.time[q] = Tn;
        if (pd >= 0) {
            if (end_edge(&S, d, x)) {
                goto out;
            }
            if (S.c0[pd] == d) {
                S.c0[pd] = q;
            } else {
                S.c1[pd] = q;
            }
            S.parent[q] = pd;
            S.edge_start[q] = x;
        } else {
            S.parent[q] = -1;
            S.root = q;
        }
        S.c0[q] = c;
        S.c1[q] = d;
        S.parent[c] = q;
        S.parent[d] = q;
        S.edge_start[c] = x;
        S.edge_start[d] = x;
        treap_insert(&T, q);
        set_branch(&S, &seg, c);
        set_branch(&S, &seg, d);
        set_branch(&S, &seg, q);
    }
    if (add_sites(&S, &seg, &rng, last_x, L, mu, scratch, scratch_cap) != 0) {
        goto out;
    }
    for (int64_t u = 0; u < S.num_nodes; u++) {
        if (end_edge(&S, (int32_t) u, L) != 0) {
            goto out;
        }
    }

    out->num_nodes = S.num_nodes;
    out->num_edges = S.num_edges;
    out->num_sites = S.num_sites;
    out->num_samples = n;
    out->node_time = S.time;
    out->edge_left = S.el;
    out->edge_right = S.er;
    out->edge_parent = S.ep;
    out->edge_child = S.ec;
    out->site_position = S.site_pos;
    out->mutation_node = S.mut_node;
    S.time = NULL;
    S.el = S.er = NULL;
    S.ep = S.ec = NULL;
    S.site_pos = NULL;
    S.mut_node = NULL;
    ret = 0;
out:
    free_state(&S);
    free(seg.sum);
    free(T.l);
    free(T.r);
    free(T.prio);
    free(T.cnt);
    free(T.tsum);
    free(bps);
    free(scratch);
    free(lineages);
    free(stack);
    free(cand);
    return ret;
}

void smc_free_result(smc_result_t *r)
{
    free(r->node_time);
    free(r->edge_left);
    free(r->edge_right);
    free(r->edge_parent);
    free(r->edge_child);
    free(r->site_position);
    free(r->mutation_node);
    memset(r, 0, sizeof(*r));
}
