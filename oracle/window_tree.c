/*
 * Seeded window-tree genotype graph for the oracle -- TEST INFRASTRUCTURE ONLY.
 *
 * The benchmark's synthetic workload, generated inside the oracle library so that the CPU
 * baseline and the reference arm of the benchmark build their graph without loading the
 * product library.  It is an independent C statement of the generator the product uses
 * (same seeds, same arithmetic, same node numbering), so both produce the same graph bit for
 * bit; a CPU test compares them.
 *
 * For window w (variants [w*W, min((w+1)*W, M))), from a SplitMix64 stream (Steele, Lea and
 * Flood's published generator) seeded with seed ^ w:
 *   - a Kingman coalescent tree over all N samples: with k lineages the waiting time is
 *     Exp(k(k-1)/2) (drawn as -ln(1-u)/rate) and a uniformly random pair merges;
 *   - one branch per variant, chosen with probability proportional to branch length; the
 *     variant's carriers are the leaves below it.
 * The tree is collapsed to its mutated nodes (a GRG built straight from a tree, the idea of
 * the reference's tree-sequence converter src/ts2grg.cpp): every mutated internal branch is a
 * node whose children are its nearest mutated descendants and the samples with no mutated node
 * in between; a mutation on a leaf branch maps to the sample itself.
 *
 * Node ids: samples 0..N-1, then each window's mutated internal nodes in tree order (children
 * before parents), windows in order, so the graph is topologically ordered and every child list
 * ascends.  Floating point is +, -, *, / and a series logarithm, compiled without FMA
 * contraction, so every platform generates the same graph.
 */
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define WT_INVALID 0xffffffffu
#define WT_INVALID_NODE 0x7fffffffu

typedef struct {
    uint64_t s;
} splitmix64;

static uint64_t sm_next(splitmix64* r) {
    uint64_t z = (r->s += 0x9e3779b97f4a7c15ull);
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}

/* uniform in [0, 1) from the top 53 bits */
static double sm_uniform(splitmix64* r) { return (double)(sm_next(r) >> 11) * (1.0 / 9007199254740992.0); }

/* uniform integer in [0, k): the high 64 bits of next * k */
static uint64_t sm_below(splitmix64* r, uint64_t k) {
    return (uint64_t)(((unsigned __int128)sm_next(r) * k) >> 64);
}

/* ln x for x > 0: x = m 2^e with m in [sqrt(1/2), sqrt(2)), ln m = 2 atanh(z), z = (m-1)/(m+1),
 * summed to the z^25 term (|z| < 0.172: past double precision). */
static double series_log(double x) {
    int e = 0;
    double m = x;
    while (m > 1.4142135623730951) {
        m *= 0.5;
        e++;
    }
    while (m < 0.7071067811865476) {
        m *= 2.0;
        e--;
    }
    const double z = (m - 1.0) / (m + 1.0);
    const double z2 = z * z;
    double term = z, sum = 0.0;
    for (int k = 1; k <= 25; k += 2) {
        sum += term / (double)k;
        term *= z2;
    }
    return (double)e * 0.6931471805599453 + 2.0 * sum;
}

/* One window's collapsed tree: `num_nodes` new nodes with children (sample id < N, or N + local
 * index of another new node) and, per variant, the sample or N + local index it maps to. */
typedef struct {
    uint32_t num_nodes;
    uint32_t* off; /* num_nodes + 1 */
    uint32_t* adj;
    uint32_t* mut_local;
    uint32_t nvar;
} window_out;

typedef struct {
    uint32_t *lin, *parent, *nma, *branch;
    int32_t* local;
    uint8_t* mutated;
    double *time, *cum;
} window_scratch;

static int scratch_alloc(window_scratch* w, uint64_t N, uint32_t W) {
    const uint64_t T = 2 * N - 1;
    w->lin = (uint32_t*)malloc(sizeof(uint32_t) * N);
    w->parent = (uint32_t*)malloc(sizeof(uint32_t) * T);
    w->nma = (uint32_t*)malloc(sizeof(uint32_t) * T);
    w->branch = (uint32_t*)malloc(sizeof(uint32_t) * (W ? W : 1));
    w->local = (int32_t*)malloc(sizeof(int32_t) * T);
    w->mutated = (uint8_t*)malloc(T);
    w->time = (double*)malloc(sizeof(double) * T);
    w->cum = (double*)malloc(sizeof(double) * T);
    return w->lin && w->parent && w->nma && w->branch && w->local && w->mutated && w->time && w->cum;
}

static void scratch_free(window_scratch* w) {
    free(w->lin);
    free(w->parent);
    free(w->nma);
    free(w->branch);
    free(w->local);
    free(w->mutated);
    free(w->time);
    free(w->cum);
}

static void window_free(window_out* o) {
    free(o->off);
    free(o->adj);
    free(o->mut_local);
    memset(o, 0, sizeof(*o));
}

static int simulate_window(uint64_t N, uint64_t seed, uint64_t w, uint32_t nvar, window_out* out, window_scratch* sc) {
    if (N < 2 || N >= 0x40000000ull) return -2;
    splitmix64 rng = {seed ^ w};
    const uint64_t T = 2 * N - 1; /* leaves 0..N-1, internal N..2N-2, root 2N-2 */
    const uint64_t root = T - 1;
    for (uint64_t i = 0; i < N; i++) sc->lin[i] = (uint32_t)i;
    for (uint64_t v = 0; v < T; v++) {
        sc->parent[v] = WT_INVALID;
        sc->time[v] = 0.0;
    }
    /* Kingman merges: k lineages, waiting time Exp(k(k-1)/2), a random pair (i, j != i) merges
     * into the next internal node, which takes slot i; slot j takes the last lineage. */
    double t = 0.0;
    uint64_t next = N;
    for (uint64_t k = N; k > 1; k--) {
        const double rate = 0.5 * (double)k * (double)(k - 1);
        t += -series_log(1.0 - sm_uniform(&rng)) / rate;
        const uint64_t i = sm_below(&rng, k);
        uint64_t j = sm_below(&rng, k - 1);
        if (j >= i) j++;
        const uint32_t p = (uint32_t)(next++);
        sc->parent[sc->lin[i]] = p;
        sc->parent[sc->lin[j]] = p;
        sc->time[p] = t;
        sc->lin[i] = p;
        sc->lin[j] = sc->lin[k - 1];
    }
    /* branch-length prefix sums over the non-root nodes, in node order */
    double acc = 0.0;
    for (uint64_t v = 0; v < root; v++) {
        acc += sc->time[sc->parent[v]] - sc->time[v];
        sc->cum[v] = acc;
    }
    /* each variant's branch: the first node whose prefix sum exceeds u * total */
    for (uint32_t j = 0; j < nvar; j++) {
        const double u = sm_uniform(&rng) * acc;
        uint64_t lo = 0, hi = root;
        while (lo < hi) {
            const uint64_t mid = (lo + hi) >> 1;
            if (sc->cum[mid] > u) hi = mid;
            else lo = mid + 1;
        }
        if (lo >= root) lo = root - 1;
        sc->branch[j] = (uint32_t)lo;
    }
    /* mutated internal nodes get local ids in tree-node order */
    memset(sc->mutated, 0, T);
    for (uint32_t j = 0; j < nvar; j++) sc->mutated[sc->branch[j]] = 1;
    uint32_t cnt = 0;
    for (uint64_t v = 0; v < T; v++) sc->local[v] = -1;
    for (uint64_t v = N; v < T; v++)
        if (sc->mutated[v]) sc->local[v] = (int32_t)(cnt++);
    /* nearest mutated strict ancestor, parents before children (descending node order) */
    for (uint64_t v = 0; v < T; v++) sc->nma[v] = WT_INVALID;
    for (uint64_t vv = root; vv > 0; vv--) {
        const uint64_t v = vv - 1;
        const uint32_t p = sc->parent[v];
        sc->nma[v] = sc->mutated[p] ? p : sc->nma[p];
    }
    /* children lists: samples ascending, then mutated internal nodes ascending */
    out->num_nodes = cnt;
    out->nvar = nvar;
    out->off = (uint32_t*)calloc((size_t)cnt + 1, sizeof(uint32_t));
    out->mut_local = (uint32_t*)malloc(sizeof(uint32_t) * (nvar ? nvar : 1));
    if (!out->off || !out->mut_local) return -1;
    for (uint64_t s = 0; s < N; s++)
        if (sc->nma[s] != WT_INVALID) out->off[sc->local[sc->nma[s]] + 1]++;
    for (uint64_t v = N; v < root; v++)
        if (sc->mutated[v] && sc->nma[v] != WT_INVALID) out->off[sc->local[sc->nma[v]] + 1]++;
    for (uint32_t i = 0; i < cnt; i++) out->off[i + 1] += out->off[i];
    out->adj = (uint32_t*)malloc(sizeof(uint32_t) * (out->off[cnt] ? out->off[cnt] : 1));
    uint32_t* fill = (uint32_t*)malloc(sizeof(uint32_t) * (cnt ? cnt : 1));
    if (!out->adj || !fill) {
        free(fill);
        return -1;
    }
    memcpy(fill, out->off, sizeof(uint32_t) * cnt);
    for (uint64_t s = 0; s < N; s++)
        if (sc->nma[s] != WT_INVALID) out->adj[fill[sc->local[sc->nma[s]]]++] = (uint32_t)s;
    for (uint64_t v = N; v < root; v++)
        if (sc->mutated[v] && sc->nma[v] != WT_INVALID)
            out->adj[fill[sc->local[sc->nma[v]]]++] = (uint32_t)(N + (uint64_t)sc->local[v]);
    free(fill);
    for (uint32_t j = 0; j < nvar; j++) {
        const uint32_t b = sc->branch[j];
        out->mut_local[j] = (b < N) ? b : (uint32_t)(N + (uint64_t)sc->local[b]);
    }
    return 0;
}

typedef struct {
    uint64_t N, M, seed, w0, w1;
    uint32_t W;
    window_out* outs; /* indexed by w - batch start */
    uint64_t batch0;
    int rc;
} wt_job;

static void* wt_worker(void* arg) {
    wt_job* j = (wt_job*)arg;
    window_scratch sc;
    memset(&sc, 0, sizeof(sc));
    if (!scratch_alloc(&sc, j->N, j->W)) {
        scratch_free(&sc);
        j->rc = -1;
        return NULL;
    }
    for (uint64_t w = j->w0; w < j->w1 && j->rc == 0; w++) {
        const uint64_t left = j->M - w * j->W;
        const uint32_t nvar = (uint32_t)(left < j->W ? left : j->W);
        j->rc = simulate_window(j->N, j->seed, w, nvar, &j->outs[w - j->batch0], &sc);
    }
    scratch_free(&sc);
    return NULL;
}

/* The generated graph: num_nodes + 1 row offsets, num_edges child ids, num_mutations mapped
 * nodes.  Free with oracle_window_tree_free. */
typedef struct {
    uint64_t num_nodes, num_edges, num_mutations;
    uint64_t* down_off;
    uint32_t* down_adj;
    uint32_t* mut_node;
} oracle_wt_graph;

void oracle_window_tree_free(oracle_wt_graph* g) {
    if (!g) return;
    free(g->down_off);
    free(g->down_adj);
    free(g->mut_node);
    memset(g, 0, sizeof(*g));
}

/* Returns 0, or -1 out of memory, -2 bad arguments, -3 too many nodes for 31-bit ids. */
int oracle_window_tree(uint64_t N, uint64_t M, uint64_t seed, uint32_t W, int threads, oracle_wt_graph* out) {
    memset(out, 0, sizeof(*out));
    if (N < 2 || N >= 0x40000000ull || W < 1) return -2;
    if (threads < 1) threads = 1;
    const uint64_t nwin = (M + W - 1) / W;
    /* edges are at most nwin * (N + W); nodes at most N + M */
    uint64_t capE = nwin * (N + W), capN = N + M;
    out->down_off = (uint64_t*)malloc(sizeof(uint64_t) * (capN + 1));
    out->down_adj = (uint32_t*)malloc(sizeof(uint32_t) * (capE ? capE : 1));
    out->mut_node = (uint32_t*)malloc(sizeof(uint32_t) * (M ? M : 1));
    if (!out->down_off || !out->down_adj || !out->mut_node) {
        oracle_window_tree_free(out);
        return -1;
    }
    out->num_mutations = M;
    for (uint64_t m = 0; m < M; m++) out->mut_node[m] = WT_INVALID_NODE;
    for (uint64_t v = 0; v <= N; v++) out->down_off[v] = 0;
    uint64_t nodes = N, edges = 0;

    const uint64_t batch = (uint64_t)threads * 2;
    window_out* outs = (window_out*)calloc(batch, sizeof(window_out));
    wt_job* jobs = (wt_job*)calloc((size_t)threads, sizeof(wt_job));
    pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * (size_t)threads);
    int rc = (outs && jobs && th) ? 0 : -1;
    for (uint64_t w0 = 0; rc == 0 && w0 < nwin; w0 += batch) {
        const uint64_t w1 = (w0 + batch < nwin) ? w0 + batch : nwin;
        const uint64_t per = (w1 - w0 + (uint64_t)threads - 1) / (uint64_t)threads;
        int started = 0;
        for (int t = 0; t < threads; t++) {
            const uint64_t a = w0 + (uint64_t)t * per, b = (a + per < w1) ? a + per : w1;
            if (a >= b) break;
            jobs[t] = (wt_job){N, M, seed, a, b, W, outs, w0, 0};
            pthread_create(&th[t], NULL, wt_worker, &jobs[t]);
            started++;
        }
        for (int t = 0; t < started; t++) {
            pthread_join(th[t], NULL);
            if (jobs[t].rc) rc = jobs[t].rc;
        }
        for (uint64_t w = w0; rc == 0 && w < w1; w++) {
            window_out* o = &outs[w - w0];
            const uint64_t base = nodes;
            if (base + o->num_nodes > WT_INVALID_NODE) {
                rc = -3;
                break;
            }
            for (uint32_t i = 0; i < o->num_nodes; i++) {
                for (uint32_t e = o->off[i]; e < o->off[i + 1]; e++) {
                    const uint32_t c = o->adj[e];
                    out->down_adj[edges++] = (c < N) ? c : (uint32_t)(base + (c - N));
                }
                out->down_off[base + i + 1] = edges;
            }
            for (uint32_t j = 0; j < o->nvar; j++) {
                const uint32_t x = o->mut_local[j];
                out->mut_node[w * W + j] = (x < N) ? x : (uint32_t)(base + (x - N));
            }
            nodes += o->num_nodes;
        }
        for (uint64_t w = w0; w < w1; w++) window_free(&outs[w - w0]);
    }
    free(outs);
    free(jobs);
    free(th);
    if (rc != 0) {
        oracle_window_tree_free(out);
        return rc;
    }
    out->num_nodes = nodes;
    out->num_edges = edges;
    return 0;
}
