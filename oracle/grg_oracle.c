/*
 * CPU oracle for GRG matrix multiplication -- TEST INFRASTRUCTURE ONLY.
 *
 * This file is the checker, never the product: only the tests, the smoke check and the
 * CPU-baseline leg of the benchmark may load it.  It is a plain-C restatement of the
 * reference CPU algorithm, GRG::matrixMultiplication (include/grgl/grg.h:1341-1517), with
 * the same loop orders so that integer results are bit-identical and floating point sums
 * are taken in the same order:
 *
 *   init fill          grg.h:1370-1402  (ZERO / VECTOR / MATRIX / XTX = 2*coals)
 *   DOWN seed          grg.h:1405-1427  (triples sorted by node, then mutation id)
 *   DOWN sweep         grg.h:1428-1431, matmulSumChildrenDown grg.h:1312-1322
 *   DOWN gather        grg.h:1440-1453  (by_individual folds ploidy samples)
 *   UP seed            grg.h:1458-1469
 *   UP sweep           grg.h:1470-1474, matmulSumChildrenUp grg.h:1324-1334
 *   UP gather          grg.h:1483-1505  (miss is an in/out accumulator)
 *   emit_all_nodes     grg.h:1507-1516
 *   element add        internal_mult.h:42-49 (plain +=, integers wrap)
 *   bool (GF(2))       internal_mult.h:111-128, 207-241 (XOR)
 *
 * For graphs whose node ids are not topologically ordered the reference falls back to a
 * topological order or a DFS visitor (grg.h:1432-1438, 1475-1481); here a Kahn order is
 * used, which gives the same integer results.
 *
 * A second entry point, oracle_matmul_sharded, restates the reference's own multi-core
 * pattern (test/endtoend/test_matmul.py:264-325): the mutations are split into ranges,
 * each range's sub-graph (the nodes below its mutations) is multiplied on its own thread,
 * DOWN partial outputs are summed and UP outputs are disjoint.
 */
#define _POSIX_C_SOURCE 199309L
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#define ORACLE_INVALID_NODE 0x7fffffffu
#define ORACLE_COAL_NOT_SET 0xffffffffu

enum { OR_DOWN = 1, OR_UP = 2 };
enum { OR_INIT_ZERO = 0, OR_INIT_VECTOR = 1, OR_INIT_MATRIX = 2, OR_INIT_XTX = 3 };
enum {
    OR_F64 = 0, OR_F32 = 1, OR_I64 = 2, OR_I32 = 3, OR_I16 = 4, OR_I8 = 5,
    OR_U64 = 6, OR_U32 = 7, OR_U16 = 8, OR_U8 = 9, OR_BOOL = 10
};

typedef struct {
    uint64_t num_nodes;
    uint64_t num_samples;
    uint64_t ploidy;
    uint64_t num_mutations;
    const uint64_t* down_off; /* num_nodes + 1 */
    const uint32_t* down_adj; /* children, ascending per node */
    const uint32_t* mut_node; /* num_mutations; ORACLE_INVALID_NODE when unmapped */
    const uint32_t* miss_node; /* num_mutations or NULL */
    const uint32_t* coals;     /* num_nodes - num_samples or NULL */
} oracle_graph;

typedef struct {
    uint32_t node;
    uint32_t mut;
    uint32_t miss;
} triple_t;

static int triple_cmp(const void* a, const void* b) {
    const triple_t* x = (const triple_t*)a;
    const triple_t* y = (const triple_t*)b;
    if (x->node != y->node) return x->node < y->node ? -1 : 1;
    if (x->mut != y->mut) return x->mut < y->mut ? -1 : 1;
    if (x->miss != y->miss) return x->miss < y->miss ? -1 : 1;
    return 0;
}

/* Mutation triples in the order GRG::getNodesAndMutations yields them (grg.cpp:265-300). */
static triple_t* sorted_triples(const oracle_graph* g) {
    triple_t* t = (triple_t*)malloc(sizeof(triple_t) * (g->num_mutations ? g->num_mutations : 1));
    for (uint64_t m = 0; m < g->num_mutations; m++) {
        t[m].node = g->mut_node[m];
        t[m].mut = (uint32_t)m;
        t[m].miss = g->miss_node ? g->miss_node[m] : ORACLE_INVALID_NODE;
    }
    qsort(t, g->num_mutations, sizeof(triple_t), triple_cmp);
    return t;
}

static int nodes_are_ordered(const oracle_graph* g) {
    for (uint64_t v = 0; v < g->num_nodes; v++)
        for (uint64_t e = g->down_off[v]; e < g->down_off[v + 1]; e++)
            if (g->down_adj[e] >= v) return 0;
    return 1;
}

/* Kahn order with children before parents. */
static uint32_t* children_first_order(const oracle_graph* g) {
    uint64_t n = g->num_nodes;
    uint32_t* pending = (uint32_t*)calloc(n ? n : 1, sizeof(uint32_t));
    uint32_t* order = (uint32_t*)malloc(sizeof(uint32_t) * (n ? n : 1));
    uint64_t* up_off = (uint64_t*)calloc(n + 1, sizeof(uint64_t));
    uint64_t ne = g->down_off[n];
    uint32_t* up_adj = (uint32_t*)malloc(sizeof(uint32_t) * (ne ? ne : 1));
    for (uint64_t e = 0; e < ne; e++) up_off[g->down_adj[e] + 1]++;
    for (uint64_t v = 0; v < n; v++) up_off[v + 1] += up_off[v];
    uint64_t* fill = (uint64_t*)malloc(sizeof(uint64_t) * (n ? n : 1));
    for (uint64_t v = 0; v < n; v++) fill[v] = up_off[v];
    for (uint64_t v = 0; v < n; v++) {
        pending[v] = (uint32_t)(g->down_off[v + 1] - g->down_off[v]);
        for (uint64_t e = g->down_off[v]; e < g->down_off[v + 1]; e++) up_adj[fill[g->down_adj[e]]++] = (uint32_t)v;
    }
    uint64_t head = 0, tail = 0;
    for (uint64_t v = 0; v < n; v++)
        if (pending[v] == 0) order[tail++] = (uint32_t)v;
    while (head < tail) {
        uint32_t v = order[head++];
        for (uint64_t e = up_off[v]; e < up_off[v + 1]; e++)
            if (--pending[up_adj[e]] == 0) order[tail++] = up_adj[e];
    }
    free(pending);
    free(up_off);
    free(up_adj);
    free(fill);
    return order;
}

/* Node subset restriction used by the sharded form: active[v] != 0 marks the nodes of a
 * shard.  NULL means every node. */
#define ORACLE_BODY(T)                                                                                         \
    static int matmul_##T(const oracle_graph* g, const T* in, uint64_t in_cols, uint64_t rows, int direction,  \
                          T* out, uint64_t out_cols, int emit_all, int by_indiv, const T* init, int init_kind, \
                          T* miss, const uint8_t* active, const triple_t* trip, uint64_t ntrip,                \
                          const uint32_t* order) {                                                             \
        const uint64_t n = g->num_nodes, K = rows;                                                             \
        T* val = (T*)calloc((n * K) != 0 ? n * K : 1, sizeof(T));                                                   \
        if (!val) return -1;                                                                                   \
        switch (init_kind) {                                                                                   \
        case OR_INIT_XTX:                                                                                      \
            for (uint64_t i = 0; i < n; i++) {                                                                 \
                uint32_t c = (i < g->num_samples) ? 0u : (g->coals ? g->coals[i - g->num_samples]             \
                                                                    : ORACLE_COAL_NOT_SET);                   \
                if (c == ORACLE_COAL_NOT_SET) { free(val); return -2; }                                        \
                for (uint64_t k = 0; k < K; k++) val[i * K + k] += (T)(c * 2);                                  \
            }                                                                                                  \
            break;                                                                                             \
        case OR_INIT_VECTOR:                                                                                   \
            for (uint64_t i = 0; i < n; i++)                                                                   \
                for (uint64_t k = 0; k < K; k++) val[i * K + k] += init[k];                                    \
            break;                                                                                             \
        case OR_INIT_MATRIX:                                                                                   \
            for (uint64_t i = 0; i < n; i++)                                                                   \
                for (uint64_t k = 0; k < K; k++) val[i * K + k] += init[k * n + i];                            \
            break;                                                                                             \
        default: break;                                                                                        \
        }                                                                                                      \
        if (direction == OR_DOWN) {                                                                            \
            for (uint64_t t = 0; t < ntrip; t++) {                                                             \
                const uint32_t node = trip[t].node, mut = trip[t].mut, mn = trip[t].miss;                      \
                if (node != ORACLE_INVALID_NODE && (!active || active[node]))                                  \
                    for (uint64_t k = 0; k < K; k++) val[node * K + k] += in[k * in_cols + mut];               \
                if (miss && mn != ORACLE_INVALID_NODE && (!active || active[mn]))                              \
                    for (uint64_t k = 0; k < K; k++) val[mn * K + k] += miss[k * in_cols + mut];               \
            }                                                                                                  \
            for (uint64_t i = n; i > 0; i--) {                                                                 \
                const uint64_t v = order ? order[i - 1] : i - 1;                                               \
                if (active && !active[v]) continue;                                                            \
                for (uint64_t e = g->down_off[v]; e < g->down_off[v + 1]; e++) {                               \
                    const uint64_t c = g->down_adj[e];                                                         \
                    for (uint64_t k = 0; k < K; k++) val[c * K + k] += val[v * K + k];                          \
                }                                                                                              \
            }                                                                                                  \
            if (!emit_all) {                                                                                   \
                for (uint64_t k = 0; k < K; k++)                                                               \
                    for (uint64_t s = 0; s < g->num_samples; s++) {                                            \
                        const uint64_t col = by_indiv ? s / g->ploidy : s;                                     \
                        out[k * out_cols + col] += val[s * K + k];                                             \
                    }                                                                                          \
            }                                                                                                  \
        } else {                                                                                               \
            for (uint64_t s = 0; s < g->num_samples; s++) {                                                    \
                const uint64_t col = by_indiv ? s / g->ploidy : s;                                             \
                for (uint64_t k = 0; k < K; k++) val[s * K + k] += in[k * in_cols + col];                      \
            }                                                                                                  \
            for (uint64_t i = 0; i < n; i++) {                                                                 \
                const uint64_t v = order ? order[i] : i;                                                       \
                if (!order && v < g->num_samples) continue;                                                    \
                if (active && !active[v]) continue;                                                            \
                for (uint64_t e = g->down_off[v]; e < g->down_off[v + 1]; e++) {                               \
                    const uint64_t c = g->down_adj[e];                                                         \
                    for (uint64_t k = 0; k < K; k++) val[v * K + k] += val[c * K + k];                          \
                }                                                                                              \
            }                                                                                                  \
            if (!emit_all) {                                                                                   \
                for (uint64_t k = 0; k < K; k++)                                                               \
                    for (uint64_t t = 0; t < ntrip; t++) {                                                     \
                        const uint32_t node = trip[t].node, mut = trip[t].mut, mn = trip[t].miss;              \
                        if (node != ORACLE_INVALID_NODE && (!active || active[node]))                          \
                            out[k * out_cols + mut] += val[(uint64_t)node * K + k];                            \
                        if (miss && mn != ORACLE_INVALID_NODE && (!active || active[mn]))                      \
                            miss[k * out_cols + mut] += val[(uint64_t)mn * K + k];                             \
                    }                                                                                          \
            }                                                                                                  \
        }                                                                                                      \
        if (emit_all)                                                                                          \
            for (uint64_t k = 0; k < K; k++)                                                                   \
                for (uint64_t v = 0; v < n; v++) out[k * out_cols + v] += val[v * K + k];                      \
        free(val);                                                                                             \
        return 0;                                                                                              \
    }

typedef double f64;
typedef float f32;
ORACLE_BODY(f64)
ORACLE_BODY(f32)
ORACLE_BODY(int64_t)
ORACLE_BODY(int32_t)
ORACLE_BODY(int16_t)
ORACLE_BODY(int8_t)
ORACLE_BODY(uint64_t)
ORACLE_BODY(uint32_t)
ORACLE_BODY(uint16_t)
ORACLE_BODY(uint8_t)

/* GF(2): the reference packs K bits per node and XORs them (internal_mult.h:111-128); a byte
 * per bit with XOR gives the same values. Input/output are bool arrays (one byte, 0 or 1). */
static int matmul_bool(const oracle_graph* g, const uint8_t* in, uint64_t in_cols, uint64_t rows, int direction,
                       uint8_t* out, uint64_t out_cols, int emit_all, int by_indiv, uint8_t* miss,
                       const uint8_t* active, const triple_t* trip, uint64_t ntrip, const uint32_t* order) {
    const uint64_t n = g->num_nodes, K = rows;
    uint8_t* val = (uint8_t*)calloc((n * K) != 0 ? n * K : 1, 1);
    if (!val) return -1;
    if (direction == OR_DOWN) {
        for (uint64_t t = 0; t < ntrip; t++) {
            const uint32_t node = trip[t].node, mut = trip[t].mut, mn = trip[t].miss;
            if (node != ORACLE_INVALID_NODE && (!active || active[node]))
                for (uint64_t k = 0; k < K; k++) val[node * K + k] ^= (in[k * in_cols + mut] != 0);
            if (miss && mn != ORACLE_INVALID_NODE && (!active || active[mn]))
                for (uint64_t k = 0; k < K; k++) val[mn * K + k] ^= (miss[k * in_cols + mut] != 0);
        }
        for (uint64_t i = n; i > 0; i--) {
            const uint64_t v = order ? order[i - 1] : i - 1;
            if (active && !active[v]) continue;
            for (uint64_t e = g->down_off[v]; e < g->down_off[v + 1]; e++)
                for (uint64_t k = 0; k < K; k++) val[g->down_adj[e] * (uint64_t)K + k] ^= val[v * K + k];
        }
        if (!emit_all)
            for (uint64_t k = 0; k < K; k++)
                for (uint64_t s = 0; s < g->num_samples; s++) {
                    const uint64_t col = by_indiv ? s / g->ploidy : s;
                    out[k * out_cols + col] = (out[k * out_cols + col] != 0) != (val[s * K + k] != 0);
                }
    } else {
        for (uint64_t s = 0; s < g->num_samples; s++) {
            const uint64_t col = by_indiv ? s / g->ploidy : s;
            for (uint64_t k = 0; k < K; k++) val[s * K + k] ^= (in[k * in_cols + col] != 0);
        }
        for (uint64_t i = 0; i < n; i++) {
            const uint64_t v = order ? order[i] : i;
            if (!order && v < g->num_samples) continue;
            if (active && !active[v]) continue;
            for (uint64_t e = g->down_off[v]; e < g->down_off[v + 1]; e++)
                for (uint64_t k = 0; k < K; k++) val[v * K + k] ^= val[g->down_adj[e] * (uint64_t)K + k];
        }
        if (!emit_all)
            for (uint64_t k = 0; k < K; k++)
                for (uint64_t t = 0; t < ntrip; t++) {
                    const uint32_t node = trip[t].node, mut = trip[t].mut, mn = trip[t].miss;
                    if (node != ORACLE_INVALID_NODE && (!active || active[node]))
                        out[k * out_cols + mut] = (out[k * out_cols + mut] != 0) != (val[(uint64_t)node * K + k] != 0);
                    if (miss && mn != ORACLE_INVALID_NODE && (!active || active[mn]))
                        miss[k * out_cols + mut] = (miss[k * out_cols + mut] != 0) != (val[(uint64_t)mn * K + k] != 0);
                }
    }
    if (emit_all)
        for (uint64_t k = 0; k < K; k++)
            for (uint64_t v = 0; v < n; v++) out[k * out_cols + v] = (out[k * out_cols + v] != 0) != (val[v * K + k] != 0);
    free(val);
    return 0;
}

static int dispatch(const oracle_graph* g, int dtype, const void* in, uint64_t in_cols, uint64_t rows, int direction,
                    void* out, uint64_t out_cols, int emit_all, int by_indiv, const void* init, int init_kind,
                    void* miss, const uint8_t* active, const triple_t* trip, uint64_t ntrip, const uint32_t* order) {
#define CASE(code, T)                                                                                   \
    case code:                                                                                          \
        return matmul_##T(g, (const T*)in, in_cols, rows, direction, (T*)out, out_cols, emit_all, by_indiv, \
                          (const T*)init, init_kind, (T*)miss, active, trip, ntrip, order);
    switch (dtype) {
        CASE(OR_F64, f64)
        CASE(OR_F32, f32)
        CASE(OR_I64, int64_t)
        CASE(OR_I32, int32_t)
        CASE(OR_I16, int16_t)
        CASE(OR_I8, int8_t)
        CASE(OR_U64, uint64_t)
        CASE(OR_U32, uint32_t)
        CASE(OR_U16, uint16_t)
        CASE(OR_U8, uint8_t)
    case OR_BOOL:
        if (init_kind != OR_INIT_ZERO) return -3;
        return matmul_bool(g, (const uint8_t*)in, in_cols, rows, direction, (uint8_t*)out, out_cols, emit_all,
                           by_indiv, (uint8_t*)miss, active, trip, ntrip, order);
    default: return -4;
    }
#undef CASE
}

/* Returns 0 on success, -1 out of memory, -2 coal counts missing (init=xtx), -3 init with
 * bool, -4 unknown dtype.  Shapes are the caller's responsibility (the Python wrapper
 * checks them with the reference's messages). `out` must be zero-filled by the caller
 * (the reference zero-fills, _grgl.cpp:111-114). */
int oracle_matmul(const oracle_graph* g, int dtype, const void* in, uint64_t in_cols, uint64_t rows, int direction,
                  void* out, uint64_t out_cols, int emit_all, int by_indiv, const void* init, int init_kind,
                  void* miss) {
    triple_t* trip = sorted_triples(g);
    uint32_t* order = nodes_are_ordered(g) ? NULL : children_first_order(g);
    int rc = dispatch(g, dtype, in, in_cols, rows, direction, out, out_cols, emit_all, by_indiv, init, init_kind,
                      miss, NULL, trip, g->num_mutations, order);
    free(order);
    free(trip);
    return rc;
}

/* ---- sharded multi-core form ------------------------------------------------------------ */

typedef struct {
    const oracle_graph* g;
    int dtype;
    const void* in;
    uint64_t in_cols, rows;
    int direction;
    void* out; /* private DOWN partial or shared UP output */
    uint64_t out_cols;
    const triple_t* trip;
    uint64_t ntrip;
    int rc;
} shard_job;

static void* shard_main(void* arg) {
    shard_job* j = (shard_job*)arg;
    j->rc = dispatch(j->g, j->dtype, j->in, j->in_cols, j->rows, j->direction, j->out, j->out_cols, 0, 0, NULL,
                     OR_INIT_ZERO, NULL, NULL, j->trip, j->ntrip, NULL);
    return NULL;
}

/* One shard: the sub-graph that saveGRGSubset keeps for a mutation range (serialize.h:147-166):
 * every sample, and the nodes reachable downward from the range's mutation nodes, renumbered in
 * ascending order (samples keep ids 0..N-1), so the shard is a graph of its own whose node
 * values take (N + its nodes) x K.  Its triples hold the new node ids and the original mutation
 * ids, so a shard reads and writes the full-width input and output columns. */
typedef struct {
    oracle_graph g;
    uint64_t* off;
    uint32_t* adj;
    triple_t* trip;
    uint64_t ntrip;
    uint64_t nedges;
} oracle_shard;

typedef struct {
    int nshards;
    oracle_shard* sh;
} oracle_shards;

typedef struct {
    const oracle_graph* g;
    oracle_shards* s;
    int first, last;
    uint64_t align;
    int rc;
} shard_build_job;

/* First mutation of shard sh: M*sh/n rounded to a multiple of `align` (1: no rounding). */
static uint64_t shard_start(uint64_t M, int sh, int n, uint64_t align) {
    if (sh >= n) return M;
    const uint64_t m = M * (uint64_t)sh / (uint64_t)n;
    const uint64_t r = (m + align / 2) / align * align;
    return r < M ? r : M;
}

static void* shard_build_main(void* arg) {
    shard_build_job* j = (shard_build_job*)arg;
    const oracle_graph* g = j->g;
    oracle_shards* s = j->s;
    const uint64_t M = g->num_mutations, n = g->num_nodes, N = g->num_samples;
    uint8_t* act = (uint8_t*)malloc(n ? n : 1);
    uint32_t* newid = (uint32_t*)malloc(sizeof(uint32_t) * (n ? n : 1));
    if (!act || !newid) {
        j->rc = -1;
        free(act);
        free(newid);
        return NULL;
    }
    for (int sh = j->first; sh < j->last; sh++) {
        oracle_shard* out = &s->sh[sh];
        const uint64_t m0 = shard_start(M, sh, s->nshards, j->align), m1 = shard_start(M, sh + 1, s->nshards, j->align);
        memset(act, 0, n);
        for (uint64_t m = m0; m < m1; m++)
            if (g->mut_node[m] != ORACLE_INVALID_NODE) act[g->mut_node[m]] = 1;
        uint64_t ne = 0;
        for (uint64_t i = n; i > 0; i--) {
            const uint64_t v = i - 1;
            if (!act[v]) continue;
            ne += g->down_off[v + 1] - g->down_off[v];
            for (uint64_t e = g->down_off[v]; e < g->down_off[v + 1]; e++) act[g->down_adj[e]] = 1;
        }
        uint64_t cnt = 0;
        for (uint64_t v = 0; v < n; v++)
            if (v < N || act[v]) newid[v] = (uint32_t)(cnt++);
        out->off = (uint64_t*)malloc(sizeof(uint64_t) * (cnt + 1));
        out->adj = (uint32_t*)malloc(sizeof(uint32_t) * (ne ? ne : 1));
        out->trip = (triple_t*)malloc(sizeof(triple_t) * ((m1 - m0) ? (m1 - m0) : 1));
        if (!out->off || !out->adj || !out->trip) {
            j->rc = -1;
            break;
        }
        uint64_t r = 0, e2 = 0;
        out->off[0] = 0;
        for (uint64_t v = 0; v < n; v++) {
            if (!(v < N || act[v])) continue;
            if (act[v])
                for (uint64_t e = g->down_off[v]; e < g->down_off[v + 1]; e++) out->adj[e2++] = newid[g->down_adj[e]];
            out->off[++r] = e2;
        }
        uint64_t nt = 0;
        for (uint64_t m = m0; m < m1; m++) {
            const uint32_t node = g->mut_node[m];
            out->trip[nt].node = (node == ORACLE_INVALID_NODE) ? ORACLE_INVALID_NODE : newid[node];
            out->trip[nt].mut = (uint32_t)m;
            out->trip[nt].miss = ORACLE_INVALID_NODE;
            nt++;
        }
        qsort(out->trip, nt, sizeof(triple_t), triple_cmp);
        out->ntrip = nt;
        out->nedges = ne;
        out->g.num_nodes = cnt;
        out->g.num_samples = N;
        out->g.ploidy = g->ploidy;
        out->g.num_mutations = M;
        out->g.down_off = out->off;
        out->g.down_adj = out->adj;
        out->g.mut_node = NULL; /* the triples carry the mapping */
        out->g.miss_node = NULL;
        out->g.coals = NULL;
    }
    free(act);
    free(newid);
    return NULL;
}

void oracle_shards_destroy(oracle_shards* s) {
    if (!s) return;
    for (int i = 0; i < s->nshards; i++) {
        free(s->sh[i].off);
        free(s->sh[i].adj);
        free(s->sh[i].trip);
    }
    free(s->sh);
    free(s);
}

/* Split the mutations into `nshards` contiguous id ranges whose starts are multiples of `align`
 * (so that ranges of whole windows share no node with children), built on `threads` threads.
 * Requires ordered node ids. */
oracle_shards* oracle_shards_create_mt(const oracle_graph* g, int nshards, int threads, uint64_t align) {
    if (!nodes_are_ordered(g) || nshards < 1) return NULL;
    if (align < 1) align = 1;
    if (threads < 1) threads = 1;
    if (threads > nshards) threads = nshards;
    oracle_shards* s = (oracle_shards*)calloc(1, sizeof(oracle_shards));
    s->nshards = nshards;
    s->sh = (oracle_shard*)calloc(nshards, sizeof(oracle_shard));
    pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * threads);
    shard_build_job* jobs = (shard_build_job*)calloc(threads, sizeof(shard_build_job));
    for (int t = 0; t < threads; t++) {
        jobs[t].g = g;
        jobs[t].s = s;
        jobs[t].first = (int)((int64_t)nshards * t / threads);
        jobs[t].last = (int)((int64_t)nshards * (t + 1) / threads);
        jobs[t].align = align;
        pthread_create(&th[t], NULL, shard_build_main, &jobs[t]);
    }
    int rc = 0;
    for (int t = 0; t < threads; t++) {
        pthread_join(th[t], NULL);
        if (jobs[t].rc) rc = jobs[t].rc;
    }
    free(th);
    free(jobs);
    if (rc) {
        oracle_shards_destroy(s);
        return NULL;
    }
    return s;
}

oracle_shards* oracle_shards_create(const oracle_graph* g, int nshards) {
    return oracle_shards_create_mt(g, nshards, 1, 1);
}

uint64_t oracle_shard_edges(const oracle_shards* s, int shard) {
    return (shard >= 0 && shard < s->nshards) ? s->sh[shard].nedges : 0;
}

uint64_t oracle_shard_nodes(const oracle_shards* s, int shard) {
    return (shard >= 0 && shard < s->nshards) ? s->sh[shard].g.num_nodes : 0;
}

static uint64_t dtype_size(int dtype) {
    switch (dtype) {
    case OR_F64: case OR_I64: case OR_U64: return 8;
    case OR_F32: case OR_I32: case OR_U32: return 4;
    case OR_I16: case OR_U16: return 2;
    default: return 1;
    }
}

static double now_seconds(void) {
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

/* Shards [first, first + count), one thread each; DOWN partial outputs are summed into `out` in
 * shard order (the time that summation takes goes to *reduce_seconds when it is not NULL); UP
 * outputs of different shards are disjoint.  Plain numeric dtypes only, no options (the
 * benchmarked configuration). */
int oracle_matmul_shard_range(const oracle_graph* g, const oracle_shards* s, int first, int count, int dtype,
                              const void* in, uint64_t in_cols, uint64_t rows, int direction, void* out,
                              uint64_t out_cols, double* reduce_seconds) {
    if (dtype == OR_BOOL) return -4;
    if (first < 0 || count < 1 || first + count > s->nshards) return -5;
    const int ns = count;
    pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * ns);
    shard_job* jobs = (shard_job*)calloc(ns, sizeof(shard_job));
    const uint64_t esz = dtype_size(dtype), outBytes = rows * out_cols * esz;
    for (int i = 0; i < ns; i++) {
        shard_job* j = &jobs[i];
        j->g = &s->sh[first + i].g;
        j->dtype = dtype;
        j->in = in;
        j->in_cols = in_cols;
        j->rows = rows;
        j->direction = direction;
        j->out = (direction == OR_DOWN) ? calloc(outBytes ? outBytes : 1, 1) : out;
        j->out_cols = out_cols;
        j->trip = s->sh[first + i].trip;
        j->ntrip = s->sh[first + i].ntrip;
        pthread_create(&th[i], NULL, shard_main, j);
    }
    int rc = 0;
    for (int i = 0; i < ns; i++) {
        pthread_join(th[i], NULL);
        if (jobs[i].rc) rc = jobs[i].rc;
    }
    if (direction == OR_DOWN) {
        const double t0 = now_seconds();
        const uint64_t cnt = rows * out_cols;
        for (int i = 0; i < ns; i++) {
#define SUMINTO(T)                                                       \
    {                                                                   \
        T* o = (T*)out;                                                 \
        const T* p = (const T*)jobs[i].out;                             \
        for (uint64_t x = 0; x < cnt; x++) o[x] += p[x];                \
    }
            switch (dtype) {
            case OR_F64: SUMINTO(f64) break;
            case OR_F32: SUMINTO(f32) break;
            case OR_I64: case OR_U64: SUMINTO(uint64_t) break;
            case OR_I32: case OR_U32: SUMINTO(uint32_t) break;
            case OR_I16: case OR_U16: SUMINTO(uint16_t) break;
            default: SUMINTO(uint8_t) break;
            }
#undef SUMINTO
            free(jobs[i].out);
        }
        if (reduce_seconds) *reduce_seconds = now_seconds() - t0;
    } else if (reduce_seconds) {
        *reduce_seconds = 0.0;
    }
    free(th);
    free(jobs);
    return rc;
}

/* Every shard, one thread each (the reference's all-cores pattern). */
int oracle_matmul_sharded(const oracle_graph* g, const oracle_shards* s, int dtype, const void* in,
                          uint64_t in_cols, uint64_t rows, int direction, void* out, uint64_t out_cols) {
    return oracle_matmul_shard_range(g, s, 0, s->nshards, dtype, in, in_cols, rows, direction, out, out_cols, NULL);
}
