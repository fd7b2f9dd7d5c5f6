/*
 * grgx -- GB300-native GRG matrix multiplication, C ABI.
 *
 * Drop-in boundary for GRGL's graph matrix multiplication.  Each entry point names the
 * reference interface (aprilweilab/grgl 2.10) it stands in for.  Plain pointers and sizes
 * only; no C++ or framework types cross this boundary, and no exception escapes it: every
 * call returns a grgx_status, with a human-readable message from grgx_last_error() (the
 * reference's own message text where the reference has one).
 *
 * Threading: a graph handle is immutable after creation; any number of threads may call
 * grgx_matmul on one handle at once.  Each call allocates its own scratch from the device's
 * stream-ordered memory pool, on the stream it is given.
 */
#ifndef GRGX_H
#define GRGX_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct grgx_graph grgx_graph;

typedef enum {
    GRGX_OK = 0,
    GRGX_ERR_API_MISUSE = 1, /* reference ApiMisuseFailure (common.h:45-58) -> RuntimeError */
    GRGX_ERR_CUDA = 2,       /* a CUDA runtime call failed */
    GRGX_ERR_OUT_OF_MEMORY = 3,
    GRGX_ERR_BAD_FILE = 4,   /* reference SerializationFailure / BadInputFileFailure */
    GRGX_ERR_UNSUPPORTED = 5,
    GRGX_ERR_NO_DEVICE = 6,
    GRGX_ERR_TIMEOUT = 7
} grgx_status;

/* TraversalDirection values (include/grgl/visitor.h:26). */
typedef enum { GRGX_DIRECTION_DOWN = 1, GRGX_DIRECTION_UP = 2 } grgx_direction;

/* Element types accepted by pygrgl.matmul (_grgl.cpp:205-238). */
typedef enum {
    GRGX_F64 = 0,
    GRGX_F32 = 1,
    GRGX_I64 = 2,
    GRGX_I32 = 3,
    GRGX_I16 = 4,
    GRGX_I8 = 5,
    GRGX_U64 = 6,
    GRGX_U32 = 7,
    GRGX_U16 = 8,
    GRGX_U8 = 9,
    GRGX_BOOL = 10 /* GF(2): one byte per value (0/1) in and out, XOR accumulation */
} grgx_dtype;

/* GRG::NodeInitEnum (include/grgl/grg.h:646-651). */
typedef enum { GRGX_INIT_ZERO = 0, GRGX_INIT_VECTOR = 1, GRGX_INIT_MATRIX = 2, GRGX_INIT_XTX = 3 } grgx_init;

/* grgx_matmul flags. */
#define GRGX_FLAG_DEVICE_POINTERS 0x1u /* input/output/init/miss are device pointers */
#define GRGX_FLAG_F32_PLAIN 0x2u       /* f32: plain (uncompensated) accumulation */
#define GRGX_FLAG_SYNC 0x4u            /* wait for the stream before returning */
#define GRGX_FLAG_OVERWRITE 0x8u       /* write the output instead of adding to it */
#define GRGX_FLAG_F64_NATIVE 0x10u     /* f64: accumulate on the FP64 pipe instead of as scaled float pairs */
#define GRGX_FLAG_NO_GRAPH 0x20u       /* never replay a captured CUDA graph for this call */
#define GRGX_FLAG_ASYNC 0x40u          /* grgx_matmul with host pointers: return once queued (below) */

typedef struct {
    uint64_t num_nodes;
    uint64_t num_edges;
    uint64_t num_samples;
    uint64_t num_mutations;
    uint64_t ploidy;
    uint64_t num_levels;
    uint64_t has_missing; /* graph carries missingness nodes */
    uint64_t has_coals;   /* every non-sample node has a coalescence count (init=xtx works) */
    uint64_t device_bytes; /* resident plan size once uploaded (0 before) */
} grgx_graph_info;

/* Message for the last failing call on this thread ("" if none). */
const char* grgx_last_error(void);

/* Library version string. */
const char* grgx_version(void);

/* Replaces grgl::loadImmutableGRG (src/serialize.cpp:923-937, readImmutableGrg :815-890):
 * reads a .grg file (format 5.x) into a host graph.  Fails with GRGX_ERR_BAD_FILE on a
 * malformed file, with the reference's message text. */
grgx_status grgx_graph_load(const char* path, grgx_graph** out);

/* Builds a graph from the arrays a CSRGRG holds (include/grgl/grg.h:1232-1303): the down-edge
 * CSR (children of node v are down_adj[down_off[v] .. down_off[v+1])), the mutation -> node
 * map (getNodesAndMutations, grg.h:406-415; 0x7fffffff = unmapped), optional missingness
 * nodes (NULL = none) and optional coalescence counts of the non-sample nodes
 * (getNumIndividualCoals, grg.h:743-747; NULL = not set).  Arrays are copied. */
grgx_status grgx_graph_from_csr(uint64_t num_nodes, uint64_t num_samples, uint64_t ploidy,
                                const uint64_t* down_off, const uint32_t* down_adj, uint64_t num_mutations,
                                const uint32_t* mut_node, const uint32_t* miss_node, const uint32_t* coals,
                                grgx_graph** out);

/* Seeded window-tree GRG: one Kingman coalescent tree over all samples per window of
 * `window` consecutive variants, mutations placed on branches in proportion to branch
 * length, each tree collapsed to its mutation nodes (no reference counterpart: the
 * synthetic-workload producer; `threads` <= 0 means all host cores). */
grgx_status grgx_graph_generate(uint64_t num_samples, uint64_t num_mutations, uint64_t seed, uint32_t window,
                                int threads, grgx_graph** out);

/* Replaces grgl::saveGRG(grg, path, allowSimplify=false) (src/serialize.cpp:939-942, writer
 * :517-669) for graphs whose children are ascending within each node: writes format 5.3, which
 * grgx_graph_load reads back.  Mutations are written with REF "A" / ALT "C" and the stored
 * positions (the matmul path reads neither). */
grgx_status grgx_graph_save(const grgx_graph* g, const char* path);

void grgx_graph_destroy(grgx_graph* g);

grgx_status grgx_graph_info_get(const grgx_graph* g, grgx_graph_info* out);

/* Copies of the host arrays (for checkers and exporters): sizes from grgx_graph_info_get;
 * miss_node / coals may be NULL to skip them. */
grgx_status grgx_graph_export(const grgx_graph* g, uint64_t* down_off, uint32_t* down_adj, uint32_t* mut_node,
                              uint32_t* miss_node, uint32_t* coals);

/* Replaces grgl::saveGRGSubset(..., DIRECTION_DOWN, seedList, ...) (include/grgl/serialize.h:147-166)
 * without the file round trip: a new graph holding the listed mutations (renumbered in list
 * order), every sample (same ids), and the nodes reachable downward from the mutations' (and
 * their missingness) nodes, in their original relative order.  Range shards of one graph have
 * disjoint mutations; their UP outputs concatenate and their DOWN outputs sum. */
grgx_status grgx_graph_subset(const grgx_graph* g, const uint32_t* mutation_ids, uint64_t n, grgx_graph** out);

/* Builds the level plan and copies it to the current device (done implicitly by the first
 * grgx_matmul; explicit here so callers can keep it out of timed regions). */
grgx_status grgx_graph_upload(grgx_graph* g);

/* Replaces GRG::matrixMultiplication<IOType, NodeValueType, useBitVector>
 * (include/grgl/grg.h:1341-1517, argument for argument) and, through it, GRG::matMul
 * (grg.h:705-716) and the pygrgl.matmul / dot_product bindings (_grgl.cpp:80-241):
 *   input       K x input_cols row-major (K = input_rows)
 *   output      output_size = K x output_cols row-major; ADDED to, like the reference
 *               (callers zero it for a plain product)
 *   init        init_kind VECTOR: K values; MATRIX: K x num_nodes; else ignored
 *   miss        K x num_mutations; an input in DOWN, an in/out accumulator in UP; NULL = none
 *   stream      cudaStream_t (NULL = legacy default stream)
 * With GRGX_FLAG_DEVICE_POINTERS the buffers are device pointers and the call is
 * asynchronous on `stream`; otherwise they are host pointers and the call returns when the
 * output (and miss) have been written back -- unless GRGX_FLAG_ASYNC is set: then the copies
 * in and out are queued on `stream` with the product and the call returns at once; the caller
 * keeps every host buffer alive and synchronizes `stream` before reading the output.  With
 * page-locked host buffers (grgx_host_alloc) the copies of one call then overlap the products
 * of calls queued on other streams.  Validation and messages follow validateMatMulInputs
 * (internal_mult.h:130-158).
 * On small graphs (at most 2^25 edges) the first call of each shape (dtype, K, direction,
 * options, stream) captures the whole call into a CUDA graph, which later calls of that shape
 * replay through staging buffers -- one launch instead of one per level.  The first call of a
 * shape therefore must not happen inside the caller's own stream capture;
 * GRGX_FLAG_NO_GRAPH turns this off. */
grgx_status grgx_matmul(grgx_graph* g, grgx_dtype dtype, const void* input, uint64_t input_cols,
                        uint64_t input_rows, grgx_direction direction, void* output, uint64_t output_size,
                        int emit_all_nodes, int by_individual, const void* init, grgx_init init_kind, void* miss,
                        uint32_t flags, void* stream);

/* No counterpart in the reference (the operator grapp's standardized LinearOperators apply on top
 * of GRGL's matmul; grapp is not part of GRGL).  Products with the standardized genotype matrix
 * Z (N x M), Z[i, j] = (X[i, j] - mu_j) / sigma_j, mu_j = p_j = count_j / N, sigma_j =
 * sqrt(p_j (1 - p_j)) (haploid), columns with sigma_j = 0 set to zero:
 *   UP:   out = V Z   = ((V X) - (V 1) mu^T) / sigma        (V: K x N, out: K x M)
 *   DOWN: out = V Z^T = X (V / sigma)^T - 1 (mu^T (V / sigma)^T)   (V: K x M, out: K x N)
 * The products with X run on the sweep in the input's dtype (float32 compensated or float64);
 * the allele frequencies are an exact int32 UP product computed once per graph, and the row
 * sums V 1 and mu^T (V / sigma) are float64 reductions on the device.  float32/float64 only;
 * `flags` as grgx_matmul (host or device pointers); the output is overwritten. */
grgx_status grgx_matmul_standardized(grgx_graph* g, grgx_dtype dtype, const void* input, uint64_t input_cols,
                                     uint64_t input_rows, grgx_direction direction, void* output,
                                     uint64_t output_size, uint32_t flags, void* stream);

/* No counterpart in the reference (grapp's XX^T-style LinearOperators chain two matmul calls
 * through host memory).  Two traversals chained on the device, the intermediate resident:
 *   first = UP:   out = V X X^T  (V, out: K x N)     first = DOWN: out = V X^T X  (V, out: K x M)
 * With `standardized` nonzero, Z (as grgx_matmul_standardized) replaces X (float32/float64).
 * Flags as grgx_matmul_standardized; the output is overwritten. */
grgx_status grgx_matmul_gram(grgx_graph* g, grgx_dtype dtype, const void* input, uint64_t input_cols,
                             uint64_t input_rows, grgx_direction first, void* output, uint64_t output_size,
                             int standardized, uint32_t flags, void* stream);

/* One request of a batch or of the server: the product (no init, miss or emit_all_nodes) of
 * `rows` x cols `input` in `direction`, written to `output` (rows x out_cols, overwritten).  Host or device memory as the call's flags say.  With
 * GRGX_REQUEST_STANDARDIZED in `options` the product is the one grgx_matmul_standardized
 * computes (float32/float64 only); it still shares the traversal with the plain requests
 * stacked beside it. */
#define GRGX_REQUEST_STANDARDIZED 0x1u
/* by_individual (grg.h:1341-1517): UP input / DOWN output columns are individuals, the samples'
 * values folded by ploidy; requests with and without it run in separate traversals. */
#define GRGX_REQUEST_BY_INDIVIDUAL 0x2u
typedef struct {
    grgx_dtype dtype;
    grgx_direction direction;
    uint64_t rows;
    const void* input;
    void* output;
    uint32_t options;
} grgx_request;

/* No counterpart in the reference (its callers loop over matMul calls).  Runs `n` requests on
 * one graph with as few traversals as possible: requests of the same direction and dtype are
 * stacked row-wise into traversals of at most `max_cols` columns (0 = 512 four-byte or 256
 * eight-byte columns), so the edge stream and the launches are shared; a request's rows may be
 * cut across two traversals, and rows that would leave a group's last traversal with a nearly
 * empty 128-column (64 for eight-byte values) tile run as a narrow traversal of their own.  The
 * stacks run on up to three internal streams that join `stream` before the call's work is
 * complete on it.  Each request's
 * result equals its own grgx_matmul result (bit-exact for integers; float sums may round
 * differently because the stacked row is wider).  Flags as grgx_matmul
 * (GRGX_FLAG_DEVICE_POINTERS, GRGX_FLAG_F32_PLAIN, GRGX_FLAG_F64_NATIVE). */
grgx_status grgx_matmul_batch(grgx_graph* g, const grgx_request* requests, uint64_t n, uint64_t max_cols,
                              uint32_t flags, void* stream);

/* ---- serving: resident graphs, continuous batching ------------------------------------------
 * No counterpart in the reference.  A server owns `workers` threads, each with its own CUDA
 * stream on the device current at creation.  Submitted requests queue; whenever a worker is
 * free it takes the oldest request plus every queued request for the same graph, direction and
 * dtype that fits `max_cols` stacked rows, admits the batch only if its estimated device
 * memory fits beside the batches in flight (`memory_budget`, 0 = 90% of the free memory at
 * creation), runs it as one traversal and hands each request its own rows.  Requests that
 * arrive while batches run are picked up as workers free up, so work from several batches
 * overlaps on the device.  Request buffers are host memory and must stay valid until
 * grgx_server_wait returns for their ticket. */
typedef struct grgx_server grgx_server;

typedef struct {
    double submit_s; /* seconds since server creation */
    double start_s;  /* batch launch */
    double done_s;   /* result written */
    uint64_t batch_requests;
    uint64_t batch_rows;
} grgx_request_stats;

grgx_status grgx_server_create(uint32_t workers, uint64_t memory_budget, uint64_t max_cols, grgx_server** out);
/* The graph must outlive the server; it is uploaded to the server's device here. */
grgx_status grgx_server_add_graph(grgx_server* s, grgx_graph* g, uint32_t* graph_id);
grgx_status grgx_server_submit(grgx_server* s, uint32_t graph_id, const grgx_request* request, uint64_t* ticket);
/* Blocks until the request is done (or `timeout_s` passes: GRGX_ERR_TIMEOUT); returns the
 * request's own status and fills `stats` (may be NULL).  A ticket can be waited for once. */
grgx_status grgx_server_wait(grgx_server* s, uint64_t ticket, double timeout_s, grgx_request_stats* stats);
/* Stops the workers after the batches in flight; queued requests fail with GRGX_ERR_TIMEOUT. */
void grgx_server_destroy(grgx_server* s);

/* Size of the static device scratch behind grgx_matmul_noalloc (64 MiB).  A device holds it
 * from the first graph upload on that device (CUDA loads device code lazily, per device; with
 * CUDA_MODULE_LOADING=EAGER from context creation) until the process exits. */
#define GRGX_NOALLOC_SCRATCH_BYTES (64ull << 20)

/* No counterpart in the reference.  The plain product (no init, miss, emit_all_nodes or
 * by_individual) for callers that cannot allocate device memory once they are running -- for
 * example a host program that hands out a fixed device budget at start-up and forbids
 * allocation afterwards.  It allocates nothing: its scratch is one static __device__ array of
 * GRGX_NOALLOC_SCRATCH_BYTES, and products that need more are rejected with
 * GRGX_ERR_UNSUPPORTED before any launch.  input/output are device pointers; the output is
 * overwritten; the call is asynchronous on `stream`.  The graph must already be resident
 * (grgx_graph_upload); the upload also reserves the static array on the device and looks up
 * its address, so upload graphs before claiming the rest of a device budget.  (A call on a
 * device where no upload happened looks the address up itself; make such a first call before
 * any stream capture.)  All calls share the array: calls that overlap on the GPU race, so
 * serialise them on one stream.  A device reset between calls is not supported.  float64
 * accumulates on the FP64 pipe (grgx_matmul's float64 default is the scaled float-pair path,
 * GRGX_FLAG_F64_NATIVE selects the same FP64 accumulation there).  bool is not supported. */
grgx_status grgx_matmul_noalloc(grgx_graph* g, grgx_dtype dtype, const void* input, uint64_t input_cols,
                                uint64_t input_rows, grgx_direction direction, void* output, uint64_t output_size,
                                void* stream);

/* No counterpart in the reference.  Device memory of the library's own stream-ordered pool on
 * `device` (the per-call scratch of grgx_matmul and the batch, server and operator entries):
 * `used` = bytes handed out to calls in flight, `reserved` = bytes the pool holds from the
 * device (kept cached between calls).  Either pointer may be NULL.  The process's default pool
 * is not used or changed by the library. */
grgx_status grgx_pool_usage(int device, uint64_t* used, uint64_t* reserved);

/* Diagnostic, no counterpart in the reference: measured L2 -> SM read bandwidth (GB/s) of the
 * current device over an L2-resident buffer of `bytes` (>= 1 MiB) read `reps` times -- the
 * ceiling of the sweep's row gathers when the gathered rows stay in L2. */
grgx_status grgx_measure_l2_bandwidth(uint64_t bytes, int reps, double* gbps);

/* No counterpart in the reference.  Page-locked host memory for results the caller will have
 * copied back (grgx_matmul / batch / server outputs in host memory): device-to-host copies
 * into it run at the link's full speed, while a freshly allocated pageable buffer pays a page
 * fault per page during the copy.  Freed blocks are cached by power-of-two size for later calls
 * (16 GiB in all, or the GRGX_HOST_POOL_BYTES environment variable).  grgx_host_free ignores
 * pointers it did not hand out. */
grgx_status grgx_host_alloc(uint64_t bytes, void** out);
void grgx_host_free(void* p);

/* ---- launch-shape autotuner -------------------------------------------------------------
 * No counterpart in the reference.  Each level of the sweep can run with G lanes per row (the
 * default for its K, half or a quarter of it: more rows per warp, more column tiles) and with
 * the default or a deep prefetch variant (twice the gathers in flight per lane).  The
 * process-wide table is keyed on (storage kind, row stride, log2 of the level's rows, log2 of
 * its mean degree); levels without an entry run the default shape.
 *
 * grgx_autotune times candidates on each level of one traversal of `g` (resident on the
 * current device; it is uploaded first) for `rows` x cols inputs of `dtype` in `direction`
 * (`flags`: GRGX_FLAG_F32_PLAIN / GRGX_FLAG_F64_NATIVE select the accumulator as in
 * grgx_matmul): the deep variant, then fewer lanes per row while that keeps winning; levels
 * with under 0.5% of the edges keep the default.  It records each level's winner when it beats
 * the default by more than 2%.  For UP on graphs with enough samples it tunes both the plain
 * level sweep and the split form (edges to samples first, in sample blocks) and records for
 * `g` and this row width which form is faster.  It
 * writes a per-level report to `report` (NUL-terminated, truncated to `report_len`;
 * `report_needed`, if not NULL, gets the full size).  It drops `g`'s captured CUDA graphs; make
 * no other call on `g` while it runs.  Float results may round differently under another shape
 * (the order of a row's terms changes); integer results do not change. */
grgx_status grgx_autotune(grgx_graph* g, grgx_dtype dtype, uint64_t rows, grgx_direction direction, uint32_t flags,
                          char* report, uint64_t report_len, uint64_t* report_needed);
/* The table as text, one entry per line ("kind stride rows_log2 degree_log2 g tiles variant"),
 * for saving; import merges such text back (entries invalid for a shape are ignored at use). */
grgx_status grgx_autotune_export(char* buf, uint64_t len, uint64_t* needed);
grgx_status grgx_autotune_import(const char* text);
void grgx_autotune_clear(void);

/* Device-time breakdown of the last grgx_matmul made by this thread with timing enabled. */
typedef struct {
    float total_ms;     /* seed + sweep + gather, CUDA events */
    float sweep_ms;     /* level sweep only */
    uint64_t launches;  /* kernels launched by the call */
    uint64_t alg_bytes; /* algorithmic bytes of the sweep (edge ids + offsets + one row per edge + one row per node) */
} grgx_timing;

/* Per-call CUDA-event timing on this thread: 1 = read back at the end of each call (adds a
 * stream sync per call; grgx_last_timing), 2 = deferred (no sync; grgx_collect_timings returns
 * every call's timing, in call order, after waiting for them), 0 = off. */
void grgx_set_timing(int enabled);
grgx_status grgx_last_timing(grgx_timing* out);
/* Deferred timings (grgx_set_timing(2)) of this thread's calls since the last collection; fails
 * without clearing when there are more than `capacity`. */
grgx_status grgx_collect_timings(grgx_timing* out, uint64_t capacity, uint64_t* count);

#ifdef __cplusplus
}
#endif

#endif /* GRGX_H */
