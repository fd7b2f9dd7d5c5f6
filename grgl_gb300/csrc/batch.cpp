// grgx_matmul_batch: coalescing requests of different K into shared traversals.
//
// Requests with the same direction and dtype are stacked row-wise (their K x cols inputs one
// under the other) into a single input of K_total rows, multiplied once, and the K_total x
// out_cols product is split back into the requests' outputs.  A traversal's cost is one pass
// over the edge ids plus K_total row gathers per edge, so stacking small-K requests shares the
// edge stream, the level launches and the vector lanes a narrow request would leave idle.
#include <cuda_runtime.h>

#include <algorithm>
#include <map>
#include <string>
#include <tuple>
#include <vector>

#include "grgx_internal.h"

namespace grgx {

void matmul_impl(grgx_graph* g, int dtype, const void* input, uint64_t in_cols, uint64_t rows, int direction,
                 void* output, uint64_t output_size, int emit_all, int by_indiv, const void* init, int init_kind,
                 void* miss, uint32_t flags, void* stream);

void matmul_standardized_impl(grgx_graph* g, int dtype, const void* input, uint64_t in_cols, uint64_t rows,
                              int direction, void* output, uint64_t output_size, uint32_t flags, void* stream);
DevicePlan* standardized_plan(grgx_graph* g, cudaStream_t s);
cudaError_t pool_malloc(void** p, size_t bytes, cudaStream_t s);
void standardized_prepare_down(int dtype, const DevicePlan* dp, void* V, long long K, long long M, double* c,
                               cudaStream_t s);
void standardized_finish_down(int dtype, void* Y, const double* c, long long K, long long N, cudaStream_t s);
void standardized_finish_up(int dtype, const DevicePlan* dp, const void* V, long long K, long long N, void* VX,
                            long long M, double* red, cudaStream_t s);

namespace {

#define BATCH_CUDA(call)                                                                             \
    do {                                                                                            \
        cudaError_t e__ = (call);                                                                   \
        if (e__ != cudaSuccess)                                                                     \
            throw Error(e__ == cudaErrorMemoryAllocation ? GRGX_ERR_OUT_OF_MEMORY : GRGX_ERR_CUDA,  \
                        std::string(#call) + ": " + cudaGetErrorString(e__));                        \
    } while (0)

size_t elem_bytes(int dtype) {
    switch (dtype) {
    case GRGX_F64: case GRGX_I64: case GRGX_U64: return 8;
    case GRGX_F32: case GRGX_I32: case GRGX_U32: return 4;
    case GRGX_I16: case GRGX_U16: return 2;
    default: return 1;
    }
}

// Streams a batch spreads its traversals over (per host thread, created on first use): a
// batch's stacks -- UP and DOWN ones, different dtypes -- run side by side instead of one after
// the other.
constexpr int kBatchStreams = 3;
struct BatchStreams {
    cudaStream_t s[kBatchStreams] = {};
    int device = -1;
    ~BatchStreams() {
        for (cudaStream_t x : s)
            if (x) cudaStreamDestroy(x);
    }
};
thread_local BatchStreams t_streams;

cudaStream_t* batch_streams() {
    int device = 0;
    BATCH_CUDA(cudaGetDevice(&device));
    if (t_streams.device != device) {
        for (cudaStream_t& x : t_streams.s) {
            if (x) cudaStreamDestroy(x);
            x = nullptr;
        }
        for (cudaStream_t& x : t_streams.s) BATCH_CUDA(cudaStreamCreateWithFlags(&x, cudaStreamNonBlocking));
        t_streams.device = device;
    }
    return t_streams.s;
}

}  // namespace

// Default stacking width: 512 four-byte or 256 eight-byte columns.  A traversal's cost per
// column keeps falling up to about that width (GB300, 2e9-edge graph: a 256-request float32 mix
// runs at 3.5e12 edge*K/s stacked 128 wide, 4.2e12 at 512, 4.3e12 at 1024) while its node values
// stay a few GB.
uint64_t default_batch_cols(int dtype) { return elem_bytes(dtype) >= 8 ? 256 : 512; }

void matmul_batch_impl(grgx_graph* g, const grgx_request* reqs, uint64_t n, uint64_t maxCols, uint32_t flags,
                       void* stream) {
    GRGX_CHECK(n == 0 || reqs != nullptr, GRGX_ERR_API_MISUSE, "null argument");
    const HostGraph& hg = *g->host;
    const bool dev = (flags & GRGX_FLAG_DEVICE_POINTERS) != 0;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    // group by (direction, dtype, by_individual), keeping submission order inside a group
    std::map<std::tuple<int, int, int>, std::vector<uint64_t>> groups;
    for (uint64_t i = 0; i < n; i++) {
        const grgx_request& r = reqs[i];
        GRGX_CHECK(r.input && r.output && r.rows > 0, GRGX_ERR_API_MISUSE, "matmul() requires non-zero dimensions.");
        GRGX_CHECK(r.direction == GRGX_DIRECTION_DOWN || r.direction == GRGX_DIRECTION_UP, GRGX_ERR_API_MISUSE,
                   "Invalid traversal direction");
        GRGX_CHECK(r.dtype >= GRGX_F64 && r.dtype <= GRGX_BOOL, GRGX_ERR_API_MISUSE, "Unsupported dtype");
        GRGX_CHECK((r.options & ~(GRGX_REQUEST_STANDARDIZED | GRGX_REQUEST_BY_INDIVIDUAL)) == 0, GRGX_ERR_API_MISUSE,
                   "Unknown request options");
        GRGX_CHECK(!(r.options & GRGX_REQUEST_STANDARDIZED) || r.dtype == GRGX_F32 || r.dtype == GRGX_F64,
                   GRGX_ERR_UNSUPPORTED, "standardized products take float32 or float64 input");
        GRGX_CHECK(!((r.options & GRGX_REQUEST_STANDARDIZED) && (r.options & GRGX_REQUEST_BY_INDIVIDUAL)),
                   GRGX_ERR_UNSUPPORTED, "standardized products are per haplotype (no by_individual)");
        GRGX_CHECK(!(r.options & GRGX_REQUEST_BY_INDIVIDUAL) || hg.num_samples % hg.ploidy == 0, GRGX_ERR_API_MISUSE,
                   "by_individual needs the number of samples to be a multiple of the ploidy");
        groups[{static_cast<int>(r.direction), static_cast<int>(r.dtype),
                (r.options & GRGX_REQUEST_BY_INDIVIDUAL) ? 1 : 0}]
            .push_back(i);
    }
    const uint32_t passFlags = (flags & (GRGX_FLAG_F32_PLAIN | GRGX_FLAG_F64_NATIVE)) | GRGX_FLAG_DEVICE_POINTERS |
                               GRGX_FLAG_OVERWRITE;
    // The stacks: per group, the requests' rows in submission order cut into stacks of `width`
    // rows (a request may span two stacks: its rows are independent products).  A traversal
    // covers a row in column tiles of 32 lanes x 16 bytes (128 four-byte or 64 eight-byte
    // columns), and a tile costs nearly a full pass however few of its columns are used; so when
    // a group's last stack would end in a tile less than a quarter full, those rows run as a
    // stack of their own with a narrow layout instead.
    struct Piece {
        uint64_t req, r0, r1;  // rows r0 .. r1 of request req
    };
    struct Stack {
        int direction, dtype, byIndiv;
        std::vector<Piece> pieces;
        uint64_t rows;
    };
    std::vector<Stack> stacks;
    for (auto& kv : groups) {
        const int direction = std::get<0>(kv.first), dtype = std::get<1>(kv.first), byIndiv = std::get<2>(kv.first);
        const uint64_t width = maxCols ? maxCols : default_batch_cols(dtype);
        const uint64_t tile = (dtype == GRGX_BOOL) ? 0 : (elem_bytes(dtype) >= 8 ? 64 : 128);
        std::vector<Stack> gs;
        Stack cur{direction, dtype, byIndiv, {}, 0};
        for (uint64_t k : kv.second) {
            uint64_t r0 = 0;
            const uint64_t rows = reqs[k].rows;
            while (r0 < rows) {
                const uint64_t take = std::min(rows - r0, width - cur.rows);
                cur.pieces.push_back({k, r0, r0 + take});
                cur.rows += take;
                r0 += take;
                if (cur.rows == width) {
                    gs.push_back(std::move(cur));
                    cur = Stack{direction, dtype, byIndiv, {}, 0};
                }
            }
        }
        if (cur.rows) {
            const uint64_t rem = tile ? cur.rows % tile : 0;
            if (tile && cur.rows > tile && rem > 0 && rem * 4 <= tile) {
                // split the last `rem` rows off into their own stack
                Stack tail{direction, dtype, byIndiv, {}, 0};
                uint64_t need = rem;
                while (need > 0) {
                    Piece& pc = cur.pieces.back();
                    const uint64_t take = std::min(need, pc.r1 - pc.r0);
                    tail.pieces.insert(tail.pieces.begin(), Piece{pc.req, pc.r1 - take, pc.r1});
                    pc.r1 -= take;
                    if (pc.r1 == pc.r0) cur.pieces.pop_back();
                    need -= take;
                }
                cur.rows -= rem;
                tail.rows = rem;
                gs.push_back(std::move(cur));
                gs.push_back(std::move(tail));
            } else {
                gs.push_back(std::move(cur));
            }
        }
        for (auto& st : gs) stacks.push_back(std::move(st));
    }
    // Several stacks: fork them over the batch streams (round robin, after the work already queued
    // on the caller's stream) and join them back onto it at the end.
    const int nstreams = static_cast<int>(std::min<size_t>(kBatchStreams, stacks.size()));
    cudaStream_t* bs = nstreams > 1 ? batch_streams() : nullptr;
    cudaEvent_t fork = nullptr;
    if (nstreams > 1) {
        BATCH_CUDA(cudaEventCreateWithFlags(&fork, cudaEventDisableTiming));
        BATCH_CUDA(cudaEventRecord(fork, s));
        for (int k = 0; k < nstreams; k++) BATCH_CUDA(cudaStreamWaitEvent(bs[k], fork, 0));
        BATCH_CUDA(cudaEventDestroy(fork));
    }
    for (size_t si = 0; si < stacks.size(); si++) {
        const Stack& st = stacks[si];
        cudaStream_t ss = nstreams > 1 ? bs[si % nstreams] : s;
        const int direction = st.direction, dtype = st.dtype, byIndiv = st.byIndiv;
        const uint64_t sampleCols = byIndiv ? hg.num_samples / hg.ploidy : hg.num_samples;
        const uint64_t cols = (direction == GRGX_DIRECTION_UP) ? sampleCols : hg.num_mutations;
        const uint64_t outCols = (direction == GRGX_DIRECTION_UP) ? hg.num_mutations : sampleCols;
        const size_t es = elem_bytes(dtype);
        if (st.pieces.size() == 1) {
            // one piece: the request's own buffers (offset to its rows)
            const Piece& pc = st.pieces[0];
            const grgx_request& r = reqs[pc.req];
            const uint64_t K = pc.r1 - pc.r0;
            const void* inp = static_cast<const char*>(r.input) + pc.r0 * cols * es;
            void* outp = static_cast<char*>(r.output) + pc.r0 * outCols * es;
            // host buffers on a batch stream are queued asynchronously; the join below orders them
            const uint32_t f = (flags & ~GRGX_FLAG_SYNC) | (nstreams > 1 && !dev ? GRGX_FLAG_ASYNC : 0u);
            if (r.options & GRGX_REQUEST_STANDARDIZED)
                matmul_standardized_impl(g, dtype, inp, cols, K, direction, outp, K * outCols, f, ss);
            else
                matmul_impl(g, dtype, inp, cols, K, direction, outp, K * outCols, 0, byIndiv, nullptr,
                            GRGX_INIT_ZERO, nullptr, f | GRGX_FLAG_OVERWRITE, ss);
            continue;
        }
        const uint64_t rowsTotal = st.rows;
        bool anyStd = false;
        for (const Piece& pc : st.pieces) anyStd |= (reqs[pc.req].options & GRGX_REQUEST_STANDARDIZED) != 0;
        DevicePlan* dp = anyStd ? standardized_plan(g, ss) : nullptr;
        double* red = nullptr;
        if (anyStd) BATCH_CUDA(pool_malloc(reinterpret_cast<void**>(&red), rowsTotal * sizeof(double), ss));
        void* in = nullptr;
        void* out = nullptr;
        BATCH_CUDA(pool_malloc(&in, rowsTotal * cols * es, ss));
        BATCH_CUDA(pool_malloc(&out, rowsTotal * outCols * es, ss));
        uint64_t row = 0;
        for (const Piece& pc : st.pieces) {
            const grgx_request& r = reqs[pc.req];
            const uint64_t K = pc.r1 - pc.r0;
            char* rowsIn = static_cast<char*>(in) + row * cols * es;
            BATCH_CUDA(cudaMemcpyAsync(rowsIn, static_cast<const char*>(r.input) + pc.r0 * cols * es, K * cols * es,
                                       dev ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, ss));
            if ((r.options & GRGX_REQUEST_STANDARDIZED) && direction == GRGX_DIRECTION_DOWN)
                standardized_prepare_down(dtype, dp, rowsIn, static_cast<long long>(K), static_cast<long long>(cols),
                                          red + row, ss);
            row += K;
        }
        matmul_impl(g, dtype, in, cols, rowsTotal, direction, out, rowsTotal * outCols, 0, byIndiv, nullptr,
                    GRGX_INIT_ZERO, nullptr, passFlags, ss);
        row = 0;
        for (const Piece& pc : st.pieces) {
            const grgx_request& r = reqs[pc.req];
            const uint64_t K = pc.r1 - pc.r0;
            char* rowsOut = static_cast<char*>(out) + row * outCols * es;
            if (r.options & GRGX_REQUEST_STANDARDIZED) {
                if (direction == GRGX_DIRECTION_DOWN)
                    standardized_finish_down(dtype, rowsOut, red + row, static_cast<long long>(K),
                                             static_cast<long long>(outCols), ss);
                else
                    standardized_finish_up(dtype, dp, static_cast<char*>(in) + row * cols * es,
                                           static_cast<long long>(K), static_cast<long long>(cols), rowsOut,
                                           static_cast<long long>(outCols), red + row, ss);
            }
            BATCH_CUDA(cudaMemcpyAsync(static_cast<char*>(r.output) + pc.r0 * outCols * es, rowsOut, K * outCols * es,
                                       dev ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, ss));
            row += K;
        }
        BATCH_CUDA(cudaFreeAsync(in, ss));
        BATCH_CUDA(cudaFreeAsync(out, ss));
        if (red) BATCH_CUDA(cudaFreeAsync(red, ss));
    }
    if (nstreams > 1) {
        for (int k = 0; k < nstreams; k++) {
            cudaEvent_t join = nullptr;
            BATCH_CUDA(cudaEventCreateWithFlags(&join, cudaEventDisableTiming));
            BATCH_CUDA(cudaEventRecord(join, bs[k]));
            BATCH_CUDA(cudaStreamWaitEvent(s, join, 0));
            BATCH_CUDA(cudaEventDestroy(join));
        }
    }
    if (!dev || (flags & GRGX_FLAG_SYNC)) BATCH_CUDA(cudaStreamSynchronize(s));
}

}  // namespace grgx
