// Gram-operator products: two traversals chained on the device, the intermediate resident in HBM.
//
//   first UP:   out = V X X^T   (V: K x N -> K x M -> K x N), the samples' genetic relatedness
//   first DOWN: out = V X^T X   (V: K x M -> K x N -> K x M), the mutations' cross products
// and the same with the standardized matrix Z in place of X.  The K x (M or N) intermediate never
// leaves the device; with Z the float64 reductions of both standardized products run on the
// device as well.
#include <cuda_runtime.h>

#include "device_plan.h"

namespace grgx {

void matmul_impl(grgx_graph* g, int dtype, const void* input, uint64_t in_cols, uint64_t rows, int direction,
                 void* output, uint64_t output_size, int emit_all, int by_indiv, const void* init, int init_kind,
                 void* miss, uint32_t flags, void* stream);
void matmul_standardized_impl(grgx_graph* g, int dtype, const void* input, uint64_t in_cols, uint64_t rows,
                              int direction, void* output, uint64_t output_size, uint32_t flags, void* stream);

namespace {
size_t elem(int dtype) {
    switch (dtype) {
    case GRGX_F64: case GRGX_I64: case GRGX_U64: return 8;
    case GRGX_F32: case GRGX_I32: case GRGX_U32: return 4;
    case GRGX_I16: case GRGX_U16: return 2;
    default: return 1;
    }
}
}  // namespace

void matmul_gram_impl(grgx_graph* g, int dtype, const void* input, uint64_t in_cols, uint64_t rows, int first,
                      void* output, uint64_t output_size, int standardized, uint32_t flags, void* stream) {
    const HostGraph& h = *g->host;
    GRGX_CHECK(first == GRGX_DIRECTION_DOWN || first == GRGX_DIRECTION_UP, GRGX_ERR_API_MISUSE,
               "Invalid traversal direction");
    GRGX_CHECK(in_cols > 0 && rows > 0, GRGX_ERR_API_MISUSE, "matmul() requires non-zero dimensions.");
    GRGX_CHECK(!standardized || dtype == GRGX_F32 || dtype == GRGX_F64, GRGX_ERR_UNSUPPORTED,
               "standardized products take float32 or float64 input");
    GRGX_CHECK(dtype >= GRGX_F64 && dtype < GRGX_BOOL, GRGX_ERR_UNSUPPORTED,
               "Gram products take numeric (non-bool) input");
    const bool up = (first == GRGX_DIRECTION_UP);
    const uint64_t cols = up ? h.num_samples : h.num_mutations;
    const uint64_t mid = up ? h.num_mutations : h.num_samples;
    GRGX_CHECK(in_cols == cols, GRGX_ERR_API_MISUSE,
               up ? "Input vector is not size N (numSamples, or numIndividuals depending on flags)"
                  : "Input vector is not size M (numMutations)");
    GRGX_CHECK(output_size == rows * cols, GRGX_ERR_API_MISUSE, "Output must be input_rows x input_cols");
    ensure_device_plan(g);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const size_t es = elem(dtype);
    const bool dev = (flags & GRGX_FLAG_DEVICE_POINTERS) != 0;
    const uint32_t pass = (flags & (GRGX_FLAG_F32_PLAIN | GRGX_FLAG_F64_NATIVE)) | GRGX_FLAG_DEVICE_POINTERS |
                          GRGX_FLAG_OVERWRITE;
    void *dIn = const_cast<void*>(input), *dOut = output, *tmp = nullptr;
    GRGX_CUDA(pool_malloc(&tmp, rows * mid * es, s));
    if (!dev) {
        GRGX_CUDA(pool_malloc(&dIn, rows * cols * es, s));
        GRGX_CUDA(cudaMemcpyAsync(dIn, input, rows * cols * es, cudaMemcpyHostToDevice, s));
        GRGX_CUDA(pool_malloc(&dOut, rows * cols * es, s));
    }
    const int second = up ? GRGX_DIRECTION_DOWN : GRGX_DIRECTION_UP;
    if (standardized) {
        matmul_standardized_impl(g, dtype, dIn, cols, rows, first, tmp, rows * mid, pass, stream);
        matmul_standardized_impl(g, dtype, tmp, mid, rows, second, dOut, rows * cols, pass, stream);
    } else {
        matmul_impl(g, dtype, dIn, cols, rows, first, tmp, rows * mid, 0, 0, nullptr, GRGX_INIT_ZERO, nullptr,
                    pass, stream);
        matmul_impl(g, dtype, tmp, mid, rows, second, dOut, rows * cols, 0, 0, nullptr, GRGX_INIT_ZERO, nullptr,
                    pass, stream);
    }
    GRGX_CUDA(cudaFreeAsync(tmp, s));
    if (!dev) {
        GRGX_CUDA(cudaMemcpyAsync(output, dOut, rows * cols * es, cudaMemcpyDeviceToHost, s));
        GRGX_CUDA(cudaFreeAsync(dIn, s));
        GRGX_CUDA(cudaFreeAsync(dOut, s));
        GRGX_CUDA(cudaStreamSynchronize(s));
    } else if (flags & GRGX_FLAG_SYNC) {
        GRGX_CUDA(cudaStreamSynchronize(s));
    }
}

}  // namespace grgx
