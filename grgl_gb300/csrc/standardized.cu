// Products with the standardized genotype matrix Z = (X - 1 mu^T) diag(1/sigma) (haploid
// allele frequencies mu_j = p_j, sigma_j = sqrt(p_j (1 - p_j)), zero columns masked).
//
//   UP   V Z   = (V X - (V 1) mu^T) diag(1/sigma)
//   DOWN V Z^T = X W^T - 1 (mu^T W^T),  W = V diag(1/sigma)
//
// The X products run on the level sweep in the input's dtype.  Everything the result is divided
// by or corrected with -- the allele frequencies (from an exact int32 UP product with ones), the
// row sums V 1 and the scalars mu^T w_k -- is computed in float64 on the device; W is rounded to
// the input dtype before both the DOWN product and its correction use it, so the two agree.
#include <cuda_runtime.h>

#include <mutex>

#include "device_plan.h"

namespace grgx {

void matmul_impl(grgx_graph* g, int dtype, const void* input, uint64_t in_cols, uint64_t rows, int direction,
                 void* output, uint64_t output_size, int emit_all, int by_indiv, const void* init, int init_kind,
                 void* miss, uint32_t flags, void* stream);

namespace {

std::mutex g_stats_mu;

__global__ void fill_ones_kernel(int* p, long long n) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        p[i] = 1;
}

__global__ void stats_kernel(const int* __restrict__ counts, long long M, double N, double* __restrict__ freq,
                             double* __restrict__ invSigma) {
    for (long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x; j < M; j += (long long)gridDim.x * blockDim.x) {
        const double p = static_cast<double>(static_cast<unsigned>(counts[j])) / N;
        const double v = p * (1.0 - p);
        freq[j] = p;
        invSigma[j] = v > 0.0 ? 1.0 / sqrt(v) : 0.0;
    }
}

// Block reduction of a double over 256 threads.
__device__ double block_sum(double x) {
    __shared__ double red[8];
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = x;
    __syncthreads();
    double r = 0.0;
    if (threadIdx.x == 0)
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) r += red[w];
    __syncthreads();
    return r;
}

template <typename T>
__global__ void row_sum_kernel(const T* __restrict__ V, long long K, long long cols, double* __restrict__ out) {
    for (long long k = blockIdx.x; k < K; k += gridDim.x) {
        double acc = 0.0;
        for (long long c = threadIdx.x; c < cols; c += blockDim.x) acc += static_cast<double>(V[k * cols + c]);
        const double r = block_sum(acc);
        if (threadIdx.x == 0) out[k] = r;
    }
}

// W may alias V (the batched path scales stacked rows in place).
template <typename T>
__global__ void down_prepare_kernel(const T* V, long long K, long long M, const double* __restrict__ freq,
                                    const double* __restrict__ invSigma, T* W, double* __restrict__ c) {
    for (long long k = blockIdx.x; k < K; k += gridDim.x) {
        double acc = 0.0;
        for (long long j = threadIdx.x; j < M; j += blockDim.x) {
            const T w = static_cast<T>(static_cast<double>(V[k * M + j]) * invSigma[j]);
            W[k * M + j] = w;
            acc += freq[j] * static_cast<double>(w);
        }
        const double r = block_sum(acc);
        if (threadIdx.x == 0) c[k] = r;
    }
}

// out may alias VX.
template <typename T>
__global__ void up_finish_kernel(const T* VX, const double* __restrict__ rowSum, const double* __restrict__ freq,
                                 const double* __restrict__ invSigma, long long K, long long M, T* out) {
    const long long total = K * M;
    for (long long x = (long long)blockIdx.x * blockDim.x + threadIdx.x; x < total; x += (long long)gridDim.x * blockDim.x) {
        const long long k = x / M, j = x % M;
        out[x] = static_cast<T>((static_cast<double>(VX[x]) - rowSum[k] * freq[j]) * invSigma[j]);
    }
}

template <typename T>
__global__ void down_finish_kernel(T* __restrict__ Y, const double* __restrict__ c, long long K, long long N) {
    const long long total = K * N;
    for (long long x = (long long)blockIdx.x * blockDim.x + threadIdx.x; x < total; x += (long long)gridDim.x * blockDim.x)
        Y[x] = static_cast<T>(static_cast<double>(Y[x]) - c[x / N]);
}

unsigned grid_for(long long n) {
    long long b = (n + 255) / 256;
    const long long cap = static_cast<long long>(sm_count()) * 32;
    if (b > cap) b = cap;
    return (unsigned)(b < 1 ? 1 : b);
}

void ensure_stats(grgx_graph* g, DevicePlan* dp, cudaStream_t s) {
    std::lock_guard<std::mutex> lk(g_stats_mu);
    if (dp->freq) return;
    const HostGraph& h = *g->host;
    const long long N = static_cast<long long>(h.num_samples), M = static_cast<long long>(h.num_mutations);
    int *ones = nullptr, *counts = nullptr;
    GRGX_CUDA(pool_malloc(reinterpret_cast<void**>(&ones), std::max<long long>(N, 1) * sizeof(int), s));
    GRGX_CUDA(pool_malloc(reinterpret_cast<void**>(&counts), std::max<long long>(M, 1) * sizeof(int), s));
    fill_ones_kernel<<<grid_for(N), 256, 0, s>>>(ones, N);
    matmul_impl(g, GRGX_I32, ones, N, 1, GRGX_DIRECTION_UP, counts, M, 0, 0, nullptr, GRGX_INIT_ZERO, nullptr,
                GRGX_FLAG_DEVICE_POINTERS | GRGX_FLAG_OVERWRITE, s);
    double *freq = nullptr, *inv = nullptr;
    GRGX_CUDA(cudaMalloc(&freq, std::max<long long>(M, 1) * sizeof(double)));
    dp->allocs.push_back(freq);
    GRGX_CUDA(cudaMalloc(&inv, std::max<long long>(M, 1) * sizeof(double)));
    dp->allocs.push_back(inv);
    stats_kernel<<<grid_for(M), 256, 0, s>>>(counts, M, static_cast<double>(N), freq, inv);
    GRGX_CUDA(cudaFreeAsync(ones, s));
    GRGX_CUDA(cudaFreeAsync(counts, s));
    GRGX_CUDA(cudaStreamSynchronize(s));
    dp->freq = freq;
    dp->inv_sigma = inv;
}

template <typename T>
void run(grgx_graph* g, DevicePlan* dp, int dtype, const T* in, long long K, int direction, T* out, uint32_t flags,
         cudaStream_t s) {
    const HostGraph& h = *g->host;
    const long long N = static_cast<long long>(h.num_samples), M = static_cast<long long>(h.num_mutations);
    const uint32_t pass = (flags & (GRGX_FLAG_F32_PLAIN | GRGX_FLAG_F64_NATIVE)) | GRGX_FLAG_DEVICE_POINTERS |
                          GRGX_FLAG_OVERWRITE;
    double* red = nullptr;
    GRGX_CUDA(pool_malloc(reinterpret_cast<void**>(&red), K * sizeof(double), s));
    const unsigned rowBlocks = static_cast<unsigned>(std::min<long long>(K, 65535));
    if (direction == GRGX_DIRECTION_UP) {
        T* vx = nullptr;
        GRGX_CUDA(pool_malloc(reinterpret_cast<void**>(&vx), K * M * sizeof(T), s));
        matmul_impl(g, dtype, in, N, K, GRGX_DIRECTION_UP, vx, K * M, 0, 0, nullptr, GRGX_INIT_ZERO, nullptr, pass, s);
        row_sum_kernel<T><<<rowBlocks, 256, 0, s>>>(in, K, N, red);
        up_finish_kernel<T><<<grid_for(K * M), 256, 0, s>>>(vx, red, dp->freq, dp->inv_sigma, K, M, out);
        GRGX_CUDA(cudaFreeAsync(vx, s));
    } else {
        T* w = nullptr;
        GRGX_CUDA(pool_malloc(reinterpret_cast<void**>(&w), K * M * sizeof(T), s));
        down_prepare_kernel<T><<<rowBlocks, 256, 0, s>>>(in, K, M, dp->freq, dp->inv_sigma, w, red);
        matmul_impl(g, dtype, w, M, K, GRGX_DIRECTION_DOWN, out, K * N, 0, 0, nullptr, GRGX_INIT_ZERO, nullptr, pass,
                    s);
        down_finish_kernel<T><<<grid_for(K * N), 256, 0, s>>>(out, red, K, N);
        GRGX_CUDA(cudaFreeAsync(w, s));
    }
    GRGX_CUDA(cudaFreeAsync(red, s));
    GRGX_CUDA(cudaGetLastError());
}

}  // namespace

// ---- pieces for stacked traversals (grgx_matmul_batch, the server) ----------------------------

DevicePlan* standardized_plan(grgx_graph* g, cudaStream_t s) {
    DevicePlan* dp = ensure_device_plan(g);
    ensure_stats(g, dp, s);
    return dp;
}

// V (K x M, in place) becomes W = V diag(1/sigma); c[k] = mu^T w_k.
void standardized_prepare_down(int dtype, const DevicePlan* dp, void* V, long long K, long long M, double* c,
                               cudaStream_t s) {
    const unsigned rowBlocks = static_cast<unsigned>(std::min<long long>(K, 65535));
    if (dtype == GRGX_F64)
        down_prepare_kernel<double><<<rowBlocks, 256, 0, s>>>(static_cast<double*>(V), K, M, dp->freq, dp->inv_sigma,
                                                              static_cast<double*>(V), c);
    else
        down_prepare_kernel<float><<<rowBlocks, 256, 0, s>>>(static_cast<float*>(V), K, M, dp->freq, dp->inv_sigma,
                                                             static_cast<float*>(V), c);
    GRGX_CUDA(cudaGetLastError());
}

// Y (K x N, in place) -= c[k].
void standardized_finish_down(int dtype, void* Y, const double* c, long long K, long long N, cudaStream_t s) {
    if (dtype == GRGX_F64)
        down_finish_kernel<double><<<grid_for(K * N), 256, 0, s>>>(static_cast<double*>(Y), c, K, N);
    else
        down_finish_kernel<float><<<grid_for(K * N), 256, 0, s>>>(static_cast<float*>(Y), c, K, N);
    GRGX_CUDA(cudaGetLastError());
}

// VX (K x M, in place) becomes (VX - (V 1) mu^T) diag(1/sigma); `red` holds K doubles.
void standardized_finish_up(int dtype, const DevicePlan* dp, const void* V, long long K, long long N, void* VX,
                            long long M, double* red, cudaStream_t s) {
    const unsigned rowBlocks = static_cast<unsigned>(std::min<long long>(K, 65535));
    if (dtype == GRGX_F64) {
        row_sum_kernel<double><<<rowBlocks, 256, 0, s>>>(static_cast<const double*>(V), K, N, red);
        up_finish_kernel<double><<<grid_for(K * M), 256, 0, s>>>(static_cast<double*>(VX), red, dp->freq,
                                                                 dp->inv_sigma, K, M, static_cast<double*>(VX));
    } else {
        row_sum_kernel<float><<<rowBlocks, 256, 0, s>>>(static_cast<const float*>(V), K, N, red);
        up_finish_kernel<float><<<grid_for(K * M), 256, 0, s>>>(static_cast<float*>(VX), red, dp->freq,
                                                                dp->inv_sigma, K, M, static_cast<float*>(VX));
    }
    GRGX_CUDA(cudaGetLastError());
}

void matmul_standardized_impl(grgx_graph* g, int dtype, const void* input, uint64_t in_cols, uint64_t rows,
                              int direction, void* output, uint64_t output_size, uint32_t flags, void* stream) {
    const HostGraph& h = *g->host;
    GRGX_CHECK(dtype == GRGX_F32 || dtype == GRGX_F64, GRGX_ERR_UNSUPPORTED,
               "standardized products take float32 or float64 input");
    GRGX_CHECK(direction == GRGX_DIRECTION_DOWN || direction == GRGX_DIRECTION_UP, GRGX_ERR_API_MISUSE,
               "Invalid traversal direction");
    GRGX_CHECK(in_cols > 0 && rows > 0, GRGX_ERR_API_MISUSE, "matmul() requires non-zero dimensions.");
    const bool up = (direction == GRGX_DIRECTION_UP);
    GRGX_CHECK(in_cols == (up ? h.num_samples : h.num_mutations), GRGX_ERR_API_MISUSE,
               up ? "Input vector is not size N (numSamples, or numIndividuals depending on flags)"
                  : "Input vector is not size M (numMutations)");
    const uint64_t outCols = up ? h.num_mutations : h.num_samples;
    GRGX_CHECK(output_size == rows * outCols, GRGX_ERR_API_MISUSE,
               up ? "Output vector is not size M (numMutations)"
                  : "Output vector is not size N (numSamples, or numIndividuals depending on flags)");
    DevicePlan* dp = ensure_device_plan(g);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    ensure_stats(g, dp, s);
    const size_t es = (dtype == GRGX_F64) ? 8 : 4;
    const bool dev = (flags & GRGX_FLAG_DEVICE_POINTERS) != 0;
    const void* dIn = input;
    void* dOut = output;
    if (!dev) {
        void* a = nullptr;
        GRGX_CUDA(pool_malloc(&a, rows * in_cols * es, s));
        GRGX_CUDA(cudaMemcpyAsync(a, input, rows * in_cols * es, cudaMemcpyHostToDevice, s));
        dIn = a;
        GRGX_CUDA(pool_malloc(&dOut, rows * outCols * es, s));
    }
    if (dtype == GRGX_F64)
        run<double>(g, dp, dtype, static_cast<const double*>(dIn), static_cast<long long>(rows), direction,
                    static_cast<double*>(dOut), flags, s);
    else
        run<float>(g, dp, dtype, static_cast<const float*>(dIn), static_cast<long long>(rows), direction,
                   static_cast<float*>(dOut), flags, s);
    if (!dev) {
        GRGX_CUDA(cudaMemcpyAsync(output, dOut, rows * outCols * es, cudaMemcpyDeviceToHost, s));
        GRGX_CUDA(cudaFreeAsync(const_cast<void*>(dIn), s));
        GRGX_CUDA(cudaFreeAsync(dOut, s));
        GRGX_CUDA(cudaStreamSynchronize(s));
    } else if (flags & GRGX_FLAG_SYNC) {
        GRGX_CUDA(cudaStreamSynchronize(s));
    }
}

}  // namespace grgx
