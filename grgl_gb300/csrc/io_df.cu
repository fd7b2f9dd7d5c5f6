// Seed and gather kernels for float64 carried as scaled float pairs (AddF64S, ops.cuh).
//
// Each input row k is scaled by the exact power of two 2^-e_k (e_k = exponent of the row's
// largest finite magnitude, clamped to the normal range) before it is split into hi + lo floats,
// and the outputs are scaled back by 2^e_k; scaling by powers of two is exact, so the only
// rounding is the split's 2^-48 relative representation error.
#include <cstdint>

#include "launch.h"

namespace grgx {
namespace {

constexpr uint32_t kInvalid = 0x7fffffffu;
constexpr unsigned long long kExpMask = 0x7ff0000000000000ull;

// Scale exponent of row k: the row is multiplied by 2^-row_exp, which puts its largest value in
// [2^60, 2^61) (clamped so both 2^row_exp and 2^-row_exp are normal doubles).
__device__ __forceinline__ int row_exp(const unsigned long long* rowmax, long long k) {
    const unsigned long long b = rowmax[k];
    if (b == 0) return 0;
    int e = static_cast<int>((b >> 52) & 0x7ff) - 1023 - 60;
    return e < -1022 ? -1022 : (e > 1022 ? 1022 : e);
}

// Binades spanned by the nonzero finite magnitudes of a row beyond which the float-pair path
// would lose the smallest terms (max at 2^60, float normals reach 2^-126).
constexpr int kMaxBinades = 180;

// 2^e for e in [-1022, 1023], built from its bit pattern (exact).
__device__ __forceinline__ double pow2(int e) {
    return __longlong_as_double(static_cast<long long>(e + 1023) << 52);
}

__global__ void fill_u64_kernel(unsigned long long* p, long long n, unsigned long long v) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        p[i] = v;
}

__global__ void rowmax_kernel(const double* __restrict__ src, long long K, long long ld, long long cols,
                              unsigned long long* __restrict__ rowmax, unsigned long long* __restrict__ rowmin) {
    __shared__ unsigned long long redMax[8], redMin[8];
    for (long long k = blockIdx.y; k < K; k += gridDim.y) {
        unsigned long long m = 0, mn = ~0ull;
        for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < cols;
             c += (long long)gridDim.x * blockDim.x) {
            const unsigned long long b = static_cast<unsigned long long>(__double_as_longlong(src[k * ld + c])) &
                                         0x7fffffffffffffffull;
            if ((b & kExpMask) != kExpMask) {  // finite
                m = b > m ? b : m;
                if (b != 0) mn = b < mn ? b : mn;
            } else {
                mn = 0;  // inf or nan: marks the row for the FP64 path
            }
        }
        for (int o = 16; o > 0; o >>= 1) {
            const unsigned long long t = __shfl_xor_sync(0xffffffffu, m, o);
            const unsigned long long u = __shfl_xor_sync(0xffffffffu, mn, o);
            m = t > m ? t : m;
            mn = u < mn ? u : mn;
        }
        if ((threadIdx.x & 31) == 0) {
            redMax[threadIdx.x >> 5] = m;
            redMin[threadIdx.x >> 5] = mn;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            unsigned long long r = 0, q = ~0ull;
            for (int w = 0; w < (int)(blockDim.x >> 5); w++) {
                r = redMax[w] > r ? redMax[w] : r;
                q = redMin[w] < q ? redMin[w] : q;
            }
            if (r) atomicMax(rowmax + k, r);
            if (q != ~0ull) atomicMin(rowmin + k, q);  // 0 when the row holds an inf or a nan
        }
        __syncthreads();
    }
}

__global__ void decide_kernel(const unsigned long long* __restrict__ rowmax, const unsigned long long* __restrict__ rowmin,
                              long long K, int* __restrict__ gate) {
    __shared__ int wide;
    if (threadIdx.x == 0) wide = 0;
    __syncthreads();
    for (long long k = threadIdx.x; k < K; k += blockDim.x) {
        const unsigned long long mx = rowmax[k], mn = rowmin[k];
        if (mn == 0) {  // an inf or a nan: only the FP64 path carries IEEE semantics through
            wide = 1;
            continue;
        }
        if (mx == 0 || mn == ~0ull) continue;
        const int emax = static_cast<int>((mx >> 52) & 0x7ff), emin = static_cast<int>((mn >> 52) & 0x7ff);
        const int re = row_exp(rowmax, k);
        // subnormal terms, or scaled magnitudes outside [2^-120, 2^62]
        if (emin == 0 || emax - emin > kMaxBinades || (emin - 1023) - re < -120 || (emax - 1023) - re > 62) wide = 1;
    }
    __syncthreads();
    if (threadIdx.x == 0) gate[0] = wide;
}

__device__ __forceinline__ DF split_scaled(double x, int e) { return AddF64S::split(x * pow2(-e)); }

__global__ void load_rows_df_kernel(const double* __restrict__ src, long long K, long long ld, long long R, int mode,
                                    long long div, const uint32_t* __restrict__ tab, DF* __restrict__ dst,
                                    long long stride, int add, const unsigned long long* __restrict__ rowmax,
                                    const int* gate) {
    if (gate != nullptr && *gate != 0) return;
    __shared__ DF tile[32][33];
    const long long i0 = (long long)blockIdx.x * 32, k0 = (long long)blockIdx.y * 32;
    const int tx = threadIdx.x, ty = threadIdx.y;
    const long long i = i0 + tx;
    long long colIdx = -1;
    if (i < R) colIdx = (mode == MAP_DIV) ? i / div : (mode == MAP_TABLE ? (long long)tab[i] : i);
#pragma unroll
    for (int j = ty; j < 32; j += 8) {
        const long long k = k0 + j;
        tile[j][tx] = (k < K && colIdx >= 0) ? split_scaled(src[k * ld + colIdx], row_exp(rowmax, k)) : DF{0.f, 0.f};
    }
    __syncthreads();
#pragma unroll
    for (int j = ty; j < 32; j += 8) {
        const long long r = i0 + j, k = k0 + tx;
        if (r < R && k < stride) {
            const long long e = r * stride + k;
            if (add) {
                if (k < K)
                    df_put(dst, e, stride,
                           AddF64S::split(AddF64S::value(df_get(dst, e, stride)) + AddF64S::value(tile[tx][j])));
            } else {
                df_put(dst, e, stride, tile[tx][j]);
            }
        }
    }
}

__global__ void store_cols_df_kernel(const DF* __restrict__ vals, long long stride, long long K, long long C,
                                     int mode, long long fold, const uint32_t* __restrict__ tab,
                                     double* __restrict__ out, long long ld, int add,
                                     const unsigned long long* __restrict__ rowmax, const int* gate) {
    if (gate != nullptr && *gate != 0) return;
    __shared__ double tile[32][33];
    const long long c0 = (long long)blockIdx.x * 32, k0 = (long long)blockIdx.y * 32;
    const int tx = threadIdx.x, ty = threadIdx.y;
#pragma unroll
    for (int j = ty; j < 32; j += 8) {
        const long long c = c0 + j, k = k0 + tx;
        double v = 0.0;
        if (c < C && k < K) {
            if (mode == MAP_FOLD) {
                for (long long p = 0; p < fold; p++) v += AddF64S::value(df_get(vals, (c * fold + p) * stride + k, stride));
            } else {
                const long long node = (mode == MAP_TABLE) ? (long long)tab[c] : c;
                if (node != (long long)kInvalid) v = AddF64S::value(df_get(vals, node * stride + k, stride));
            }
            v *= pow2(row_exp(rowmax, k));
        }
        tile[j][tx] = v;
    }
    __syncthreads();
#pragma unroll
    for (int j = ty; j < 32; j += 8) {
        const long long k = k0 + j, c = c0 + tx;
        if (k < K && c < C) {
            double* o = out + k * ld + c;
            *o = add ? (*o + tile[tx][j]) : tile[tx][j];
        }
    }
}

__global__ void init_vector_df_kernel(const double* __restrict__ init, long long K, long long n, DF* __restrict__ vals,
                                      long long stride, const unsigned long long* __restrict__ rowmax,
                                      const int* gate) {
    if (gate != nullptr && *gate != 0) return;
    const long long total = n * stride;
    for (long long x = (long long)blockIdx.x * blockDim.x + threadIdx.x; x < total;
         x += (long long)gridDim.x * blockDim.x) {
        const long long k = x % stride;
        df_put(vals, x, stride, (k < K) ? split_scaled(init[k], row_exp(rowmax, k)) : DF{0.f, 0.f});
    }
}

__global__ void init_xtx_df_kernel(const uint32_t* __restrict__ xtx, long long K, long long n, DF* __restrict__ vals,
                                   long long stride, const unsigned long long* __restrict__ rowmax, const int* gate) {
    if (gate != nullptr && *gate != 0) return;
    const long long total = n * stride;
    for (long long x = (long long)blockIdx.x * blockDim.x + threadIdx.x; x < total;
         x += (long long)gridDim.x * blockDim.x) {
        const long long k = x % stride, v = x / stride;
        df_put(vals, x, stride, (k < K) ? split_scaled(static_cast<double>(xtx[v]), row_exp(rowmax, k)) : DF{0.f, 0.f});
    }
}

unsigned grid_for(long long total) {
    long long b = (total + 255) / 256;
    const long long cap = static_cast<long long>(sm_count()) * 32;
    if (b > cap) b = cap;
    return (unsigned)(b < 1 ? 1 : b);
}

}  // namespace

void launch_fill_u64(unsigned long long* p, long long n, unsigned long long v, cudaStream_t s) {
    if (n <= 0) return;
    fill_u64_kernel<<<grid_for(n), 256, 0, s>>>(p, n, v);
}

void launch_rowmax(const double* src, long long K, long long ld, long long cols, unsigned long long* rowmax,
                   unsigned long long* rowmin, cudaStream_t s) {
    if (K <= 0 || cols <= 0) return;
    long long bx = (cols + 256 * 8 - 1) / (256 * 8);
    if (bx > 1024) bx = 1024;
    const long long by = K < 65535 ? K : 65535;
    rowmax_kernel<<<dim3((unsigned)bx, (unsigned)by), 256, 0, s>>>(src, K, ld, cols, rowmax, rowmin);
}

void launch_decide_f64_path(const unsigned long long* rowmax, const unsigned long long* rowmin, long long K, int* gate,
                            cudaStream_t s) {
    decide_kernel<<<1, 256, 0, s>>>(rowmax, rowmin, K, gate);
}

void launch_load_rows_df(const double* src, long long K, long long ld, long long R, int mode, long long div,
                         const uint32_t* tab, void* dst, long long stride, int add,
                         const unsigned long long* rowmax, cudaStream_t s, const int* gate) {
    if (R <= 0) return;
    const dim3 grid((unsigned)((R + 31) / 32), (unsigned)((stride + 31) / 32));
    load_rows_df_kernel<<<grid, dim3(32, 8), 0, s>>>(src, K, ld, R, mode, div, tab, static_cast<DF*>(dst), stride,
                                                     add, rowmax, gate);
}

void launch_store_cols_df(const void* vals, long long stride, long long K, long long C, int mode, long long fold,
                          const uint32_t* tab, double* out, long long ld, int add,
                          const unsigned long long* rowmax, cudaStream_t s, const int* gate) {
    if (C <= 0 || K <= 0) return;
    const dim3 grid((unsigned)((C + 31) / 32), (unsigned)((K + 31) / 32));
    store_cols_df_kernel<<<grid, dim3(32, 8), 0, s>>>(static_cast<const DF*>(vals), stride, K, C, mode, fold, tab,
                                                      out, ld, add, rowmax, gate);
}

void launch_init_vector_df(const double* init, long long K, long long n, void* vals, long long stride,
                           const unsigned long long* rowmax, cudaStream_t s, const int* gate) {
    init_vector_df_kernel<<<grid_for(n * stride), 256, 0, s>>>(init, K, n, static_cast<DF*>(vals), stride, rowmax,
                                                               gate);
}

void launch_init_xtx_df(const uint32_t* xtx, long long K, long long n, void* vals, long long stride,
                        const unsigned long long* rowmax, cudaStream_t s, const int* gate) {
    init_xtx_df_kernel<<<grid_for(n * stride), 256, 0, s>>>(xtx, K, n, static_cast<DF*>(vals), stride, rowmax, gate);
}

}  // namespace grgx
