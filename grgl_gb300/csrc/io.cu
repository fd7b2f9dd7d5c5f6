// Seed and gather kernels: moving K x cols row-major matrices (the reference's I/O layout,
// grg.h:1341-1517) into and out of the node-major value rows the sweep works on.
//
// Both directions use 32 x 32 shared-memory tiles so that the global reads and writes are
// coalesced on both sides of the transpose.  Element conversion between the I/O type and the
// storage type follows the accumulation kinds of ops.cuh: narrow integers are widened to 32
// bits (residues mod 2^bits are preserved) and truncated on output.
#include <cstdint>
#include <stdexcept>

#include "grgx.h"
#include "launch.h"

namespace grgx {
namespace {

constexpr uint32_t kInvalid = 0x7fffffffu;

template <typename IO> struct Store;
template <> struct Store<double> { using S = double; };
template <> struct Store<float> { using S = float; };
template <> struct Store<int64_t> { using S = unsigned long long; };
template <> struct Store<uint64_t> { using S = unsigned long long; };
template <> struct Store<int32_t> { using S = uint32_t; };
template <> struct Store<uint32_t> { using S = uint32_t; };
template <> struct Store<int16_t> { using S = uint32_t; };
template <> struct Store<uint16_t> { using S = uint32_t; };
template <> struct Store<int8_t> { using S = uint32_t; };
template <> struct Store<uint8_t> { using S = uint32_t; };

template <typename IO> struct Unsigned { using U = IO; };
template <> struct Unsigned<int64_t> { using U = unsigned long long; };
template <> struct Unsigned<uint64_t> { using U = unsigned long long; };
template <> struct Unsigned<int32_t> { using U = uint32_t; };
template <> struct Unsigned<int16_t> { using U = uint16_t; };
template <> struct Unsigned<int8_t> { using U = uint8_t; };

template <typename IO> __device__ __forceinline__ typename Store<IO>::S to_s(IO x) {
    using S = typename Store<IO>::S;
    using U = typename Unsigned<IO>::U;
    return static_cast<S>(static_cast<U>(x));
}
template <> __device__ __forceinline__ double to_s<double>(double x) { return x; }
template <> __device__ __forceinline__ float to_s<float>(float x) { return x; }

template <typename IO> __device__ __forceinline__ IO from_s(typename Store<IO>::S s) {
    using U = typename Unsigned<IO>::U;
    return static_cast<IO>(static_cast<U>(s));
}
template <> __device__ __forceinline__ double from_s<double>(double s) { return s; }
template <> __device__ __forceinline__ float from_s<float>(float s) { return s; }

// a + b with the reference's `+=` semantics (wrap-around for integers).
template <typename IO> __device__ __forceinline__ IO io_add(IO a, IO b) {
    using U = typename Unsigned<IO>::U;
    return static_cast<IO>(static_cast<U>(static_cast<U>(a) + static_cast<U>(b)));
}
template <> __device__ __forceinline__ double io_add<double>(double a, double b) { return a + b; }
template <> __device__ __forceinline__ float io_add<float>(float a, float b) { return a + b; }

template <typename S> __device__ __forceinline__ S s_add(S a, S b) { return a + b; }

template <typename IO>
__global__ void load_rows_kernel(const IO* __restrict__ src, long long K, long long ld, long long R, int mode,
                                 long long div, const uint32_t* __restrict__ tab,
                                 typename Store<IO>::S* __restrict__ dst, long long stride, int add,
                                 const int* gate, int gate_value) {
    using S = typename Store<IO>::S;
    if (gate != nullptr && *gate != gate_value) return;
    __shared__ S tile[32][33];
    const long long i0 = (long long)blockIdx.x * 32, k0 = (long long)blockIdx.y * 32;
    const int tx = threadIdx.x, ty = threadIdx.y;
    const long long i = i0 + tx;
    long long colIdx = -1;
    if (i < R) colIdx = (mode == MAP_DIV) ? i / div : (mode == MAP_TABLE ? (long long)tab[i] : i);
#pragma unroll
    for (int j = ty; j < 32; j += 8) {
        const long long k = k0 + j;
        tile[j][tx] = (k < K && colIdx >= 0) ? to_s<IO>(src[k * ld + colIdx]) : S(0);
    }
    __syncthreads();
#pragma unroll
    for (int j = ty; j < 32; j += 8) {
        const long long r = i0 + j, k = k0 + tx;
        if (r < R && k < stride) {
            S* d = dst + r * stride + k;
            if (add) {
                if (k < K) *d = s_add<S>(*d, tile[tx][j]);
            } else {
                *d = tile[tx][j];
            }
        }
    }
}

template <typename IO>
__global__ void store_cols_kernel(const typename Store<IO>::S* __restrict__ vals, long long stride, long long K,
                                  long long C, int mode, long long fold, const uint32_t* __restrict__ tab,
                                  IO* __restrict__ out, long long ld, int add, const int* gate, int gate_value) {
    using S = typename Store<IO>::S;
    if (gate != nullptr && *gate != gate_value) return;
    __shared__ S tile[32][33];
    const long long c0 = (long long)blockIdx.x * 32, k0 = (long long)blockIdx.y * 32;
    const int tx = threadIdx.x, ty = threadIdx.y;
#pragma unroll
    for (int j = ty; j < 32; j += 8) {
        const long long c = c0 + j, k = k0 + tx;
        S v = S(0);
        if (c < C && k < K) {
            if (mode == MAP_FOLD) {
                for (long long p = 0; p < fold; p++) v = (p == 0) ? vals[(c * fold) * stride + k]
                                                                   : s_add<S>(v, vals[(c * fold + p) * stride + k]);
            } else {
                const long long node = (mode == MAP_TABLE) ? (long long)tab[c] : c;
                if (node != (long long)kInvalid) v = vals[node * stride + k];
            }
        }
        tile[j][tx] = v;
    }
    __syncthreads();
#pragma unroll
    for (int j = ty; j < 32; j += 8) {
        const long long k = k0 + j, c = c0 + tx;
        if (k < K && c < C) {
            IO* o = out + k * ld + c;
            const IO x = from_s<IO>(tile[tx][j]);
            *o = add ? io_add<IO>(*o, x) : x;
        }
    }
}

template <typename IO>
__global__ void init_vector_kernel(const IO* __restrict__ init, long long K, long long n,
                                   typename Store<IO>::S* __restrict__ vals, long long stride, const int* gate,
                                   int gate_value) {
    using S = typename Store<IO>::S;
    if (gate != nullptr && *gate != gate_value) return;
    const long long total = n * stride;
    for (long long x = (long long)blockIdx.x * blockDim.x + threadIdx.x; x < total;
         x += (long long)gridDim.x * blockDim.x) {
        const long long k = x % stride;
        vals[x] = (k < K) ? to_s<IO>(init[k]) : S(0);
    }
}

template <typename IO>
__global__ void init_xtx_kernel(const uint32_t* __restrict__ xtx, long long K, long long n,
                                typename Store<IO>::S* __restrict__ vals, long long stride, const int* gate,
                                int gate_value) {
    using S = typename Store<IO>::S;
    if (gate != nullptr && *gate != gate_value) return;
    const long long total = n * stride;
    for (long long x = (long long)blockIdx.x * blockDim.x + threadIdx.x; x < total;
         x += (long long)gridDim.x * blockDim.x) {
        const long long k = x % stride, v = x / stride;
        vals[x] = (k < K) ? to_s<IO>(static_cast<IO>(xtx[v])) : S(0);
    }
}

// ---- GF(2): one byte per value in I/O, 32 columns per storage word ----------------------------

__global__ void load_bits_kernel(const uint8_t* __restrict__ src, long long K, long long ld, long long R, int mode,
                                 long long div, const uint32_t* __restrict__ tab, uint32_t* __restrict__ dst,
                                 long long stride, int add) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long w = blockIdx.y;
    if (i >= R || w >= stride) return;
    const long long colIdx = (mode == MAP_DIV) ? i / div : (mode == MAP_TABLE ? (long long)tab[i] : i);
    uint32_t word = 0;
    for (int b = 0; b < 32; b++) {
        const long long k = w * 32 + b;
        if (k < K && src[k * ld + colIdx]) word |= (1u << b);
    }
    uint32_t* d = dst + i * stride + w;
    *d = add ? (*d ^ word) : word;
}

__global__ void store_bits_kernel(const uint32_t* __restrict__ vals, long long stride, long long K, long long C,
                                  int mode, long long fold, const uint32_t* __restrict__ tab, uint8_t* __restrict__ out,
                                  long long ld, int add) {
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long k = blockIdx.y;
    if (c >= C || k >= K) return;
    const long long w = k >> 5;
    const uint32_t bit = 1u << (k & 31);
    uint32_t v = 0;
    if (mode == MAP_FOLD) {
        for (long long p = 0; p < fold; p++) v ^= vals[(c * fold + p) * stride + w];
    } else {
        const long long node = (mode == MAP_TABLE) ? (long long)tab[c] : c;
        if (node != (long long)kInvalid) v = vals[node * stride + w];
    }
    const uint8_t x = (v & bit) ? 1 : 0;
    uint8_t* o = out + k * ld + c;
    *o = add ? static_cast<uint8_t>((*o != 0) != (x != 0)) : x;
}

template <typename IO>
void load_rows_t(const void* src, long long K, long long ld, long long R, int mode, long long div, const uint32_t* tab,
                 void* dst, long long stride, int add, const int* gate, int gv, cudaStream_t s) {
    if (R <= 0) return;
    const dim3 grid((unsigned)((R + 31) / 32), (unsigned)((stride + 31) / 32));
    load_rows_kernel<IO><<<grid, dim3(32, 8), 0, s>>>(static_cast<const IO*>(src), K, ld, R, mode, div, tab,
                                                      static_cast<typename Store<IO>::S*>(dst), stride, add, gate, gv);
}

template <typename IO>
void store_cols_t(const void* vals, long long stride, long long K, long long C, int mode, long long fold,
                  const uint32_t* tab, void* out, long long ld, int add, const int* gate, int gv, cudaStream_t s) {
    if (C <= 0 || K <= 0) return;
    const dim3 grid((unsigned)((C + 31) / 32), (unsigned)((K + 31) / 32));
    store_cols_kernel<IO><<<grid, dim3(32, 8), 0, s>>>(static_cast<const typename Store<IO>::S*>(vals), stride, K,
                                                       C, mode, fold, tab, static_cast<IO*>(out), ld, add, gate, gv);
}

unsigned grid_for(long long total) {
    long long b = (total + 255) / 256;
    const long long cap = static_cast<long long>(sm_count()) * 32;
    if (b > cap) b = cap;
    return (unsigned)(b < 1 ? 1 : b);
}

}  // namespace

#define GRGX_IO_DISPATCH(dtype, CALL)                                        \
    switch (dtype) {                                                         \
    case GRGX_F64: CALL(double); break;                                      \
    case GRGX_F32: CALL(float); break;                                       \
    case GRGX_I64: CALL(int64_t); break;                                     \
    case GRGX_I32: CALL(int32_t); break;                                     \
    case GRGX_I16: CALL(int16_t); break;                                     \
    case GRGX_I8: CALL(int8_t); break;                                       \
    case GRGX_U64: CALL(uint64_t); break;                                    \
    case GRGX_U32: CALL(uint32_t); break;                                    \
    case GRGX_U16: CALL(uint16_t); break;                                    \
    case GRGX_U8: CALL(uint8_t); break;                                      \
    default: throw std::runtime_error("unsupported dtype");                  \
    }

void launch_load_rows(int dtype, const void* src, long long K, long long ld, long long R, int mode, long long div,
                      const uint32_t* tab, void* dst, long long stride, int add, cudaStream_t s, const int* gate,
                      int gv) {
    if (dtype == GRGX_BOOL) {
        if (R <= 0) return;
        const dim3 grid((unsigned)((R + 127) / 128), (unsigned)stride);
        load_bits_kernel<<<grid, 128, 0, s>>>(static_cast<const uint8_t*>(src), K, ld, R, mode, div, tab,
                                              static_cast<uint32_t*>(dst), stride, add);
        return;
    }
#define CALL(T) load_rows_t<T>(src, K, ld, R, mode, div, tab, dst, stride, add, gate, gv, s)
    GRGX_IO_DISPATCH(dtype, CALL)
#undef CALL
}

void launch_store_cols(int dtype, const void* vals, long long stride, long long K, long long C, int mode,
                       long long fold, const uint32_t* tab, void* out, long long ld, int add, cudaStream_t s,
                       const int* gate, int gv) {
    if (dtype == GRGX_BOOL) {
        if (C <= 0 || K <= 0) return;
        const dim3 grid((unsigned)((C + 127) / 128), (unsigned)K);
        store_bits_kernel<<<grid, 128, 0, s>>>(static_cast<const uint32_t*>(vals), stride, K, C, mode, fold, tab,
                                               static_cast<uint8_t*>(out), ld, add);
        return;
    }
#define CALL(T) store_cols_t<T>(vals, stride, K, C, mode, fold, tab, out, ld, add, gate, gv, s)
    GRGX_IO_DISPATCH(dtype, CALL)
#undef CALL
}

void launch_init_vector(int dtype, const void* init, long long K, long long n, void* vals, long long stride,
                        cudaStream_t s, const int* gate, int gv) {
    const unsigned grid = grid_for(n * stride);
#define CALL(T)                                                                                            \
    init_vector_kernel<T><<<grid, 256, 0, s>>>(static_cast<const T*>(init), K, n,                          \
                                               static_cast<typename Store<T>::S*>(vals), stride, gate, gv)
    GRGX_IO_DISPATCH(dtype, CALL)
#undef CALL
}

void launch_init_xtx(int dtype, const uint32_t* xtx, long long K, long long n, void* vals, long long stride,
                     cudaStream_t s, const int* gate, int gv) {
    const unsigned grid = grid_for(n * stride);
#define CALL(T) \
    init_xtx_kernel<T><<<grid, 256, 0, s>>>(xtx, K, n, static_cast<typename Store<T>::S*>(vals), stride, gate, gv)
    GRGX_IO_DISPATCH(dtype, CALL)
#undef CALL
}

}  // namespace grgx
