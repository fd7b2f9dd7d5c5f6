// Host-side launch entry points of the device kernels (internal to libgrgx).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "sweep.cuh"

namespace grgx {

// SM count of the current device (looked up once per device, matmul.cu).
int sm_count();

// Storage/accumulation kinds (see ops.cuh).
enum class Kind { U32, U64, F64, F32C, F32, XOR, F64S };

// One level (or seed pass) of the sweep; VW elements per lane, G lanes per row, `variant` 0 for
// the default depth or 1 for the deep variant (float32, compensated float32, int32 and
// float-pair float64 storage only).
void launch_sweep_u32(const SweepParams<uint32_t>& p, int vw, int g, int variant, dim3 grid,
                      int sms, cudaStream_t s);
void launch_sweep_xor(const SweepParams<uint32_t>& p, int vw, int g, int variant, dim3 grid,
                      int sms, cudaStream_t s);
void launch_sweep_u64(const SweepParams<unsigned long long>& p, int vw, int g, int variant, dim3 grid,
                      int sms, cudaStream_t s);
void launch_sweep_f64(const SweepParams<double>& p, int vw, int g, int variant, dim3 grid,
                      int sms, cudaStream_t s);
void launch_sweep_f32c(const SweepParams<float>& p, int vw, int g, int variant, dim3 grid,
                      int sms, cudaStream_t s);
void launch_sweep_f32(const SweepParams<float>& p, int vw, int g, int variant, dim3 grid,
                      int sms, cudaStream_t s);
void launch_sweep_f64s(const SweepParams<DF>& p, int vw, int g, int variant, dim3 grid,
                      int sms, cudaStream_t s);

// Staged single-column sweeps of one split block (sweep_kernel_staged; p.src = the block's first
// source value, p.src_rows <= kStagedRows values), 4-byte storage kinds.
void launch_sweep_staged_u32(const SweepParams<uint32_t>& p, dim3 grid, cudaStream_t s);
void launch_sweep_staged_xor(const SweepParams<uint32_t>& p, dim3 grid, cudaStream_t s);
void launch_sweep_staged_f32c(const SweepParams<float>& p, dim3 grid, cudaStream_t s);
void launch_sweep_staged_f32(const SweepParams<float>& p, dim3 grid, cudaStream_t s);

// Column-map modes of the transposing loads/stores.
enum MapMode { MAP_IDENT = 0, MAP_DIV = 1, MAP_TABLE = 2, MAP_FOLD = 3 };

// dst[i*stride + k] (=, or += when add) IO->S(src[k*ld + col(i)]) for i < R, k < K; columns
// K..stride-1 are zeroed when assigning.  col(i) = i, i/div, or tab[i].
// `gate`: when non-null the kernel runs only if *gate == gate_value (device-side path choice).
void launch_load_rows(int dtype, const void* src, long long K, long long ld, long long R, int mode, long long div,
                      const uint32_t* tab, void* dst, long long stride, int add, cudaStream_t s,
                      const int* gate = nullptr, int gate_value = 0);

// out[k*ld + c] (=, or += when add) S->IO(vals[map(c)]) for c < C, k < K; map(c) = c, tab[c]
// (INVALID -> 0), or the sum of rows c*fold .. c*fold+fold-1.
void launch_store_cols(int dtype, const void* vals, long long stride, long long K, long long C, int mode,
                       long long fold, const uint32_t* tab, void* out, long long ld, int add, cudaStream_t s,
                       const int* gate = nullptr, int gate_value = 0);

// Node-value initialisation: VECTOR (vals[v][k] = init[k]) and XTX (vals[v][k] = xtx[v]).
void launch_init_vector(int dtype, const void* init, long long K, long long n, void* vals, long long stride,
                        cudaStream_t s, const int* gate = nullptr, int gate_value = 0);
void launch_init_xtx(int dtype, const uint32_t* xtx, long long K, long long n, void* vals, long long stride,
                     cudaStream_t s, const int* gate = nullptr, int gate_value = 0);

// ---- float64 as scaled float pairs (AddF64S) ----------------------------------------------
// rowmax[k] = max over finite |x| of row k, as IEEE bits (0 for an all-zero row); callers
// fill it first (0, or a floor such as the largest XTX init value) and may fold several
// matrices into it.  Row k is scaled by 2^(60 - e_k), e_k the exponent of rowmax[k], so the
// row's largest value sits in [2^60, 2^61) and values down to 2^-126 of float range (186
// binades below the maximum) keep full precision.  The float-pair kernels run when
// gate[0] == 0.
void launch_fill_u64(unsigned long long* p, long long n, unsigned long long v, cudaStream_t s);
// Also folds the smallest nonzero finite magnitude into rowmin[k] (filled with ~0 first).
void launch_rowmax(const double* src, long long K, long long ld, long long cols, unsigned long long* rowmax,
                   unsigned long long* rowmin, cudaStream_t s);
// gate[0] = 1 when some row spans more binades than the float-pair path holds, or holds an inf
// or a nan (the call then runs on the FP64 pipe), else 0.
void launch_decide_f64_path(const unsigned long long* rowmax, const unsigned long long* rowmin, long long K, int* gate,
                            cudaStream_t s);
void launch_load_rows_df(const double* src, long long K, long long ld, long long R, int mode, long long div,
                         const uint32_t* tab, void* dst, long long stride, int add,
                         const unsigned long long* rowmax, cudaStream_t s, const int* gate);
void launch_store_cols_df(const void* vals, long long stride, long long K, long long C, int mode, long long fold,
                          const uint32_t* tab, double* out, long long ld, int add,
                          const unsigned long long* rowmax, cudaStream_t s, const int* gate);
void launch_init_vector_df(const double* init, long long K, long long n, void* vals, long long stride,
                           const unsigned long long* rowmax, cudaStream_t s, const int* gate);
void launch_init_xtx_df(const uint32_t* xtx, long long K, long long n, void* vals, long long stride,
                        const unsigned long long* rowmax, cudaStream_t s, const int* gate);

}  // namespace grgx
