// grgx_matmul_noalloc: the plain matmul for callers that may not allocate device memory.
//
// Some callers cannot call cudaMalloc or any allocating routine once they are running: a host
// program that hands out a fixed device-memory budget at start-up and forbids allocation
// afterwards (a real-time pipeline, or a framework whose own allocator owns every device byte),
// or code that must not grow its footprint while it serves requests.  This entry point runs the
// same kernels as grgx_matmul, but every byte of scratch it needs -- the node values, the
// per-mutation input rows of a DOWN product, the heavy-row partial sums and the work counters --
// is carved from one file-scope __device__ array of GRGX_NOALLOC_SCRATCH_BYTES bytes.
//
// When the array takes device memory: CUDA loads a library's device code per device on first
// use (lazy module loading, the default of this CUDA runtime), and the array is reserved when
// the module holding it loads on that device.  That happens when a graph first becomes resident
// on the device (grgx_graph_upload, or the first call that uploads it): the upload resolves the
// array's address there, with the device current.  From then on the device holds the array
// until the process exits.  With CUDA_MODULE_LOADING=EAGER in the environment it is reserved
// on every device when the CUDA context is created instead.  A caller that claims its device
// budget should upload its graphs first.
//
// Rules of use:
//   * The graph must already be resident on the current device (grgx_graph_upload).
//   * Input and output are device pointers; the output is overwritten, not added to.
//   * The array's device address is looked up once per device (cudaGetSymbolAddress, with that
//     device current) by the graph upload; a call on a device where that has not happened yet
//     looks it up itself, so make the first call before any stream capture.
//   * A device reset (cudaDeviceReset) between calls is not supported: the address looked up
//     before it would be stale.
//   * Every call shares the one array and leaves its contents behind; the call clears what must
//     start at zero itself.  Calls whose work overlaps on the GPU (different streams, or
//     different host threads) race on the array: serialise them on one stream.
//   * Products whose scratch would exceed the array are rejected with GRGX_ERR_UNSUPPORTED
//     before anything is launched.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "device_plan.h"
#include "launch.h"

namespace grgx {
namespace {

static __device__ __align__(256) unsigned char g_noalloc_scratch[GRGX_NOALLOC_SCRATCH_BYTES];

constexpr int kMaxDevices = 64;
std::mutex g_scratch_mu;
void* g_scratch_ptr[kMaxDevices] = {};

// Device address of the static scratch on `device` (looked up once per device, with that device
// current -- the host-side symbol is only a stand-in and must never reach a kernel).
void* scratch_address(int device) {
    GRGX_CHECK(device >= 0 && device < kMaxDevices, GRGX_ERR_UNSUPPORTED, "device index out of range");
    std::lock_guard<std::mutex> lk(g_scratch_mu);
    if (g_scratch_ptr[device] == nullptr) {
        void* ptr = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
        GRGX_CHECK(e == cudaSuccess && ptr != nullptr, GRGX_ERR_CUDA,
                   std::string("cudaGetSymbolAddress(g_noalloc_scratch): ") + cudaGetErrorString(e));
        g_scratch_ptr[device] = ptr;
    }
    return g_scratch_ptr[device];
}

// Bump allocation inside the static array (256-byte aligned pieces).
struct Carve {
    unsigned char* base;
    size_t used = 0;
    size_t take_offset(size_t bytes) {
        const size_t off = (used + 255) & ~size_t(255);
        used = off + (bytes ? bytes : 16);
        return off;
    }
    void* take(size_t bytes) { return base + take_offset(bytes); }
};

}  // namespace

// Called with `device` current when a graph becomes resident there: loads this file's module
// on the device, which reserves the static scratch, and caches its address.
void noalloc_prepare_device(int device) { scratch_address(device); }

void matmul_noalloc_impl(grgx_graph* g, int dtype, const void* input, uint64_t in_cols, uint64_t rows, int direction,
                         void* output, uint64_t output_size, void* stream_ptr) {
    const HostGraph& hg = *g->host;
    const uint64_t n = hg.num_nodes, N = hg.num_samples, M = hg.num_mutations;
    GRGX_CHECK(dtype >= GRGX_F64 && dtype <= GRGX_U8, GRGX_ERR_UNSUPPORTED,
               "grgx_matmul_noalloc supports the numeric dtypes (not bool)");
    GRGX_CHECK(direction == GRGX_DIRECTION_DOWN || direction == GRGX_DIRECTION_UP, GRGX_ERR_API_MISUSE,
               "Invalid traversal direction");
    GRGX_CHECK(in_cols > 0 && rows > 0, GRGX_ERR_API_MISUSE, "matmul() requires non-zero dimensions.");
    GRGX_CHECK(output_size % rows == 0, GRGX_ERR_API_MISUSE, "Output size must be divisible by the number of rows");
    const uint64_t out_cols = output_size / rows;
    const bool down = (direction == GRGX_DIRECTION_DOWN);
    if (down) {
        GRGX_CHECK(in_cols == M, GRGX_ERR_API_MISUSE, "Input vector is not size M (numMutations)");
        GRGX_CHECK(out_cols == N, GRGX_ERR_API_MISUSE,
                   "Output vector is not size N (numSamples, or numIndividuals depending on flags)");
    } else {
        GRGX_CHECK(in_cols == N, GRGX_ERR_API_MISUSE,
                   "Input vector is not size N (numSamples, or numIndividuals depending on flags)");
        GRGX_CHECK(out_cols == M, GRGX_ERR_API_MISUSE, "Output vector is not size M (numMutations)");
    }
    GRGX_CHECK(rows <= 2000000ull, GRGX_ERR_UNSUPPORTED, "too many input rows for one call; split the rows");
    int device = 0;
    GRGX_CUDA(cudaGetDevice(&device));
    const DevicePlan* dp = nullptr;
    {
        std::lock_guard<std::mutex> lk(g->mu);  // the upload writes g->dev under this lock
        dp = g->dev.get();
    }
    GRGX_CHECK(dp != nullptr && dp->device == device, GRGX_ERR_UNSUPPORTED,
               "grgx_matmul_noalloc needs the graph resident on the current device: call grgx_graph_upload first");

    const long long K = static_cast<long long>(rows);
    const Layout L = choose_layout(dtype, K, /*plainF32=*/false, /*nativeF64=*/true);
    const DevCSR& sweep = down ? dp->down : dp->up;
    const long long pieces = down ? std::max(dp->down.n_pieces, dp->seed.n_pieces) : dp->up.n_pieces;
    const long long nh = down ? (dp->down.n_heavy + dp->seed.n_heavy) : dp->up.n_heavy;
    const long long nslots = down ? 1 + static_cast<long long>(dp->down.lb.size()) : static_cast<long long>(dp->up.lb.size());
    const size_t valBytes = static_cast<size_t>(n) * L.stride * L.ssize;
    const size_t vtBytes = (down && dp->seed.n_edges > 0) ? static_cast<size_t>(M) * L.stride * L.ssize : 0;
    const size_t partBytes = static_cast<size_t>(pieces) * L.stride * L.asize;
    const size_t counterBytes = static_cast<size_t>(nh + nslots) * L.ntiles * sizeof(unsigned);

    // Size check before anything is launched.
    Carve plan{nullptr};
    plan.take_offset(valBytes);
    if (vtBytes) plan.take_offset(vtBytes);
    plan.take_offset(partBytes);
    plan.take_offset(counterBytes);
    GRGX_CHECK(plan.used <= GRGX_NOALLOC_SCRATCH_BYTES, GRGX_ERR_UNSUPPORTED,
               "grgx_matmul_noalloc: this product needs " + std::to_string(plan.used) +
                   " bytes of scratch, more than its static scratch of " +
                   std::to_string(static_cast<unsigned long long>(GRGX_NOALLOC_SCRATCH_BYTES)) +
                   " bytes; use grgx_matmul or fewer rows");

    Carve c{static_cast<unsigned char*>(scratch_address(device))};
    void* vals = c.take(valBytes);
    void* vt = vtBytes ? c.take(vtBytes) : nullptr;
    void* partials = c.take(partBytes);
    unsigned* tickets = static_cast<unsigned*>(c.take(counterBytes));
    unsigned* work = tickets + nh * L.ntiles;

    cudaStream_t s = static_cast<cudaStream_t>(stream_ptr);
    // What must start at zero: the node values (zero init) and every counter.
    GRGX_CUDA(cudaMemsetAsync(vals, 0, valBytes, s));
    GRGX_CUDA(cudaMemsetAsync(tickets, 0, counterBytes, s));
    if (down) {
        unsigned* tk = tickets;
        if (vt) {
            launch_load_rows(dtype, input, K, static_cast<long long>(in_cols), static_cast<long long>(M), MAP_IDENT,
                             1, nullptr, vt, L.stride, 0, s);
            launch_level(L, dp->seed, 0, vt, vals, 0, partials, tk, work, s);
        }
        tk += dp->seed.n_heavy * L.ntiles;
        for (size_t lvl = 0; lvl < sweep.lb.size(); lvl++)
            launch_level(L, sweep, lvl, vals, vals, 1, partials, tk, work + (1 + lvl) * L.ntiles, s);
        launch_store_cols(dtype, vals, L.stride, K, static_cast<long long>(N), MAP_IDENT, 1, nullptr, output,
                          static_cast<long long>(out_cols), 0, s);
    } else {
        launch_load_rows(dtype, input, K, static_cast<long long>(in_cols), static_cast<long long>(N), MAP_IDENT, 1,
                         nullptr, vals, L.stride, 0, s);
        for (size_t lvl = 0; lvl < sweep.lb.size(); lvl++)
            launch_level(L, sweep, lvl, vals, vals, 0, partials, tickets, work + lvl * L.ntiles, s);
        launch_store_cols(dtype, vals, L.stride, K, static_cast<long long>(M), MAP_TABLE, 1, dp->mut_new, output,
                          static_cast<long long>(out_cols), 0, s);
    }
    GRGX_CUDA(cudaGetLastError());
}

}  // namespace grgx
