// Device-resident plan and launch helpers shared by the matmul entry points (internal).
#pragma once
#include <cuda_runtime.h>

#include <map>
#include <string>
#include <vector>

#include "grgx_internal.h"
#include "launch.h"

namespace grgx {

#define GRGX_CUDA(call)                                                                               \
    do {                                                                                             \
        cudaError_t err__ = (call);                                                                  \
        if (err__ != cudaSuccess) {                                                                  \
            const int code__ = (err__ == cudaErrorMemoryAllocation) ? GRGX_ERR_OUT_OF_MEMORY         \
                                                                    : GRGX_ERR_CUDA;                 \
            throw ::grgx::Error(code__, std::string(#call) + ": " + cudaGetErrorString(err__));       \
        }                                                                                            \
    } while (0)

struct DevCSR {
    uint32_t* adj = nullptr;  // 32-bit ids, or 16-bit block-relative ids when id16
    bool id16 = false;
    // id16: per level (= split block), the block's first source id and its number of source ids
    std::vector<long long> level_base, level_src_rows;
    int* rows = nullptr;
    ChunkDev* chunks = nullptr;
    HeavyDev* heavy = nullptr;
    std::vector<int32_t> lb, le;
    std::vector<long long> level_rows, level_edges;  // per level, for the launch-shape table
    long long n_heavy = 0, n_pieces = 0, n_edges = 0, n_rows = 0;
};

struct DevicePlan {
    int device = -1;
    DevCSR up, down, seed, miss;
    // up / down (and below up0b, up_int, down0b) on the fine chunking: the same adjacency and
    // rows, kFineChunkFactor times the chunks per level (sweep_csrs picks them for wide rows)
    DevCSR up_f, down_f;
    // UP in split form (empty when the height-0 nodes make fewer than two blocks):
    //   up0b    the edges to height-0 children, cut by blocks of `split_block` height-0 ids;
    //           level j = block j, rows = every node with children in the block
    //   up_int  the edges to children of height >= 1, one level per UP level (same order)
    //   fin     per UP level, the nodes without such children (finished from their state alone),
    //           concatenated; fin_begin[j] .. fin_begin[j+1] for level j
    // Built on the first call that runs UP in split form (use_up_split), from the UP row offsets
    // and level boundaries kept here.
    DevCSR up0b, up_int, up0b_f, up_int_f;
    int* fin = nullptr;
    std::vector<long long> fin_begin;
    long long split_block = 0, split_src = 0;  // split_src = height-0 ids = first UP row's node id
    bool split_built = false;
    std::map<std::pair<int, long long>, bool> split_choice;  // (storage kind, stride) -> measured choice
    // DOWN in split form (empty when the parents of height-0 rows make fewer than two blocks):
    //   down0b  the edges of the height-0 DOWN rows, cut by blocks of `split_block` parent ids
    //           starting at split_src (parents all have height >= 1); level j = block j, rows =
    //           every height-0 row with parents in the block; 16-bit block-relative ids
    //   fin_down the height-0 DOWN rows, finished from their state after the block passes
    // Built on the first call that runs DOWN in split form (use_down_split).
    DevCSR down0b, down0b_f;
    int* fin_down = nullptr;
    long long n_fin_down = 0;
    bool down_split_built = false;
    std::map<std::pair<int, long long>, bool> down_split_choice;
    std::vector<int64_t> down_off;       // DOWN row offsets (host copy)
    long long down_h0_row = 0;           // first DOWN row of height 0
    std::vector<int64_t> up_off;         // UP row offsets (host copy)
    std::vector<uint64_t> level_begin;   // node-id range of each height
    uint32_t* mut_new = nullptr;
    uint32_t* miss_new = nullptr;
    uint32_t* old2new = nullptr;
    uint32_t* new2old = nullptr;
    uint32_t* xtx_new = nullptr;
    uint64_t bytes = 0;
    uint64_t num_levels = 0;
    bool has_coals = false;
    bool has_miss = false;
    double xtx_max = 0.0;  // largest XTX init value (2 * coalescences)
    double* freq = nullptr;       // allele frequency per mutation (standardized products)
    double* inv_sigma = nullptr;  // 1/sqrt(p(1-p)) per mutation, 0 where p(1-p) == 0
    std::vector<void*> allocs;
};

struct Layout {
    Kind kind;
    int ssize;     // storage bytes per element
    int asize;     // accumulator bytes per element (heavy partials)
    long long stride;
    int vw, g, ntiles;
};

// Element layout of one call: storage kind, row stride and the default (VW, G) sweep shape.
Layout choose_layout(int dtype, long long K, bool plainF32, bool nativeF64);

// Launch shape of one level: G lanes per row, the column tiles that G leaves (the K-tile
// count), and the prefetch-depth variant (0 default, 1 deep).
struct LevelShape {
    int g = 1;
    int ntiles = 1;
    int variant = 0;
};
LevelShape default_shape(const Layout& L);
// The shape a level runs with: the autotuner's entry for (storage kind, row stride, the level's
// width and mean degree) when there is one, else the default.
LevelShape level_shape(const Layout& L, const DevCSR& c, size_t level);
// Column tiles of the widest shape the autotuner may pick for L: the stride of the per-launch
// work counters and of the heavy-row tickets.
int max_tiles(const Layout& L);

// The sweep CSRs a call with layout L runs on: rows of 32 bytes or more (K >= 8 four-byte or
// K >= 4 eight-byte values) take the fine chunking, narrower rows -- whose chunks cost little
// each, so that more of them only adds per-chunk work (the staged single-column passes lose
// 10-20%) -- the coarse one.  The split copies' members are empty until they are built.
struct SweepCSRs {
    const DevCSR* up;
    const DevCSR* down;
    const DevCSR* up0b;
    const DevCSR* up_int;
    const DevCSR* down0b;
};
bool fine_chunks(const Layout& L);
SweepCSRs sweep_csrs(const DevicePlan* dp, const Layout& L);
// `coarse` with the chunks, heavy rows and level ranges of `fine` (uploaded; the adjacency and
// rows are shared).
DevCSR fine_view(DevicePlan& d, const DevCSR& coarse, const PullCSR& fine);

// Launches one level of a CSR (a no-op when the level has no chunks); `work` points at
// `tileStride` (0: L.ntiles) zeroed counters owned by this launch, and the heavy-row tickets
// are `tileStride` apart.  `shape` null: the default shape.  Returns the kernels launched.
// `state` set: each node's Op::A accumulator lives at state + (node - stateBase) rows; with
// stateMode 1 a row's sum is merged into it (nothing written), with 2 the node value is written
// from the accumulator merged with the row's sum.
int launch_level(const Layout& L, const DevCSR& c, size_t level, const void* src, void* dst, int rmw,
                 void* partials, unsigned* tickets, unsigned* work, cudaStream_t s, const int* gate = nullptr,
                 int gateValue = 0, const LevelShape* shape = nullptr, int tileStride = 0, void* state = nullptr,
                 long long stateBase = 0, int stateMode = 1);

// UP in split form (up_split.cu): writes vals[node] from its accumulator state (added onto the
// value when rmw) for the `count` nodes listed at `nodes`.
void launch_state_finish(Kind kind, const void* state, void* vals, const int* nodes, long long count,
                         long long stateBase, long long stride, int rmw, cudaStream_t s, const int* gate,
                         int gateValue);
// Height-0 row bytes (height-0 ids x stride x element size) above which UP runs in split form,
// and the block of height-0 ids each split pass covers; both adjustable for tests.
uint64_t split_threshold_bytes();
long long split_block_size();
// Whether a call with layout L runs UP in split form: the choice grgx_autotune measured for
// (storage kind, stride) on this graph, else whether the height-0 rows exceed the threshold.
// Builds the split copy on first use.
bool use_up_split(grgx_graph* g, DevicePlan* dp, const Layout& L);
bool up_split_possible(const DevicePlan* dp);
void ensure_up_split(grgx_graph* g, DevicePlan* dp);
void set_up_split_choice(grgx_graph* g, DevicePlan* dp, const Layout& L, bool split);
// The same for DOWN: the height-0 level in parent blocks.  Without a measured choice a call runs
// DOWN in split form when its block passes run staged (staged_layout); UP likewise, or when the
// height-0 rows exceed the threshold.
bool use_down_split(grgx_graph* g, DevicePlan* dp, const Layout& L);
bool down_split_possible(const DevicePlan* dp);
void ensure_down_split(grgx_graph* g, DevicePlan* dp);
void set_down_split_choice(grgx_graph* g, DevicePlan* dp, const Layout& L, bool split);
// Whether single-column 4-byte split passes stage their block's source values in shared memory
// (sweep_kernel_staged); on by default, switchable for tests.
bool staged_enabled();
void set_staged(bool on);
// Whether split block passes of layout L run staged: a single 4-byte column (K = 1 for the
// 4-byte dtypes, bool up to 32 columns), staging on.
bool staged_layout(const Layout& L);
// DOWN split form: 0 chosen as above, 1 always (where possible), 2 never (tests).
void set_down_split_mode(int mode);

// Resolves (once per device, with `device` current) the address of grgx_matmul_noalloc's
// static scratch, which loads its module and so reserves the array on the device.
void noalloc_prepare_device(int device);

// Builds (once) and returns the graph's plan on the current device.
DevicePlan* ensure_device_plan(grgx_graph* g);

// The library's own stream-ordered memory pool on `device` (created on first use).
cudaMemPool_t library_pool(int device);
// Bytes of the library pool on `device` handed out to calls now, and held by the pool.
void pool_usage(int device, uint64_t* used, uint64_t* reserved);

// Stream-ordered allocation from the library's pool on the current device.  The pool never makes a call wait for
// a call on another stream, so under memory pressure the blocks such calls have freed can still
// be in flight: then the device is drained once and the allocation retried (not inside a stream
// capture, where the first error stands).
cudaError_t pool_malloc(void** p, size_t bytes, cudaStream_t s);
// Hands the memory the pool keeps cached between calls back to the device (after an ordinary
// allocation ran out of memory).
void trim_pool();

}  // namespace grgx
