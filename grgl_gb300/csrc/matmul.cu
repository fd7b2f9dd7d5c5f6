// Device plan upload and the matmul orchestration behind grgx_matmul.
//
// One call is, on one stream:
//   init      memset / VECTOR / MATRIX / XTX fill of the node values   (grg.h:1370-1402)
//   seed      UP: samples <- input columns (transposing load)          (grg.h:1458-1469)
//             DOWN: input -> per-mutation rows, then one gather-sum pass over the
//             node -> mutations CSR (and the missingness CSR)          (grg.h:1405-1427)
//   sweep     one launch per level, pull form, no atomics on values   (grg.h:1428-1431, 1470-1474)
//   gather    node rows -> output columns (transposing store)          (grg.h:1440-1453, 1483-1516)
// Scratch (node values, transposed inputs, heavy-row partials) comes from the device's
// stream-ordered memory pool and is released on the same stream.
#include <cuda_runtime.h>

#include <atomic>
#include <cstring>
#include <map>
#include <sstream>
#include <thread>

#include "grgx_internal.h"
#include "device_plan.h"
#include "launch.h"

namespace grgx {


void destroy_device_plan(DevicePlan* p) {
    if (!p) return;
    int cur = -1;
    cudaGetDevice(&cur);
    cudaSetDevice(p->device);
    for (void* a : p->allocs) cudaFree(a);
    if (cur >= 0) cudaSetDevice(cur);
    delete p;
}

namespace {

static_assert(sizeof(Chunk) == sizeof(ChunkDev), "chunk layout");
static_assert(sizeof(HeavyRow) == sizeof(HeavyDev), "heavy layout");

template <typename T> T* upload(DevicePlan& d, const std::vector<T>& v) {
    if (v.empty()) return nullptr;
    void* p = nullptr;
    GRGX_CUDA(cudaMalloc(&p, v.size() * sizeof(T)));
    d.allocs.push_back(p);
    d.bytes += v.size() * sizeof(T);
    GRGX_CUDA(cudaMemcpy(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice));
    return static_cast<T*>(p);
}

DevCSR upload_csr(DevicePlan& d, const PullCSR& c) {
    DevCSR r;
    r.adj = upload(d, c.adj);  // null when the adjacency is built on the device
    r.rows = upload(d, c.rows);
    r.chunks = reinterpret_cast<ChunkDev*>(upload(d, c.chunks));
    r.heavy = reinterpret_cast<HeavyDev*>(upload(d, c.heavy));
    r.lb = c.level_chunk_begin;
    r.le = c.level_chunk_end;
    r.n_heavy = static_cast<long long>(c.heavy.size());
    r.n_pieces = c.num_pieces;
    r.n_edges = c.num_edges;
    r.n_rows = static_cast<long long>(c.rows.size());
    for (size_t l = 0; l < c.level_chunk_begin.size(); l++) {
        const Chunk& a = c.chunks[static_cast<size_t>(c.level_chunk_begin[l])];
        const Chunk& b = c.chunks[static_cast<size_t>(c.level_chunk_end[l])];
        r.level_rows.push_back(static_cast<long long>(b.r0) - a.r0);
        r.level_edges.push_back(static_cast<long long>(b.e0 - a.e0));
    }
    return r;
}

}  // namespace

DevCSR fine_view(DevicePlan& d, const DevCSR& coarse, const PullCSR& fine) {
    DevCSR r = coarse;
    r.chunks = reinterpret_cast<ChunkDev*>(upload(d, fine.chunks));
    r.heavy = reinterpret_cast<HeavyDev*>(upload(d, fine.heavy));
    r.lb = fine.level_chunk_begin;
    r.le = fine.level_chunk_end;
    r.n_heavy = static_cast<long long>(fine.heavy.size());
    r.n_pieces = fine.num_pieces;
    return r;
}

bool fine_chunks(const Layout& L) { return L.stride * L.ssize >= 32; }

SweepCSRs sweep_csrs(const DevicePlan* dp, const Layout& L) {
    if (fine_chunks(L)) return SweepCSRs{&dp->up_f, &dp->down_f, &dp->up0b_f, &dp->up_int_f, &dp->down0b_f};
    return SweepCSRs{&dp->up, &dp->down, &dp->up0b, &dp->up_int, &dp->down0b};
}

// The library's own stream-ordered pool on `device` (created once per device; the process's
// default pool, which the host application may use too, is left as it is).  Memory freed into it
// stays cached for the next call (release threshold: never).  Calls on different streams are not
// chained through it: a block freed by a call still running on one stream is not handed to
// another stream's call (which would make it wait for the first); only blocks whose free has
// completed are.
cudaMemPool_t library_pool(int device) {
    constexpr int kMaxDev = 64;
    static std::mutex mu;
    static cudaMemPool_t pools[kMaxDev] = {};
    GRGX_CHECK(device >= 0 && device < kMaxDev, GRGX_ERR_UNSUPPORTED, "device index out of range");
    std::lock_guard<std::mutex> lk(mu);
    if (pools[device] != nullptr) return pools[device];
    cudaMemPoolProps props{};
    props.allocType = cudaMemAllocationTypePinned;
    props.handleTypes = cudaMemHandleTypeNone;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = device;
    cudaMemPool_t pool = nullptr;
    GRGX_CUDA(cudaMemPoolCreate(&pool, &props));
    uint64_t threshold = UINT64_MAX;
    GRGX_CUDA(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &threshold));
    int noChain = 0;
    GRGX_CUDA(cudaMemPoolSetAttribute(pool, cudaMemPoolReuseAllowInternalDependencies, &noChain));
    pools[device] = pool;
    return pool;
}

long long next_pow2(long long x) {
    long long p = 1;
    while (p < x) p <<= 1;
    return p;
}

Layout choose_layout(int dtype, long long K, bool plainF32, bool nativeF64) {
    Layout L{};
    long long base = K;
    switch (dtype) {
    case GRGX_F64: L.kind = nativeF64 ? Kind::F64 : Kind::F64S; L.ssize = 8; break;
    case GRGX_F32: L.kind = plainF32 ? Kind::F32 : Kind::F32C; L.ssize = 4; break;
    case GRGX_I64: case GRGX_U64: L.kind = Kind::U64; L.ssize = 8; break;
    case GRGX_BOOL: L.kind = Kind::XOR; L.ssize = 4; base = (K + 31) / 32; break;
    default: L.kind = Kind::U32; L.ssize = 4; break;
    }
    L.asize = (L.kind == Kind::F32C || L.kind == Kind::F64S) ? static_cast<int>(L.kind == Kind::F32C ? sizeof(F32Pair)
                                                                                               : sizeof(F64Run))
                                                              : L.ssize;
    const int maxVw = 16 / L.ssize;
    if (base == 1) {
        L.stride = 1; L.vw = 1; L.g = 1; L.ntiles = 1;
    } else if (base == 2 && maxVw == 4) {
        L.stride = 2; L.vw = 2; L.g = 1; L.ntiles = 1;
    } else {
        L.vw = maxVw;
        L.stride = (base + maxVw - 1) / maxVw * maxVw;
        const long long vecs = L.stride / L.vw;
        L.g = static_cast<int>(std::min<long long>(32, next_pow2(vecs)));
        L.ntiles = static_cast<int>((vecs + L.g - 1) / L.g);
    }
    return L;
}

namespace {

struct Scratch {
    cudaStream_t s;
    std::vector<void*> ptrs;
    explicit Scratch(cudaStream_t st) : s(st) {}
    void* get(size_t bytes) {
        if (bytes == 0) bytes = 16;
        void* p = nullptr;
        GRGX_CUDA(pool_malloc(&p, bytes, s));
        ptrs.push_back(p);
        return p;
    }
    ~Scratch() {
        for (void* p : ptrs) cudaFreeAsync(p, s);
    }
};

thread_local int t_timing = 0;  // 0 off, 1 per call (synchronises), 2 deferred
thread_local grgx_timing t_last{};
// Deferred timing: each call's events, read back by collect_timings after the caller syncs.
struct PendingTiming {
    cudaEvent_t ev[4];
    uint64_t launches, alg_bytes;
};
thread_local std::vector<PendingTiming> t_pending;

}  // namespace

// SM count of the current device (looked up once per device).
int sm_count() {
    constexpr int kMaxDev = 64;
    static std::atomic<int> cache[kMaxDev];
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= kMaxDev) dev = 0;
    int sms = cache[dev].load(std::memory_order_relaxed);
    if (sms == 0) {
        int v = 0;
        cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
        sms = v > 0 ? v : 1;
        cache[dev].store(sms, std::memory_order_relaxed);
    }
    return sms;
}

template <typename S>
SweepParams<S> make_params(const DevCSR& c, long long cb, long long ce, const void* src, void* dst, long long stride,
                           int rmw, void* partials, unsigned* tickets, unsigned* work, int ntiles) {
    SweepParams<S> p;
    p.adj = c.adj;
    p.rows = c.rows;
    p.chunks = c.chunks;
    p.heavy = c.heavy;
    p.c_begin = cb;
    p.c_end = ce;
    p.src = static_cast<const S*>(src);
    p.dst = static_cast<S*>(dst);
    p.stride = stride;
    p.rmw = rmw;
    p.partials = partials;
    p.tickets = tickets;
    p.work = work;
    p.ntiles = ntiles;
    p.gate = nullptr;
    p.gate_value = 0;
    p.state = nullptr;
    p.state_base = 0;
    p.state_mode = 0;
    p.id16 = 0;
    p.id_base = 0;
    p.src_rows = 0;
    p.col_base = 0;
    return p;
}

// Launches one level of a CSR; returns the number of kernels launched (0, 1, or 2 when a nearly
// empty last column tile runs on its own).  `work` points at `tileStride` zeroed counters owned
// by this level.
int launch_level(const Layout& L, const DevCSR& c, size_t level, const void* src, void* dst, int rmw,
                 void* partials, unsigned* tickets, unsigned* work, cudaStream_t s, const int* gate,
                 int gateValue, const LevelShape* shape, int tileStride, void* state, long long stateBase,
                 int stateMode) {
    const long long cb = c.lb[level], ce = c.le[level];
    if (ce <= cb) return 0;
    const LevelShape sh = shape ? *shape : default_shape(L);
    const int ts = tileStride > 0 ? tileStride : L.ntiles;
    if (sh.ntiles > ts) throw Error(GRGX_ERR_CUDA, "launch shape has more column tiles than counters");
    const int sms = sm_count();
    const long long base = c.id16 ? c.level_base[level] : 0;
    // One launch of `tiles` column tiles of g lanes from column colBase; its work counters and
    // heavy-row tickets are those of tile slot `slot` onwards.
    auto launch = [&](int g, int tiles, int variant, int colBase, int slot) {
        const dim3 grid(static_cast<unsigned>((ce - cb + 7) / 8), static_cast<unsigned>(tiles));
        auto prm = [&](auto tag) {
            using S = decltype(tag);
            SweepParams<S> p = make_params<S>(c, cb, ce, src, dst, L.stride, rmw, partials, tickets + slot,
                                              work + slot, ts);
            p.gate = gate;
            p.gate_value = gateValue;
            p.state = state;
            p.state_base = stateBase;
            p.state_mode = stateMode;
            p.col_base = colBase;
            // a split block: 16-bit ids relative to the block's first source id
            p.id16 = c.id16 ? 1 : 0;
            p.id_base = base;
            return p;
        };
        const int vw = L.vw;
        switch (L.kind) {
        case Kind::U32: launch_sweep_u32(prm(uint32_t{}), vw, g, variant, grid, sms, s); break;
        case Kind::XOR: launch_sweep_xor(prm(uint32_t{}), vw, g, variant, grid, sms, s); break;
        case Kind::U64: launch_sweep_u64(prm(static_cast<unsigned long long>(0)), vw, g, variant, grid, sms, s); break;
        case Kind::F64: launch_sweep_f64(prm(double{}), vw, g, variant, grid, sms, s); break;
        case Kind::F32C: launch_sweep_f32c(prm(float{}), vw, g, variant, grid, sms, s); break;
        case Kind::F32: launch_sweep_f32(prm(float{}), vw, g, variant, grid, sms, s); break;
        case Kind::F64S: launch_sweep_f64s(prm(DF{}), vw, g, variant, grid, sms, s); break;
        }
    };
    if (c.id16) {
        // single-column 4-byte rows stage the block's sources in shared memory (one 1024-thread
        // block per SM)
        const long long srows = c.level_src_rows[level];
        if (staged_layout(L) && srows <= kStagedRows && sh.ntiles == 1) {
            const dim3 sgrid(static_cast<unsigned>(std::min<long long>((ce - cb + 7) / 8, sms)), 1);
            auto sp = [&](auto tag) {
                using S = decltype(tag);
                SweepParams<S> p = make_params<S>(c, cb, ce, src, dst, L.stride, rmw, partials, tickets, work, ts);
                p.gate = gate;
                p.gate_value = gateValue;
                p.state = state;
                p.state_base = stateBase;
                p.state_mode = stateMode;
                p.id16 = 1;
                p.id_base = 0;
                p.src = static_cast<const S*>(src) + base;
                p.src_rows = srows;
                return p;
            };
            switch (L.kind) {
            case Kind::U32: launch_sweep_staged_u32(sp(uint32_t{}), sgrid, s); break;
            case Kind::XOR: launch_sweep_staged_xor(sp(uint32_t{}), sgrid, s); break;
            case Kind::F32C: launch_sweep_staged_f32c(sp(float{}), sgrid, s); break;
            case Kind::F32: launch_sweep_staged_f32(sp(float{}), sgrid, s); break;
            default: break;
            }
            return 1;
        }
    }
    // A last column tile under a quarter full costs nearly a full pass at g lanes per row (its
    // warps gather one or two edges per sub-step): it runs as a launch of its own with as few
    // lanes per row as its columns need.
    const long long vecs = (L.stride + L.vw - 1) / L.vw;
    const long long full = vecs / sh.g, rem = vecs % sh.g;
    if (full >= 1 && rem > 0 && rem * 4 <= sh.g && full + 1 <= ts && full + 1 == sh.ntiles) {
        const int gr = static_cast<int>(next_pow2(rem));
        launch(sh.g, static_cast<int>(full), sh.variant, 0, 0);
        launch(gr, 1, 0, static_cast<int>(full * sh.g * L.vw), static_cast<int>(full));
        return 2;
    }
    launch(sh.g, sh.ntiles, sh.variant, 0, 0);
    return 1;
}

namespace {

size_t io_size(int dtype) {
    switch (dtype) {
    case GRGX_F64: case GRGX_I64: case GRGX_U64: return 8;
    case GRGX_F32: case GRGX_I32: case GRGX_U32: return 4;
    case GRGX_I16: case GRGX_U16: return 2;
    default: return 1;
    }
}

}  // namespace

uint32_t* build_down_adj_device(const uint32_t* upAdj, const int* upRows, const ChunkDev* upChunks, long long upChunkCount,
                                long long E, const std::vector<int32_t>& rowOf, const std::vector<int64_t>& downOff);

uint32_t* build_plan_device(const HostGraph& g, const unsigned long long* dOff, const uint32_t* dAdj, uint64_t E,
                            HostPlan& plan);

void decode_edges_device(const HostGraph& hg, void** dOff, void** dAdj);

namespace {
// The E-sized passes of the plan on the device (plan_device.cu) from the down CSR, uploaded
// from the host or decoded on the device from an encoded graph's vbyte buckets; returns the
// device UP adjacency (null: use the host builder).
uint32_t* device_plan_build(const HostGraph& hg, std::unique_ptr<HostPlan>& out) {
    const uint64_t n = hg.num_nodes, E = hg.num_edges();
    void *dOff = nullptr, *dAdj = nullptr;
    auto freeAll = [&] {
        if (dOff) cudaFree(dOff);
        if (dAdj) cudaFree(dAdj);
    };
    auto hp = std::make_unique<HostPlan>();
    uint32_t* up = nullptr;
    try {
        if (hg.encoded()) {
            decode_edges_device(hg, &dOff, &dAdj);
        } else {
            GRGX_CUDA(cudaMalloc(&dOff, (n + 1) * sizeof(uint64_t)));
            GRGX_CUDA(cudaMalloc(&dAdj, (E ? E : 1) * sizeof(uint32_t)));
            GRGX_CUDA(cudaMemcpy(dOff, hg.down_off.data(), (n + 1) * sizeof(uint64_t), cudaMemcpyHostToDevice));
            if (E) GRGX_CUDA(cudaMemcpy(dAdj, hg.down_adj.data(), E * sizeof(uint32_t), cudaMemcpyHostToDevice));
        }
        up = build_plan_device(hg, static_cast<const unsigned long long*>(dOff), static_cast<const uint32_t*>(dAdj), E,
                               *hp);
    } catch (...) {
        freeAll();
        throw;
    }
    freeAll();
    if (up) out = std::move(hp);
    return up;
}
}  // namespace

cudaError_t pool_malloc(void** p, size_t bytes, cudaStream_t s) {
    int device = 0;
    cudaError_t e = cudaGetDevice(&device);
    if (e != cudaSuccess) return e;
    const cudaMemPool_t pool = library_pool(device);
    e = cudaMallocFromPoolAsync(p, bytes, pool, s);
    if (e != cudaErrorMemoryAllocation) return e;
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(s, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone) return e;
    cudaGetLastError();
    // let pending frees complete, then try once more (the synchronisation itself may be refused
    // while another thread captures a CUDA graph: the retry then sees what has completed)
    cudaDeviceSynchronize();
    cudaGetLastError();
    return cudaMallocFromPoolAsync(p, bytes, pool, s);
}

void trim_pool() {
    int device = 0;
    if (cudaGetDevice(&device) != cudaSuccess) return;
    const cudaMemPool_t pool = library_pool(device);
    cudaDeviceSynchronize();
    cudaMemPoolTrimTo(pool, 0);
    cudaGetLastError();
}

void pool_usage(int device, uint64_t* used, uint64_t* reserved) {
    const cudaMemPool_t pool = library_pool(device);
    uint64_t u = 0, r = 0;  // the pool attributes are 64-bit values
    GRGX_CUDA(cudaMemPoolGetAttribute(pool, cudaMemPoolAttrUsedMemCurrent, &u));
    GRGX_CUDA(cudaMemPoolGetAttribute(pool, cudaMemPoolAttrReservedMemCurrent, &r));
    if (used) *used = static_cast<uint64_t>(u);
    if (reserved) *reserved = static_cast<uint64_t>(r);
}

namespace {
DevicePlan* ensure_device_plan_once(grgx_graph* g) {
    std::lock_guard<std::mutex> lk(g->mu);
    int device = 0;
    GRGX_CUDA(cudaGetDevice(&device));
    if (g->dev) {
        GRGX_CHECK(g->dev->device == device, GRGX_ERR_UNSUPPORTED,
                   "graph is resident on device " + std::to_string(g->dev->device));
        return g->dev.get();
    }
    library_pool(device);
    noalloc_prepare_device(device);
    const PlanDeviceScope planSms(sm_count());
    uint32_t* upAdjDev = nullptr;
    if (!g->plan && !g->host_plan && g->host->num_nodes > 0) upAdjDev = device_plan_build(*g->host, g->plan);
    if (!g->plan) g->plan = build_plan(g->host_edges());
    const HostPlan& hp = *g->plan;
    std::unique_ptr<DevicePlan, DevicePlanDeleter> d(new DevicePlan());
    d->device = device;
    if (upAdjDev) {
        d->allocs.push_back(upAdjDev);
        d->bytes += static_cast<uint64_t>(hp.up.off.empty() ? 0 : hp.up.off.back()) * sizeof(uint32_t);
    }
    d->up = upload_csr(*d, hp.up);
    if (upAdjDev) d->up.adj = upAdjDev;
    d->down = upload_csr(*d, hp.down);
    d->down.adj = build_down_adj_device(d->up.adj, d->up.rows, d->up.chunks,
                                        static_cast<long long>(hp.up.chunks.size()) - 1, hp.down.num_edges,
                                        hp.down_row_of, hp.down.off);
    if (d->down.adj) {
        d->allocs.push_back(d->down.adj);
        d->bytes += static_cast<uint64_t>(hp.down.num_edges) * sizeof(uint32_t);
    }
    d->up_f = fine_view(*d, d->up, hp.up_fine);
    d->down_f = fine_view(*d, d->down, hp.down_fine);
    d->seed = upload_csr(*d, hp.seed);
    d->miss = upload_csr(*d, hp.miss);
    d->mut_new = upload(*d, hp.mut_new);
    d->miss_new = upload(*d, hp.miss_new);
    d->old2new = upload(*d, hp.old2new);
    d->new2old = upload(*d, hp.new2old);
    d->xtx_new = upload(*d, hp.xtx_new);
    d->num_levels = hp.num_levels;
    d->has_coals = hp.has_coals;
    d->has_miss = hp.has_miss;
    for (uint32_t x : hp.xtx_new)
        if (x != COAL_NOT_SET) d->xtx_max = std::max(d->xtx_max, static_cast<double>(x));
    d->up_off = hp.up.off;
    d->down_off = hp.down.off;
    if (!hp.down.level_chunk_begin.empty())
        d->down_h0_row = hp.down.chunks[static_cast<size_t>(hp.down.level_chunk_begin.back())].r0;
    d->level_begin = hp.level_begin;
    g->dev = std::move(d);
    g->plan.reset();  // the device copy is authoritative; free the host copy
    return g->dev.get();
}
}  // namespace

DevicePlan* ensure_device_plan(grgx_graph* g) {
    try {
        return ensure_device_plan_once(g);
    } catch (const Error& e) {
        if (e.code != GRGX_ERR_OUT_OF_MEMORY) throw;
    }
    // out of device memory: hand the memory the pool keeps between calls back to the device
    // and build the plan once more from the start
    {
        std::lock_guard<std::mutex> lk(g->mu);
        g->plan.reset();
    }
    trim_pool();
    return ensure_device_plan_once(g);
}

uint64_t device_plan_bytes(const grgx_graph* g) { return g->dev ? g->dev->bytes : 0; }
uint64_t device_plan_levels(const grgx_graph* g) { return g->dev ? g->dev->num_levels : 0; }

// Argument checks of validateMatMulInputs (internal_mult.h:130-158) and of the binding, with the
// reference's messages; host-only, so misuse is reported before any device work.
void validate_matmul(grgx_graph* g, int dtype, uint64_t in_cols, uint64_t rows, int direction, uint64_t output_size,
                     int emit_all, int by_indiv, const void* init, int init_kind, void* miss) {
    const HostGraph& hg = *g->host;
    const uint64_t n = hg.num_nodes, N = hg.num_samples, M = hg.num_mutations, P = hg.ploidy;
    GRGX_CHECK(dtype >= GRGX_F64 && dtype <= GRGX_BOOL, GRGX_ERR_API_MISUSE, "Unsupported dtype");
    GRGX_CHECK(direction == GRGX_DIRECTION_DOWN || direction == GRGX_DIRECTION_UP, GRGX_ERR_API_MISUSE,
               "Invalid traversal direction");
    GRGX_CHECK(in_cols > 0 && rows > 0, GRGX_ERR_API_MISUSE, "matmul() requires non-zero dimensions.");
    GRGX_CHECK(output_size % rows == 0, GRGX_ERR_API_MISUSE, "Output size must be divisible by the number of rows");
    const uint64_t out_cols = output_size / rows;
    GRGX_CHECK(!by_indiv || N % P == 0, GRGX_ERR_API_MISUSE,
               "by_individual needs the number of samples to be a multiple of the ploidy");
    GRGX_CHECK(rows <= (dtype == GRGX_BOOL ? 65535ull : 2000000ull), GRGX_ERR_UNSUPPORTED,
               "too many input rows for one call; split the rows");
    const uint64_t expectSampleCols = by_indiv ? N / P : N;
    if (direction == GRGX_DIRECTION_DOWN) {
        GRGX_CHECK(in_cols == M, GRGX_ERR_API_MISUSE, "Input vector is not size M (numMutations)");
        GRGX_CHECK(emit_all || out_cols == expectSampleCols, GRGX_ERR_API_MISUSE,
                   "Output vector is not size N (numSamples, or numIndividuals depending on flags)");
    } else {
        GRGX_CHECK(in_cols == expectSampleCols, GRGX_ERR_API_MISUSE,
                   "Input vector is not size N (numSamples, or numIndividuals depending on flags)");
        GRGX_CHECK(emit_all || out_cols == M, GRGX_ERR_API_MISUSE, "Output vector is not size M (numMutations)");
    }
    GRGX_CHECK(!emit_all || out_cols == n, GRGX_ERR_API_MISUSE, "Output vector is not size numNodes");
    GRGX_CHECK(init_kind == GRGX_INIT_ZERO || dtype != GRGX_BOOL, GRGX_ERR_API_MISUSE,
               "Node initialization and bit vector type cannot be mixed");
    GRGX_CHECK(init_kind >= GRGX_INIT_ZERO && init_kind <= GRGX_INIT_XTX, GRGX_ERR_API_MISUSE,
               "Unexpected init value");
    GRGX_CHECK((init_kind != GRGX_INIT_VECTOR && init_kind != GRGX_INIT_MATRIX) || init != nullptr,
               GRGX_ERR_API_MISUSE, "init matrix is missing");
    GRGX_CHECK(!(miss && emit_all), GRGX_ERR_API_MISUSE,
               "The \"miss\" parameter cannot be mixed with the \"emit_all_nodes\" parameter");

    if (init_kind == GRGX_INIT_XTX) {
        {
            std::lock_guard<std::mutex> lk(g->mu);
            if (g->has_coals < 0) {
                bool ok = hg.coals.size() >= n - N;
                for (uint64_t i = 0; ok && i < n - N; i++) ok = (hg.coals[i] != COAL_NOT_SET);
                g->has_coals = ok ? 1 : 0;
            }
        }
        GRGX_CHECK(g->has_coals == 1, GRGX_ERR_API_MISUSE,
                   "Coalescent counts not available for this GRG (init=XTX won't work)");
    }
}

void matmul_direct(grgx_graph* g, int dtype, const void* input, uint64_t in_cols, uint64_t rows, int direction,
                   void* output, uint64_t output_size, int emit_all, int by_indiv, const void* init, int init_kind,
                   void* miss, uint32_t flags, void* stream_ptr) {
    const HostGraph& hg = *g->host;
    const uint64_t n = hg.num_nodes, N = hg.num_samples, M = hg.num_mutations, P = hg.ploidy;
    validate_matmul(g, dtype, in_cols, rows, direction, output_size, emit_all, by_indiv, init, init_kind, miss);
    const uint64_t out_cols = output_size / rows;
    DevicePlan* dp = ensure_device_plan(g);

    cudaStream_t s = static_cast<cudaStream_t>(stream_ptr);
    const bool devPtrs = (flags & GRGX_FLAG_DEVICE_POINTERS) != 0;
    const bool overwrite = (flags & GRGX_FLAG_OVERWRITE) != 0;
    const long long K = static_cast<long long>(rows);
    const Layout L = choose_layout(dtype, K, (flags & GRGX_FLAG_F32_PLAIN) != 0, (flags & GRGX_FLAG_F64_NATIVE) != 0);
    const bool df = (L.kind == Kind::F64S);
    const size_t esz = io_size(dtype);
    const bool down = (direction == GRGX_DIRECTION_DOWN);
    const bool useMiss = (miss != nullptr) && dp->has_miss;

    cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
    if (t_timing) {
        for (auto& e : ev) GRGX_CUDA(cudaEventCreate(&e));
        GRGX_CUDA(cudaEventRecord(ev[0], s));
    }
    uint64_t launches = 0;
    {
        Scratch sc(s);
        // ---- I/O buffers -------------------------------------------------------------------
        const size_t inBytes = rows * in_cols * esz, outBytes = rows * out_cols * esz;
        const size_t missBytes = rows * M * esz;
        const size_t initBytes = (init_kind == GRGX_INIT_VECTOR) ? rows * esz
                                 : (init_kind == GRGX_INIT_MATRIX) ? rows * n * esz : 0;
        const void* dIn = input;
        void* dOut = output;
        const void* dInit = init;
        void* dMiss = useMiss ? miss : nullptr;
        if (!devPtrs) {
            void* a = sc.get(inBytes);
            GRGX_CUDA(cudaMemcpyAsync(a, input, inBytes, cudaMemcpyHostToDevice, s));
            dIn = a;
            dOut = sc.get(outBytes);
            if (!overwrite) GRGX_CUDA(cudaMemcpyAsync(dOut, output, outBytes, cudaMemcpyHostToDevice, s));
            if (initBytes) {
                void* b = sc.get(initBytes);
                GRGX_CUDA(cudaMemcpyAsync(b, init, initBytes, cudaMemcpyHostToDevice, s));
                dInit = b;
            }
            if (useMiss) {
                dMiss = sc.get(missBytes);
                GRGX_CUDA(cudaMemcpyAsync(dMiss, miss, missBytes, cudaMemcpyHostToDevice, s));
            }
        }
        // ---- node values and the per-call scratch ---------------------------------------------
        const size_t valBytes = static_cast<size_t>(n) * L.stride * L.ssize;
        void* vals = sc.get(valBytes);
        // UP in split form when the height-0 rows outgrow L2: their edges first, in blocked
        // passes, then the other edges level by level (up_split.cu)
        const bool split = !down && use_up_split(g, dp, L);
        // DOWN in split form: the height-0 level in parent blocks (up_split.cu)
        const bool dsplit = down && use_down_split(g, dp, L);
        // coarse or fine chunking for this row width (the split copies are built by now)
        const SweepCSRs cs = sweep_csrs(dp, L);
        const DevCSR& cUp = *cs.up;
        const DevCSR& cDown = *cs.down;
        const DevCSR& cUp0b = *cs.up0b;
        const DevCSR& cUpInt = *cs.up_int;
        const DevCSR& cDown0b = *cs.down0b;
        long long pieces = down ? std::max(cDown.n_pieces, std::max(dp->seed.n_pieces, dp->miss.n_pieces))
                                : (split ? std::max(cUp0b.n_pieces, cUpInt.n_pieces) : cUp.n_pieces);
        if (dsplit) pieces = std::max(pieces, cDown0b.n_pieces);
        void* partials = sc.get(static_cast<size_t>(pieces) * L.stride * L.asize);
        const long long nh = down ? (cDown.n_heavy + dp->seed.n_heavy + dp->miss.n_heavy +
                                     (dsplit ? cDown0b.n_heavy : 0))
                                  : (split ? cUp0b.n_heavy + cUpInt.n_heavy : cUp.n_heavy);
        const long long nslots = down ? (2 + static_cast<long long>(cDown.lb.size()) +
                                         (dsplit ? static_cast<long long>(cDown0b.lb.size()) : 0))
                                      : static_cast<long long>(split ? cUp0b.lb.size() + cUpInt.lb.size()
                                                                     : cUp.lb.size());
        const long long h0 = static_cast<long long>(dp->level_begin.size() > 1 ? dp->level_begin[1] : 0);
        const size_t stateBytes = split    ? static_cast<size_t>(n - dp->split_src) * L.stride * std::max(L.asize, 8)
                                  : dsplit ? static_cast<size_t>(h0) * L.stride * std::max(L.asize, 8)
                                           : 0;
        void* state = (split || dsplit) ? sc.get(stateBytes) : nullptr;
        // counters per launch and per heavy row: enough column tiles for any launch shape
        const int TS = max_tiles(L);
        const size_t counterBytes = static_cast<size_t>(nh + nslots) * TS * sizeof(unsigned);
        unsigned* tickets = static_cast<unsigned*>(sc.get(counterBytes));
        GRGX_CUDA(cudaMemsetAsync(tickets, 0, counterBytes, s));
        unsigned* work = tickets + nh * TS;  // one set of TS counters per launch

        // ---- float64: row scales and the device-side choice between the float-pair path (gate
        // 0) and the FP64-pipe path (gate 1, for rows spanning too many binades) ---------------
        unsigned long long* rowmax = nullptr;
        int* gate = nullptr;
        if (df) {
            rowmax = static_cast<unsigned long long*>(sc.get(2 * static_cast<size_t>(K) * sizeof(unsigned long long)));
            unsigned long long* rowmin = rowmax + K;
            gate = static_cast<int*>(sc.get(sizeof(int)));
            unsigned long long floor = 0;
            if (init_kind == GRGX_INIT_XTX) std::memcpy(&floor, &dp->xtx_max, sizeof(floor));
            launch_fill_u64(rowmax, K, floor, s);
            unsigned long long two = 0;  // smallest nonzero XTX value, 2 * one coalescence
            const double twoD = 2.0;
            std::memcpy(&two, &twoD, sizeof(two));
            launch_fill_u64(rowmin, K, (init_kind == GRGX_INIT_XTX && floor) ? two : ~0ull, s);
            launch_rowmax(static_cast<const double*>(dIn), K, in_cols, in_cols, rowmax, rowmin, s);
            launches += 3;
            if (init_kind == GRGX_INIT_VECTOR) {
                launch_rowmax(static_cast<const double*>(dInit), K, 1, 1, rowmax, rowmin, s);
                launches++;
            }
            if (init_kind == GRGX_INIT_MATRIX) {
                launch_rowmax(static_cast<const double*>(dInit), K, n, n, rowmax, rowmin, s);
                launches++;
            }
            if (down && dMiss) {
                launch_rowmax(static_cast<const double*>(dMiss), K, M, M, rowmax, rowmin, s);
                launches++;
            }
            launch_decide_f64_path(rowmax, rowmin, K, gate, s);
            launches++;
        }
        const int hasInit = (init_kind != GRGX_INIT_ZERO);
        const int add = overwrite ? 0 : 1;
        if (init_kind == GRGX_INIT_ZERO) GRGX_CUDA(cudaMemsetAsync(vals, 0, valBytes, s));
        // Scratch shared by both float64 paths (same 8-byte elements).
        void* vt = (down && dp->seed.n_edges > 0) ? sc.get(static_cast<size_t>(M) * L.stride * L.ssize) : nullptr;
        void* mt = (down && useMiss && dp->miss.n_edges > 0) ? sc.get(static_cast<size_t>(M) * L.stride * L.ssize)
                                                              : nullptr;

        // One full pipeline (init, seed, level sweep, gather) for layout LL; `pdf` selects the
        // float-pair I/O kernels; kernels run only where *g == gv when g is set.
        auto pipeline = [&](const Layout& LL, bool pdf, const int* g, int gv, bool timed) {
            auto load_rows = [&](const void* src, long long ld, long long R, int mode, long long div,
                                 const uint32_t* tab, void* dst, int addTo) {
                if (pdf)
                    launch_load_rows_df(static_cast<const double*>(src), K, ld, R, mode, div, tab, dst, LL.stride,
                                        addTo, rowmax, s, g);
                else
                    launch_load_rows(dtype, src, K, ld, R, mode, div, tab, dst, LL.stride, addTo, s, g, gv);
                launches++;
            };
            auto store_cols = [&](long long C, int mode, long long fold, const uint32_t* tab, void* out, long long ld,
                                  int addTo) {
                if (pdf)
                    launch_store_cols_df(vals, LL.stride, K, C, mode, fold, tab, static_cast<double*>(out), ld, addTo,
                                         rowmax, s, g);
                else
                    launch_store_cols(dtype, vals, LL.stride, K, C, mode, fold, tab, out, ld, addTo, s, g, gv);
                launches++;
            };
            auto level = [&](const DevCSR& c, size_t lvl, const void* src, int rmw, unsigned* tk, unsigned* wk) {
                const LevelShape sh = level_shape(LL, c, lvl);
                return launch_level(LL, c, lvl, src, vals, rmw, partials, tk, wk, s, g, gv, &sh, TS);
            };
            switch (init_kind) {
            case GRGX_INIT_VECTOR:
                if (pdf)
                    launch_init_vector_df(static_cast<const double*>(dInit), K, n, vals, LL.stride, rowmax, s, g);
                else
                    launch_init_vector(dtype, dInit, K, n, vals, LL.stride, s, g, gv);
                launches++;
                break;
            case GRGX_INIT_MATRIX: load_rows(dInit, n, n, MAP_TABLE, 1, dp->new2old, vals, 0); break;
            case GRGX_INIT_XTX:
                if (pdf)
                    launch_init_xtx_df(dp->xtx_new, K, n, vals, LL.stride, rowmax, s, g);
                else
                    launch_init_xtx(dtype, dp->xtx_new, K, n, vals, LL.stride, s, g, gv);
                launches++;
                break;
            default: break;
            }
            if (down) {
                // DOWN seed: mutation rows, then node <- sum of its mutations (and missingness)
                unsigned* tk = tickets;
                if (vt) {
                    load_rows(dIn, in_cols, M, MAP_IDENT, 1, nullptr, vt, 0);
                    launches += level(dp->seed, 0, vt, hasInit, tk, work);
                }
                tk += dp->seed.n_heavy * TS;
                if (mt) {
                    load_rows(dMiss, M, M, MAP_IDENT, 1, nullptr, mt, 0);
                    launches += level(dp->miss, 0, mt, 1, tk, work + TS);
                }
                tk += dp->miss.n_heavy * TS;
                if (timed && t_timing) GRGX_CUDA(cudaEventRecord(ev[1], s));
                const size_t nlv = cDown.lb.size();
                for (size_t lvl = 0; lvl < nlv; lvl++) {
                    if (dsplit && lvl + 1 == nlv) break;  // the height-0 level runs in split form below
                    launches += level(cDown, lvl, vals, 1, tk, work + (2 + lvl) * TS);
                }
                if (dsplit) {
                    // parent-block passes merge each height-0 row's sums into its state; then the
                    // rows are written from it, onto their seed / init values
                    GRGX_CUDA(cudaMemsetAsync(state, 0, stateBytes, s));
                    unsigned* tS = tk + cDown.n_heavy * TS;
                    unsigned* wS = work + (2 + nlv) * TS;
                    for (size_t j = 0; j < cDown0b.lb.size(); j++) {
                        const LevelShape sh = level_shape(LL, cDown0b, j);
                        launches += launch_level(LL, cDown0b, j, vals, vals, 0, partials, tS, wS + j * TS, s, g,
                                                 gv, &sh, TS, state, 0, 1);
                    }
                    launch_state_finish(LL.kind, state, vals, dp->fin_down, dp->n_fin_down, 0, LL.stride, 1, s, g,
                                        gv);
                    launches++;
                }
                if (timed && t_timing) GRGX_CUDA(cudaEventRecord(ev[2], s));
                if (emit_all) {
                    store_cols(n, MAP_TABLE, 1, dp->old2new, dOut, out_cols, add);
                } else if (by_indiv) {
                    store_cols(out_cols, MAP_FOLD, P, nullptr, dOut, out_cols, add);
                } else {
                    store_cols(out_cols, MAP_IDENT, 1, nullptr, dOut, out_cols, add);
                }
            } else {
                // UP seed: samples <- input columns
                load_rows(dIn, in_cols, N, by_indiv ? MAP_DIV : MAP_IDENT, P, nullptr, vals, hasInit);
                if (timed && t_timing) GRGX_CUDA(cudaEventRecord(ev[1], s));
                if (split) {
                    GRGX_CUDA(cudaMemsetAsync(state, 0, stateBytes, s));
                    unsigned* t0b = tickets;
                    unsigned* tIn = tickets + cUp0b.n_heavy * TS;
                    unsigned* w0b = work;
                    unsigned* wIn = work + cUp0b.lb.size() * TS;
                    const long long base = dp->split_src;
                    for (size_t j = 0; j < cUp0b.lb.size(); j++) {
                        const LevelShape sh = level_shape(LL, cUp0b, j);
                        launches += launch_level(LL, cUp0b, j, vals, vals, 0, partials, t0b, w0b + j * TS, s, g,
                                                 gv, &sh, TS, state, base, 1);
                    }
                    for (size_t lvl = 0; lvl < cUpInt.lb.size(); lvl++) {
                        const LevelShape sh = level_shape(LL, cUpInt, lvl);
                        launches += launch_level(LL, cUpInt, lvl, vals, vals, hasInit, partials, tIn,
                                                 wIn + lvl * TS, s, g, gv, &sh, TS, state, base, 2);
                        const long long f0 = dp->fin_begin[lvl], f1 = dp->fin_begin[lvl + 1];
                        if (f1 > f0) {
                            launch_state_finish(LL.kind, state, vals, dp->fin + f0, f1 - f0, base, LL.stride, hasInit,
                                                s, g, gv);
                            launches++;
                        }
                    }
                } else {
                    for (size_t lvl = 0; lvl < cUp.lb.size(); lvl++)
                        launches += level(cUp, lvl, vals, hasInit, tickets, work + lvl * TS);
                }
                if (timed && t_timing) GRGX_CUDA(cudaEventRecord(ev[2], s));
                if (emit_all) {
                    store_cols(n, MAP_TABLE, 1, dp->old2new, dOut, out_cols, add);
                } else {
                    store_cols(M, MAP_TABLE, 1, dp->mut_new, dOut, out_cols, add);
                    if (useMiss) store_cols(M, MAP_TABLE, 1, dp->miss_new, dMiss, M, 1);
                }
            }
        };
        if (df) {
            Layout LN = L;
            LN.kind = Kind::F64;
            pipeline(L, true, gate, 0, true);
            pipeline(LN, false, gate, 1, false);
        } else {
            pipeline(L, false, nullptr, 0, true);
        }
        GRGX_CUDA(cudaGetLastError());
        if (!devPtrs) {
            GRGX_CUDA(cudaMemcpyAsync(output, dOut, outBytes, cudaMemcpyDeviceToHost, s));
            if (useMiss && !down) GRGX_CUDA(cudaMemcpyAsync(miss, dMiss, missBytes, cudaMemcpyDeviceToHost, s));
        }
    }  // scratch released (stream-ordered)
    if (t_timing) {
        GRGX_CUDA(cudaEventRecord(ev[3], s));
        const DevCSR& c = down ? dp->down : dp->up;
        const uint64_t algBytes = static_cast<uint64_t>(c.n_edges) * (4 + static_cast<uint64_t>(K) * L.ssize) +
                                  static_cast<uint64_t>(c.n_rows) * (8 + static_cast<uint64_t>(K) * L.ssize);
        if (t_timing == 2) {
            t_pending.push_back(PendingTiming{{ev[0], ev[1], ev[2], ev[3]}, launches, algBytes});
        } else {
            GRGX_CUDA(cudaEventSynchronize(ev[3]));
            float tot = 0, sw = 0;
            cudaEventElapsedTime(&tot, ev[0], ev[3]);
            cudaEventElapsedTime(&sw, ev[1], ev[2]);
            for (auto& e : ev) cudaEventDestroy(e);
            t_last.total_ms = tot;
            t_last.sweep_ms = sw;
            t_last.launches = launches;
            t_last.alg_bytes = algBytes;
        }
    } else {
        t_last.launches = launches;
    }
    const bool hostWait = !devPtrs && !(flags & GRGX_FLAG_ASYNC);
    if (hostWait || (flags & GRGX_FLAG_SYNC)) GRGX_CUDA(cudaStreamSynchronize(s));
}

// ---- captured CUDA graphs of whole calls (small graphs) ----------------------------------------

struct GraphEntry {
    std::mutex mu;
    cudaStream_t stream = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaEvent_t ready = nullptr, done = nullptr;
    void *in = nullptr, *out = nullptr, *init = nullptr, *miss = nullptr;
    size_t inBytes = 0, outBytes = 0, initBytes = 0, missBytes = 0;
    ~GraphEntry() {
        if (exec) cudaGraphExecDestroy(exec);
        if (ready) cudaEventDestroy(ready);
        if (done) cudaEventDestroy(done);
        for (void* p : {in, out, init, miss})
            if (p) cudaFree(p);
        if (stream) cudaStreamDestroy(stream);
    }
};

struct GraphCache {
    std::mutex mu;
    std::map<std::vector<uint64_t>, std::unique_ptr<GraphEntry>> entries;
};

void destroy_graph_cache(GraphCache* c) { delete c; }

namespace {
constexpr uint64_t kGraphMaxEdges = 1ull << 25;
constexpr size_t kGraphMaxEntries = 64;
}  // namespace

void matmul_impl(grgx_graph* g, int dtype, const void* input, uint64_t in_cols, uint64_t rows, int direction,
                 void* output, uint64_t output_size, int emit_all, int by_indiv, const void* init, int init_kind,
                 void* miss, uint32_t flags, void* stream_ptr) {
    const HostGraph& hg = *g->host;
    validate_matmul(g, dtype, in_cols, rows, direction, output_size, emit_all, by_indiv, init, init_kind, miss);
    const bool eligible = !(flags & GRGX_FLAG_NO_GRAPH) && !t_timing && hg.num_edges() <= kGraphMaxEdges &&
                          hg.num_edges() > 0 && rows > 0 && in_cols > 0 && output_size % rows == 0;
    if (!eligible) {
        matmul_direct(g, dtype, input, in_cols, rows, direction, output, output_size, emit_all, by_indiv, init,
                      init_kind, miss, flags, stream_ptr);
        return;
    }
    const bool devPtrs = (flags & GRGX_FLAG_DEVICE_POINTERS) != 0;
    const bool overwrite = (flags & GRGX_FLAG_OVERWRITE) != 0;
    const bool useMiss = miss != nullptr && !hg.miss_node.empty();
    const size_t esz = io_size(dtype);
    const uint64_t M = hg.num_mutations, n = hg.num_nodes;
    cudaStream_t user = static_cast<cudaStream_t>(stream_ptr);
    const std::vector<uint64_t> key = {static_cast<uint64_t>(dtype), rows, in_cols, output_size,
                                       static_cast<uint64_t>(direction), static_cast<uint64_t>(emit_all),
                                       static_cast<uint64_t>(by_indiv), static_cast<uint64_t>(init_kind),
                                       static_cast<uint64_t>(useMiss),
                                       static_cast<uint64_t>(flags & (GRGX_FLAG_F32_PLAIN | GRGX_FLAG_F64_NATIVE)),
                                       static_cast<uint64_t>(overwrite),
                                       reinterpret_cast<uint64_t>(user), static_cast<uint64_t>(devPtrs)};
    GraphEntry* e = nullptr;
    {
        std::lock_guard<std::mutex> lk(g->mu);
        if (!g->graphs) g->graphs.reset(new GraphCache());
    }
    {
        std::lock_guard<std::mutex> lk(g->graphs->mu);
        auto it = g->graphs->entries.find(key);
        if (it != g->graphs->entries.end()) e = it->second.get();
    }
    if (e == nullptr) {
        ensure_device_plan(g);
        auto ent = std::make_unique<GraphEntry>();
        ent->inBytes = rows * in_cols * esz;
        ent->outBytes = output_size * esz;
        ent->initBytes = (init_kind == GRGX_INIT_VECTOR) ? rows * esz : (init_kind == GRGX_INIT_MATRIX ? rows * n * esz : 0);
        ent->missBytes = useMiss ? rows * M * esz : 0;
        GRGX_CUDA(cudaStreamCreateWithFlags(&ent->stream, cudaStreamNonBlocking));
        GRGX_CUDA(cudaEventCreateWithFlags(&ent->ready, cudaEventDisableTiming));
        GRGX_CUDA(cudaEventCreateWithFlags(&ent->done, cudaEventDisableTiming));
        GRGX_CUDA(cudaMalloc(&ent->in, ent->inBytes));
        GRGX_CUDA(cudaMalloc(&ent->out, ent->outBytes));
        if (ent->initBytes) GRGX_CUDA(cudaMalloc(&ent->init, ent->initBytes));
        if (ent->missBytes) GRGX_CUDA(cudaMalloc(&ent->miss, ent->missBytes));
        // a first direct run on the staging buffers validates the call (errors before capture)
        GRGX_CUDA(cudaMemsetAsync(ent->in, 0, ent->inBytes, ent->stream));
        matmul_direct(g, dtype, ent->in, in_cols, rows, direction, ent->out, output_size, emit_all, by_indiv,
                      init_kind == GRGX_INIT_VECTOR || init_kind == GRGX_INIT_MATRIX ? ent->init : init, init_kind,
                      useMiss ? ent->miss : nullptr, (flags | GRGX_FLAG_DEVICE_POINTERS | GRGX_FLAG_NO_GRAPH) & ~GRGX_FLAG_SYNC,
                      ent->stream);
        GRGX_CUDA(cudaStreamSynchronize(ent->stream));
        cudaGraph_t graph = nullptr;
        bool captured = false;
        if (cudaStreamBeginCapture(ent->stream, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
            bool ok = true;
            try {
                matmul_direct(g, dtype, ent->in, in_cols, rows, direction, ent->out, output_size, emit_all, by_indiv,
                              init_kind == GRGX_INIT_VECTOR || init_kind == GRGX_INIT_MATRIX ? ent->init : init,
                              init_kind, useMiss ? ent->miss : nullptr,
                              (flags | GRGX_FLAG_DEVICE_POINTERS | GRGX_FLAG_NO_GRAPH) & ~GRGX_FLAG_SYNC, ent->stream);
            } catch (...) {
                ok = false;
            }
            const cudaError_t ee = cudaStreamEndCapture(ent->stream, &graph);
            captured = ok && ee == cudaSuccess && graph != nullptr &&
                       cudaGraphInstantiate(&ent->exec, graph, 0) == cudaSuccess;
            if (graph) cudaGraphDestroy(graph);
        }
        if (!captured) {
            // The capture failed -- another thread's device-wide operation (a synchronisation, a
            // free that synchronises) invalidates a capture in progress: this call runs directly
            // and a later call of the same shape captures again.
            cudaGetLastError();
            matmul_direct(g, dtype, input, in_cols, rows, direction, output, output_size, emit_all, by_indiv, init,
                          init_kind, miss, flags | GRGX_FLAG_NO_GRAPH, stream_ptr);
            return;
        }
        std::lock_guard<std::mutex> lk(g->graphs->mu);
        auto it = g->graphs->entries.find(key);
        if (it != g->graphs->entries.end()) {
            e = it->second.get();  // another thread won the race
        } else if (g->graphs->entries.size() < kGraphMaxEntries) {
            e = ent.get();
            g->graphs->entries[key] = std::move(ent);
        } else {
            // cache full: run directly
            matmul_direct(g, dtype, input, in_cols, rows, direction, output, output_size, emit_all, by_indiv, init,
                          init_kind, miss, flags | GRGX_FLAG_NO_GRAPH, stream_ptr);
            return;
        }
    }
    std::lock_guard<std::mutex> lk(e->mu);
    const cudaMemcpyKind in = devPtrs ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
    const cudaMemcpyKind outk = devPtrs ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
    // ordered after the caller's stream (device buffers, or host buffers queued asynchronously)
    const bool onUser = devPtrs || (flags & GRGX_FLAG_ASYNC);
    if (onUser) {
        GRGX_CUDA(cudaEventRecord(e->ready, user));
        GRGX_CUDA(cudaStreamWaitEvent(e->stream, e->ready, 0));
    }
    GRGX_CUDA(cudaMemcpyAsync(e->in, input, e->inBytes, in, e->stream));
    if (e->initBytes) GRGX_CUDA(cudaMemcpyAsync(e->init, init, e->initBytes, in, e->stream));
    if (e->missBytes) GRGX_CUDA(cudaMemcpyAsync(e->miss, miss, e->missBytes, in, e->stream));
    if (!overwrite) GRGX_CUDA(cudaMemcpyAsync(e->out, output, e->outBytes, in, e->stream));
    GRGX_CUDA(cudaGraphLaunch(e->exec, e->stream));
    GRGX_CUDA(cudaMemcpyAsync(output, e->out, e->outBytes, outk, e->stream));
    if (e->missBytes && direction == GRGX_DIRECTION_UP)
        GRGX_CUDA(cudaMemcpyAsync(miss, e->miss, e->missBytes, outk, e->stream));
    if (onUser) {
        GRGX_CUDA(cudaEventRecord(e->done, e->stream));
        GRGX_CUDA(cudaStreamWaitEvent(user, e->done, 0));
        if (flags & GRGX_FLAG_SYNC) GRGX_CUDA(cudaStreamSynchronize(user));
    } else {
        GRGX_CUDA(cudaStreamSynchronize(e->stream));
    }
}

void clear_graph_replays(grgx_graph* g) {
    std::lock_guard<std::mutex> lk(g->mu);
    g->graphs.reset();
}

void set_timing(int enabled) { t_timing = enabled == 2 ? 2 : (enabled != 0 ? 1 : 0); }
grgx_timing last_timing() { return t_last; }

// Reads back (waiting for them) and clears this thread's deferred timings, in call order.
std::vector<grgx_timing> collect_timings() {
    std::vector<grgx_timing> out;
    for (PendingTiming& p : t_pending) {
        grgx_timing t{};
        cudaEventSynchronize(p.ev[3]);
        cudaEventElapsedTime(&t.total_ms, p.ev[0], p.ev[3]);
        cudaEventElapsedTime(&t.sweep_ms, p.ev[1], p.ev[2]);
        for (auto& e : p.ev) cudaEventDestroy(e);
        t.launches = p.launches;
        t.alg_bytes = p.alg_bytes;
        out.push_back(t);
    }
    t_pending.clear();
    return out;
}

}  // namespace grgx
