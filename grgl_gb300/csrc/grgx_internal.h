// Internal host-side types shared by the grgx translation units.
#pragma once

#include <cstddef>
#include <cstdint>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>
#include <vector>

#include "grgx.h"

namespace grgx {

constexpr uint32_t INVALID_NODE = 0x7fffffffu;   // grgnode.h:58
constexpr uint32_t COAL_NOT_SET = 0xffffffffu;   // node_data.h:31
constexpr uint32_t HEAD_BIT = 0x80000000u;       // marks the first edge of a row in a device CSR
constexpr uint64_t MAX_NODES = 0x7fffffffu - 1;  // grgnode.h:57

// Error carrying a grgx status code; the C-ABI turns it into a return value plus the
// thread-local message returned by grgx_last_error().
struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string& msg) : std::runtime_error(msg), code(c) {}
};

#define GRGX_CHECK(cond, code, msg)                                                                    \
    do {                                                                                              \
        if (!(cond)) throw ::grgx::Error((code), (msg));                                              \
    } while (0)

// A GRG as the matmul path needs it: the down-edge CSR (children in ascending id order, as a
// CSRGRG stores them), the mutation -> node map, optional missingness nodes and coalescence
// counts.  Samples are nodes 0..num_samples-1 (grg.h:271-275).
struct HostGraph {
    uint64_t num_nodes = 0;
    uint64_t num_samples = 0;
    uint64_t ploidy = 2;
    uint64_t num_mutations = 0;
    bool phased = true;
    std::vector<uint64_t> down_off;   // num_nodes + 1
    std::vector<uint32_t> down_adj;   // num_edges
    std::vector<uint32_t> mut_node;   // num_mutations (INVALID_NODE when unmapped)
    std::vector<uint32_t> miss_node;  // empty, or num_mutations (INVALID_NODE when none)
    std::vector<uint32_t> coals;      // empty, or num_nodes - num_samples
    std::vector<uint64_t> mut_pos;    // optional positions (bp)
    // A graph read from a .grg file keeps its edges as the file stores them -- one vbyte
    // bucket per node -- until something needs them: the device plan decodes the buckets on
    // the GPU (grg_decode.cu); host consumers call materialize_edges first.
    std::vector<uint8_t> enc_buckets;
    std::vector<uint64_t> enc_index;  // bucket byte offset of each node, num_nodes + 1
    uint64_t enc_edges = 0;           // edge count from the file header
    bool encoded() const { return !enc_index.empty(); }
    uint64_t num_edges() const { return encoded() ? enc_edges : down_adj.size(); }
};

// Decodes the vbyte buckets of an encoded graph into down_off / down_adj on the host and drops
// the encoded copy (no-op for a decoded graph).  Throws GRGX_ERR_BAD_FILE on malformed buckets.
void materialize_edges(HostGraph& g);

// Load a .grg file (format 5.x, serialize.cpp:815-890 + readGrgCommon :697-758).
std::unique_ptr<HostGraph> load_grg_file(const std::string& path);
// Save a (decoded) graph as a .grg file (format 5.3) that load_grg_file reads back.
void save_grg_file(const HostGraph& g, const std::string& path);

// Seeded window-tree generator (one Kingman tree per 100-variant window, collapsed to its
// mutation nodes).
std::unique_ptr<HostGraph> generate_window_tree(uint64_t num_samples, uint64_t num_mutations, uint64_t seed,
                                                uint32_t window, int threads);

// ---- level plan (host side; built once per graph) ------------------------------------------

// One unit of warp work in a level sweep: the edges [e0, next.e0) of the direction's CSR.
// `r0` is the index (into rows) of the row that holds edge e0.  `heavy` is -1 for a chunk of
// whole rows, else the index of the heavy row this chunk is a piece of.
struct Chunk {
    int64_t e0;
    int32_t r0;
    int32_t heavy;
};
static_assert(sizeof(Chunk) == 16, "Chunk layout");

struct HeavyRow {
    int32_t first_chunk;  // chunk index of piece 0
    int32_t n_pieces;
    int64_t slot_base;    // first partial slot
};
static_assert(sizeof(HeavyRow) == 16, "HeavyRow layout");

// A pull-form CSR over (renumbered) node ids, arranged level by level in processing order.
struct PullCSR {
    std::vector<int32_t> rows;     // row -> destination node id
    std::vector<uint32_t> adj;     // source ids, HEAD_BIT on each row's first edge (empty when
                                   // the adjacency is built on the device, see HostPlan::down)
    std::vector<int64_t> off;      // row offsets (kept for device-side construction)
    int64_t num_edges = 0;
    std::vector<Chunk> chunks;     // + sentinel {E, R, -1}
    std::vector<HeavyRow> heavy;
    std::vector<int32_t> level_chunk_begin;  // per processed level, chunk range [b, e)
    std::vector<int32_t> level_chunk_end;
    int64_t num_pieces = 0;        // total partial slots
    int64_t max_level_edges = 0;
};

struct HostPlan {
    uint64_t num_levels = 0;              // heights 0..num_levels-1
    std::vector<uint32_t> old2new, new2old;
    std::vector<uint64_t> level_begin;    // new-id range of each height
    PullCSR up;     // levels 1..H ascending; rows = nodes, adj = children
    PullCSR down;   // levels H..0 descending; rows = nodes with parents, adj = parents
                    // (adj left empty: built on the device from `up` by a stable sort)
    std::vector<int32_t> down_row_of;  // new id -> DOWN row (or -1)
    // The same UP and DOWN rows and levels cut into kFineChunkFactor times as many chunks (only
    // chunks, heavy rows and level ranges are filled): calls whose rows are wide enough for the
    // per-chunk cost not to matter run on these (shorter tails at level ends, heavy rows in more
    // pieces).
    PullCSR up_fine, down_fine;
    PullCSR seed;   // one "level": rows = mutation nodes, adj = mutation ids
    PullCSR miss;   // one "level": rows = missingness nodes, adj = mutation ids
    std::vector<uint32_t> mut_new, miss_new;  // mutation -> new node id (or INVALID)
    std::vector<uint32_t> xtx_new;            // 2*coals by new id (COAL_NOT_SET when unknown)
    bool has_coals = false;
    bool has_miss = false;
};

std::unique_ptr<HostPlan> build_plan(const HostGraph& g);

// Stages of the plan shared by the host builder (build_plan) and the device builder
// (plan_device.cu), which computes heights, the renumbering, the UP adjacency and the parent
// counts on the GPU and lays out rows and chunks here.
// Chunks rows rb..re-1 as one level, aiming at `target` chunks (0: chunk_target()).
void chunk_level(PullCSR& P, const std::vector<int64_t>& off, int64_t rb, int64_t re, int64_t target = 0);
// Finer chunking of the wide-row calls: this many times chunk_target() chunks per level.
constexpr int64_t kFineChunkFactor = 4;
// The levels of P (row offsets `off`) chunked again for `factor` times chunk_target() chunks per
// level; the result holds chunks (with the sentinel), heavy rows, level ranges and piece count.
PullCSR rechunk(const PullCSR& P, const std::vector<int64_t>& off, int64_t factor);
// While alive, plans built on this thread size their chunks for a device with `sms` SMs.
class PlanDeviceScope {
  public:
    explicit PlanDeviceScope(int sms);
    ~PlanDeviceScope();
    PlanDeviceScope(const PlanDeviceScope&) = delete;
    PlanDeviceScope& operator=(const PlanDeviceScope&) = delete;

  private:
    int saved_;
};
// Chunks per level the chunker aims for (from the SM count in scope).
int64_t chunk_target();
// SM count of the current device (looked up once per device, matmul.cu).
int sm_count();
void finish_csr(PullCSR& P, const std::vector<int64_t>& off);
void single_level_csr(PullCSR& P, const std::vector<std::pair<uint32_t, uint32_t>>& pairs);
// level_begin from the node count of each height
void plan_levels_from_counts(HostPlan& plan, const std::vector<uint64_t>& perHeight);
// UP rows (every node of height >= 1) and chunks from the row offsets
void plan_up_layout(HostPlan& plan, std::vector<int64_t> off);
// DOWN rows, offsets, down_row_of and chunks from each node's parent count (by new id)
void plan_down_layout(HostPlan& plan, const std::vector<uint64_t>& pdeg);
// mutation seeds, missingness seeds and XTX init values (needs old2new / new2old)
void plan_seeds(HostPlan& plan, const HostGraph& g);

// Device-resident copy of a HostPlan (matmul.cu); freed with destroy_device_plan.
struct DevicePlan;
void destroy_device_plan(DevicePlan* p);
struct DevicePlanDeleter {
    void operator()(DevicePlan* p) const { destroy_device_plan(p); }
};

// Captured CUDA graphs of whole calls on small graphs (matmul.cu).
struct GraphCache;
void destroy_graph_cache(GraphCache* c);
struct GraphCacheDeleter {
    void operator()(GraphCache* c) const { destroy_graph_cache(c); }
};

// Thread-local error message used by the C ABI.
void set_last_error(const std::string& msg);

}  // namespace grgx

// The opaque handle behind grgx_graph*.
struct grgx_graph {
    // The host graph with its edges decoded (decodes an encoded graph once).
    grgx::HostGraph& host_edges() {
        std::lock_guard<std::mutex> lk(edges_mu);
        grgx::materialize_edges(*host);
        return *host;
    }
    std::unique_ptr<grgx::HostGraph> host;
    std::unique_ptr<grgx::HostPlan> plan;
    std::unique_ptr<grgx::HostPlan> inspect_plan;  // host-built plan kept for grgx_debug_host_plan
    std::unique_ptr<grgx::DevicePlan, grgx::DevicePlanDeleter> dev;
    std::unique_ptr<grgx::GraphCache, grgx::GraphCacheDeleter> graphs;  // destroyed before `dev`
    std::mutex mu;  // guards plan/dev creation
    int has_coals = -1;  // cached: every non-sample node has a coalescence count (-1 = not computed)
    bool host_plan = false;  // build the plan on the host (plan.cpp) instead of the device
    std::mutex edges_mu;     // guards materialize_edges of `host`
};
