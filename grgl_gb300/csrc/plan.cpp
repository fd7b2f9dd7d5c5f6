// Level plan: flattens a GRG into the device layout the sweep kernels read.
//
// Heights: h(v) = 0 for a node without children, else 1 + max h(child) -- the same levels the
// reference GPU builder computes with its DFS visitor (include/grgl/cuda/gpu_grg.h:513-551).
// Nodes are renumbered height-major, ascending original id inside a height, so samples keep
// ids 0..N-1 and each height is one contiguous id range.
//
// Both traversal directions are pull-form, so no kernel needs atomics on node values:
//   UP   value[v] = seed[v] + sum over children   (grg.h:1324-1334), heights 1..H ascending
//   DOWN value[v] = seed[v] + sum over parents    (the push of grg.h:1312-1322 turned into a
//        pull), heights H..0 descending, over the nodes that have parents.
// Each direction is a CSR whose rows are laid out level by level in processing order; the
// first edge of every row carries HEAD_BIT so a warp can find row boundaries with one ballot.
// Every level's edge range is cut into chunks of about the same edge count; a row with more
// edges than the chunk size is cut into pieces whose partial sums are combined in piece order.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <functional>
#include <numeric>
#include <thread>

#include "grgx_internal.h"

namespace grgx {
namespace {

int host_threads() {
    unsigned t = std::thread::hardware_concurrency();
    return t == 0 ? 4 : static_cast<int>(std::min(t, 64u));
}

void parallel_for(uint64_t n, const std::function<void(uint64_t, uint64_t, int)>& fn, int threads = 0) {
    if (threads <= 0) threads = host_threads();
    if (n < 65536 || threads == 1) {
        fn(0, n, 0);
        return;
    }
    std::vector<std::thread> pool;
    for (int t = 0; t < threads; t++) {
        const uint64_t b = n * t / threads, e = n * (t + 1) / threads;
        pool.emplace_back([=, &fn] { fn(b, e, t); });
    }
    for (auto& th : pool) th.join();
}

}  // namespace

// Chunk target (the coarse chunking): SMs x 128 chunks per level -- about four per resident warp
// of the sweep kernel (32 warps per SM) -- never fewer than 64 edges per chunk; the fine chunking
// aims at kFineChunkFactor times as many.  The SM count is that of the device the plan is built
// for (PlanDeviceScope); a plan built with no device in view (host-side inspection) assumes a
// GB300's 152 SMs.
constexpr int64_t kMinChunk = 64;
constexpr int64_t kMaxChunk = 1 << 22;
constexpr int kHostOnlySms = 152;
thread_local int t_plan_sms = 0;

PlanDeviceScope::PlanDeviceScope(int sms) : saved_(t_plan_sms) { t_plan_sms = sms; }
PlanDeviceScope::~PlanDeviceScope() { t_plan_sms = saved_; }

int64_t chunk_target() { return static_cast<int64_t>(t_plan_sms > 0 ? t_plan_sms : kHostOnlySms) * 16 * 8; }

void chunk_level(PullCSR& P, const std::vector<int64_t>& off, int64_t rb, int64_t re, int64_t target) {
    P.level_chunk_begin.push_back(static_cast<int32_t>(P.chunks.size()));
    const int64_t levelEdges = off[re] - off[rb];
    P.max_level_edges = std::max(P.max_level_edges, levelEdges);
    if (target <= 0) target = chunk_target();
    int64_t C = (levelEdges + target - 1) / target;
    C = ((C + 31) / 32) * 32;
    C = std::max(kMinChunk, std::min(kMaxChunk, C));
    int64_t r = rb;
    while (r < re) {
        const int64_t deg = off[r + 1] - off[r];
        if (deg > C) {
            const int64_t np = (deg + C - 1) / C;
            HeavyRow hr{};
            hr.first_chunk = static_cast<int32_t>(P.chunks.size());
            hr.n_pieces = static_cast<int32_t>(np);
            hr.slot_base = P.num_pieces;
            const int32_t hid = static_cast<int32_t>(P.heavy.size());
            for (int64_t p = 0; p < np; p++)
                P.chunks.push_back(Chunk{off[r] + deg * p / np, static_cast<int32_t>(r), hid});
            P.heavy.push_back(hr);
            P.num_pieces += np;
            r++;
            continue;
        }
        const int64_t r0 = r;
        int64_t total = 0;
        while (r < re) {
            const int64_t d = off[r + 1] - off[r];
            if (d > C || (total + d > C && r > r0)) break;
            total += d;
            r++;
        }
        P.chunks.push_back(Chunk{off[r0], static_cast<int32_t>(r0), -1});
    }
    P.level_chunk_end.push_back(static_cast<int32_t>(P.chunks.size()));
}

PullCSR rechunk(const PullCSR& P, const std::vector<int64_t>& off, int64_t factor) {
    PullCSR Q;
    const int64_t target = chunk_target() * factor;
    for (size_t l = 0; l < P.level_chunk_begin.size(); l++) {
        // a level's rows: from its first chunk's row to the next level's (or the sentinel's)
        const int64_t rb = P.chunks[static_cast<size_t>(P.level_chunk_begin[l])].r0;
        const int64_t re = P.chunks[static_cast<size_t>(P.level_chunk_end[l])].r0;
        chunk_level(Q, off, rb, re, target);
    }
    Q.chunks.push_back(Chunk{off.empty() ? 0 : off.back(), static_cast<int32_t>(P.rows.size()), -1});
    Q.num_edges = P.num_edges;
    return Q;
}

void finish_csr(PullCSR& P, const std::vector<int64_t>& off) {
    P.chunks.push_back(Chunk{off.back(), static_cast<int32_t>(P.rows.size()), -1});
    P.num_edges = off.back();
    GRGX_CHECK(P.chunks.size() < 0x7fffffffull && P.heavy.size() < 0x7fffffffull, GRGX_ERR_UNSUPPORTED,
               "graph too large for the chunk index");
}

// A one-level CSR from (node, source) pairs sorted by node then source.
void single_level_csr(PullCSR& P, const std::vector<std::pair<uint32_t, uint32_t>>& pairs) {
    std::vector<int64_t> off;
    off.push_back(0);
    for (size_t i = 0; i < pairs.size(); i++) {
        if (i == 0 || pairs[i].first != pairs[i - 1].first) {
            if (i) off.push_back(static_cast<int64_t>(i));
            P.rows.push_back(static_cast<int32_t>(pairs[i].first));
            P.adj.push_back(pairs[i].second | HEAD_BIT);
        } else {
            P.adj.push_back(pairs[i].second);
        }
    }
    if (!pairs.empty()) off.push_back(static_cast<int64_t>(pairs.size()));
    if (!P.rows.empty()) chunk_level(P, off, 0, static_cast<int64_t>(P.rows.size()));
    finish_csr(P, off);
}

namespace {
struct PhaseTimer {
    const char* name;
    std::chrono::steady_clock::time_point t0 = std::chrono::steady_clock::now();
    bool on = std::getenv("GRGX_PLAN_TIMING") != nullptr;
    void lap(const char* what) {
        if (!on) return;
        const auto t1 = std::chrono::steady_clock::now();
        std::fprintf(stderr, "[plan] %-12s %8.3f s\n", what, std::chrono::duration<double>(t1 - t0).count());
        t0 = t1;
    }
};
}  // namespace

// ---- stages shared by the host and the device builders --------------------------------------

void plan_levels_from_counts(HostPlan& plan, const std::vector<uint64_t>& perHeight) {
    const uint64_t L = perHeight.size();
    plan.num_levels = L;
    plan.level_begin.assign(L + 1, 0);
    for (uint64_t h = 0; h < L; h++) plan.level_begin[h + 1] = plan.level_begin[h] + perHeight[h];
}

void plan_up_layout(HostPlan& plan, std::vector<int64_t> off) {
    PullCSR& P = plan.up;
    const uint64_t L = plan.num_levels;
    const uint64_t n = plan.level_begin.empty() ? 0 : plan.level_begin[L];
    const uint64_t r0 = L > 1 ? plan.level_begin[1] : n;
    const uint64_t R = n - r0;
    P.rows.resize(R);
    for (uint64_t i = 0; i < R; i++) P.rows[i] = static_cast<int32_t>(r0 + i);
    for (uint64_t h = 1; h < L; h++)
        chunk_level(P, off, static_cast<int64_t>(plan.level_begin[h] - r0),
                    static_cast<int64_t>(plan.level_begin[h + 1] - r0));
    finish_csr(P, off);
    plan.up_fine = rechunk(P, off, kFineChunkFactor);
    P.off = std::move(off);
}

void plan_down_layout(HostPlan& plan, const std::vector<uint64_t>& pdeg) {
    PullCSR& P = plan.down;
    const uint64_t L = plan.num_levels;
    const uint64_t n = pdeg.size();
    // Row order: heights descending, ids ascending inside a height.
    std::vector<uint32_t> rowNode;
    rowNode.reserve(n);
    for (uint64_t hh = L; hh > 0; hh--) {
        const uint64_t h = hh - 1;
        for (uint64_t id = plan.level_begin[h]; id < plan.level_begin[h + 1]; id++)
            if (pdeg[id]) rowNode.push_back(static_cast<uint32_t>(id));
    }
    const uint64_t R = rowNode.size();
    std::vector<int64_t> off(R + 1, 0);
    for (uint64_t i = 0; i < R; i++) off[i + 1] = off[i] + static_cast<int64_t>(pdeg[rowNode[i]]);
    P.rows.assign(rowNode.begin(), rowNode.end());
    plan.down_row_of.assign(n, -1);
    for (uint64_t i = 0; i < R; i++) plan.down_row_of[rowNode[i]] = static_cast<int32_t>(i);
    // Level ranges over rows.
    uint64_t rb = 0;
    for (uint64_t hh = L; hh > 0; hh--) {
        const uint64_t h = hh - 1;
        uint64_t re = rb;
        while (re < R && rowNode[re] >= plan.level_begin[h] && rowNode[re] < plan.level_begin[h + 1]) re++;
        chunk_level(P, off, static_cast<int64_t>(rb), static_cast<int64_t>(re));
        rb = re;
    }
    finish_csr(P, off);
    plan.down_fine = rechunk(P, off, kFineChunkFactor);
    P.off = std::move(off);
}

void plan_seeds(HostPlan& plan, const HostGraph& g) {
    const uint64_t n = g.num_nodes, N = g.num_samples;
    const auto& o2n = plan.old2new;
    const auto& n2o = plan.new2old;
    plan.mut_new.assign(g.num_mutations, INVALID_NODE);
    std::vector<std::pair<uint32_t, uint32_t>> pairs;
    for (uint64_t m = 0; m < g.num_mutations; m++) {
        if (g.mut_node[m] != INVALID_NODE) {
            plan.mut_new[m] = o2n[g.mut_node[m]];
            pairs.emplace_back(plan.mut_new[m], static_cast<uint32_t>(m));
        }
    }
    std::sort(pairs.begin(), pairs.end());
    single_level_csr(plan.seed, pairs);
    plan.has_miss = !g.miss_node.empty();
    plan.miss_new.assign(g.num_mutations, INVALID_NODE);
    pairs.clear();
    if (plan.has_miss) {
        for (uint64_t m = 0; m < g.num_mutations; m++) {
            if (g.miss_node[m] != INVALID_NODE) {
                plan.miss_new[m] = o2n[g.miss_node[m]];
                pairs.emplace_back(plan.miss_new[m], static_cast<uint32_t>(m));
            }
        }
        std::sort(pairs.begin(), pairs.end());
    }
    single_level_csr(plan.miss, pairs);

    // xtx init values by new id
    plan.xtx_new.assign(n, 0);
    plan.has_coals = true;
    for (uint64_t id = 0; id < n; id++) {
        const uint32_t old = n2o[id];
        uint32_t c = 0;
        if (old >= N) {
            const uint64_t idx = old - N;
            c = (idx < g.coals.size()) ? g.coals[idx] : COAL_NOT_SET;
        }
        if (c == COAL_NOT_SET) {
            plan.has_coals = false;
            plan.xtx_new[id] = COAL_NOT_SET;
        } else {
            plan.xtx_new[id] = c * 2u;
        }
    }
}

std::unique_ptr<HostPlan> build_plan(const HostGraph& g) {
    PhaseTimer timer{"plan"};
    const uint64_t n = g.num_nodes, N = g.num_samples;
    GRGX_CHECK(n <= MAX_NODES, GRGX_ERR_UNSUPPORTED, "too many nodes");
    auto plan = std::make_unique<HostPlan>();

    // ---- heights -------------------------------------------------------------------------
    std::vector<uint32_t> height(n, 0);
    bool ordered = true;
    for (uint64_t v = 0; v < n && ordered; v++)
        for (uint64_t e = g.down_off[v]; e < g.down_off[v + 1]; e++)
            if (g.down_adj[e] >= v) {
                ordered = false;
                break;
            }
    if (ordered) {
        for (uint64_t v = 0; v < n; v++) {
            uint32_t h = 0;
            for (uint64_t e = g.down_off[v]; e < g.down_off[v + 1]; e++) h = std::max(h, height[g.down_adj[e]] + 1);
            height[v] = h;
        }
    } else {
        // Kahn order over parents (children first).
        std::vector<uint32_t> pending(n), order;
        std::vector<uint64_t> upOff(n + 1, 0);
        for (uint64_t e = 0; e < g.num_edges(); e++) upOff[g.down_adj[e] + 1]++;
        for (uint64_t v = 0; v < n; v++) upOff[v + 1] += upOff[v];
        std::vector<uint32_t> upAdj(g.num_edges());
        std::vector<uint64_t> fill(upOff.begin(), upOff.end() - 1);
        for (uint64_t v = 0; v < n; v++) {
            pending[v] = static_cast<uint32_t>(g.down_off[v + 1] - g.down_off[v]);
            for (uint64_t e = g.down_off[v]; e < g.down_off[v + 1]; e++) upAdj[fill[g.down_adj[e]]++] = v;
        }
        order.reserve(n);
        for (uint64_t v = 0; v < n; v++)
            if (!pending[v]) order.push_back(v);
        for (size_t i = 0; i < order.size(); i++) {
            const uint32_t v = order[i];
            for (uint64_t e = upOff[v]; e < upOff[v + 1]; e++)
                if (--pending[upAdj[e]] == 0) order.push_back(upAdj[e]);
        }
        GRGX_CHECK(order.size() == n, GRGX_ERR_API_MISUSE, "GRG contains a cycle");
        for (uint32_t v : order) {
            uint32_t h = 0;
            for (uint64_t e = g.down_off[v]; e < g.down_off[v + 1]; e++) h = std::max(h, height[g.down_adj[e]] + 1);
            height[v] = h;
        }
    }
    timer.lap("heights");
    for (uint64_t s = 0; s < N; s++)
        GRGX_CHECK(height[s] == 0, GRGX_ERR_UNSUPPORTED, "sample nodes with children are not supported");
    uint32_t maxH = 0;
    for (uint64_t v = 0; v < n; v++) maxH = std::max(maxH, height[v]);
    const uint64_t L = (n == 0) ? 0 : maxH + 1;

    // ---- renumbering (stable counting sort by height) ---------------------------------------
    std::vector<uint64_t> perHeight(L, 0);
    for (uint64_t v = 0; v < n; v++) perHeight[height[v]]++;
    plan_levels_from_counts(*plan, perHeight);
    plan->old2new.resize(n);
    plan->new2old.resize(n);
    {
        std::vector<uint64_t> next(plan->level_begin.begin(), plan->level_begin.end());
        for (uint64_t v = 0; v < n; v++) {
            const uint64_t id = next[height[v]]++;
            plan->old2new[v] = static_cast<uint32_t>(id);
            plan->new2old[id] = static_cast<uint32_t>(v);
        }
    }
    const auto& o2n = plan->old2new;
    const auto& n2o = plan->new2old;

    timer.lap("renumber");
    // ---- UP: rows = every node of heights 1..H, children in stored order --------------------
    {
        PullCSR& P = plan->up;
        const uint64_t r0 = L > 1 ? plan->level_begin[1] : n;
        const uint64_t R = n - r0;
        std::vector<int64_t> off(R + 1, 0);
        for (uint64_t i = 0; i < R; i++) {
            const uint32_t old = n2o[r0 + i];
            off[i + 1] = off[i] + static_cast<int64_t>(g.down_off[old + 1] - g.down_off[old]);
        }
        P.adj.resize(off[R]);
        parallel_for(R, [&](uint64_t b, uint64_t e, int) {
            for (uint64_t i = b; i < e; i++) {
                const uint32_t old = n2o[r0 + i];
                int64_t w = off[i];
                for (uint64_t x = g.down_off[old]; x < g.down_off[old + 1]; x++)
                    P.adj[w++] = o2n[g.down_adj[x]] | (x == g.down_off[old] ? HEAD_BIT : 0u);
            }
        });
        plan_up_layout(*plan, std::move(off));
    }

    timer.lap("up csr");
    // ---- DOWN: rows = nodes with parents, heights H..0, parents ascending by new id ---------
    // The host counts parents per node (parallel, per-thread counters) to lay out rows, offsets
    // and chunks; the adjacency itself is built on the device from the UP CSR (plan_gpu.cu).
    {
        const int T = (g.num_edges() < (1u << 20)) ? 1 : host_threads();
        // parent ranges balanced by edge count
        std::vector<uint64_t> pb(T + 1, 0);
        {
            std::vector<uint64_t> cum(n + 1, 0);
            for (uint64_t pid = 0; pid < n; pid++) {
                const uint32_t old = n2o[pid];
                cum[pid + 1] = cum[pid] + (g.down_off[old + 1] - g.down_off[old]);
            }
            for (int t = 1; t < T; t++)
                pb[t] = static_cast<uint64_t>(std::lower_bound(cum.begin(), cum.end(), cum[n] * t / T) - cum.begin());
            pb[T] = n;
        }
        std::vector<std::vector<uint32_t>> cnt(T, std::vector<uint32_t>(n, 0));
        parallel_for(T, [&](uint64_t b, uint64_t e, int) {
            for (uint64_t t = b; t < e; t++) {
                std::vector<uint32_t>& c = cnt[t];
                for (uint64_t pid = pb[t]; pid < pb[t + 1]; pid++) {
                    const uint32_t old = n2o[pid];
                    for (uint64_t x = g.down_off[old]; x < g.down_off[old + 1]; x++) c[o2n[g.down_adj[x]]]++;
                }
            }
        }, T);
        timer.lap("down.count");
        std::vector<uint64_t> pdeg(n, 0);
        parallel_for(n, [&](uint64_t b, uint64_t e, int) {
            for (uint64_t c = b; c < e; c++) {
                uint64_t d = 0;
                for (int t = 0; t < T; t++) d += cnt[t][c];
                pdeg[c] = d;
            }
        });
        plan_down_layout(*plan, pdeg);
    }

    timer.lap("down csr");
    plan_seeds(*plan, g);
    timer.lap("seeds/xtx");
    return plan;
}

}  // namespace grgx
