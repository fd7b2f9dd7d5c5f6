// Launch-shape autotuner for the level sweep.
//
// A level's sweep can run with G lanes per row (G = the default for the row's K, half or a
// quarter of it -- fewer lanes per row means more rows per warp and more column tiles) and with
// the default or the deep prefetch variant (twice the gathers in flight per lane, one block per
// SM less).  Which is fastest depends on the level's width (rows), its mean degree (edges per
// row) and K, so the table is keyed on
//     (storage kind, row stride in elements, floor(log2(rows + 1)), floor(log2(edges / rows + 1)))
// and filled by measuring: grgx_autotune times candidates on each level of one traversal of a
// resident graph (CUDA events around the level's launch, best of two after a warm launch) --
// the deep variant at the default lanes, then halvings of the lanes per row while each keeps
// winning -- and records the winner when it beats the default by more than 2%.  Levels with
// under 0.5% of the traversal's edges keep the default.  For UP on graphs where the split form
// (up_split.cu) is possible it tunes both forms and records, for this graph and (storage kind,
// stride), the one whose tuned sweep is faster.  Calls on any graph then look up every
// level's key; levels without an entry run the default shape.  Shapes change only the order in
// which a row's float terms are added (integer results are bit-exact with any shape).
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cstdio>
#include <map>
#include <mutex>
#include <sstream>
#include <string>
#include <tuple>
#include <vector>

#include "device_plan.h"

namespace grgx {

namespace {

using Key = std::tuple<int, long long, int, int>;

std::mutex g_table_mu;
std::map<Key, LevelShape> g_table;
std::atomic<bool> g_table_nonempty{false};

int ilog2p1(long long x) {
    int l = 0;
    for (unsigned long long v = static_cast<unsigned long long>(x) + 1; v > 1; v >>= 1) l++;
    return l;
}

Key key_for(const Layout& L, long long rows, long long edges) {
    return Key{static_cast<int>(L.kind), L.stride, ilog2p1(rows), ilog2p1(rows > 0 ? edges / rows : 0)};
}

bool has_deep(const Layout& L) {
    const bool kindOk = L.kind == Kind::U32 || L.kind == Kind::F32C || L.kind == Kind::F32 || L.kind == Kind::F64S;
    return kindOk && L.vw * L.ssize == 16;
}

int tiles_for(const Layout& L, int g) {
    const long long vecs = L.stride / L.vw;
    return static_cast<int>((vecs + g - 1) / g);
}

// Candidate lane counts: the default and up to two halvings (each a compiled shape).
std::vector<int> candidate_g(const Layout& L) {
    std::vector<int> gs{L.g};
    if (L.vw * L.ssize == 16) {
        for (int g = L.g / 2; g >= 1 && gs.size() < 3; g /= 2) gs.push_back(g);
    }
    return gs;
}

bool valid_shape(const Layout& L, const LevelShape& s) {
    if (s.variant != 0 && !has_deep(L)) return false;
    const std::vector<int> gs = candidate_g(L);
    return std::find(gs.begin(), gs.end(), s.g) != gs.end() && s.ntiles == tiles_for(L, s.g);
}

}  // namespace

LevelShape default_shape(const Layout& L) { return LevelShape{L.g, L.ntiles, 0}; }

int max_tiles(const Layout& L) {
    int t = L.ntiles;
    for (int g : candidate_g(L)) t = std::max(t, tiles_for(L, g));
    return t;
}

LevelShape level_shape(const Layout& L, const DevCSR& c, size_t level) {
    if (!g_table_nonempty.load(std::memory_order_acquire) || level >= c.level_rows.size()) return default_shape(L);
    std::lock_guard<std::mutex> lk(g_table_mu);
    auto it = g_table.find(key_for(L, c.level_rows[level], c.level_edges[level]));
    if (it == g_table.end() || !valid_shape(L, it->second)) return default_shape(L);
    return it->second;
}

void autotune_clear() {
    std::lock_guard<std::mutex> lk(g_table_mu);
    g_table.clear();
    g_table_nonempty.store(false, std::memory_order_release);
}

// One line per entry: kind stride rows_log2 degree_log2 g ntiles variant.
std::string autotune_export() {
    std::lock_guard<std::mutex> lk(g_table_mu);
    std::ostringstream os;
    for (const auto& kv : g_table)
        os << std::get<0>(kv.first) << ' ' << std::get<1>(kv.first) << ' ' << std::get<2>(kv.first) << ' '
           << std::get<3>(kv.first) << ' ' << kv.second.g << ' ' << kv.second.ntiles << ' ' << kv.second.variant
           << '\n';
    return os.str();
}

void autotune_import(const std::string& text) {
    std::istringstream is(text);
    std::vector<std::pair<Key, LevelShape>> rows;
    std::string line;
    while (std::getline(is, line)) {
        if (line.empty()) continue;
        std::istringstream ls(line);
        int kind = 0, rl = 0, dl = 0;
        long long stride = 0;
        LevelShape s;
        GRGX_CHECK(static_cast<bool>(ls >> kind >> stride >> rl >> dl >> s.g >> s.ntiles >> s.variant), GRGX_ERR_API_MISUSE,
                   "malformed autotune table line: " + line);
        GRGX_CHECK(kind >= 0 && kind <= static_cast<int>(Kind::F64S) && stride > 0 && s.g >= 1 && s.g <= 32 &&
                       (s.g & (s.g - 1)) == 0 && s.ntiles >= 1 && (s.variant == 0 || s.variant == 1),
                   GRGX_ERR_API_MISUSE, "invalid autotune table entry: " + line);
        rows.push_back({Key{kind, stride, rl, dl}, s});
    }
    std::lock_guard<std::mutex> lk(g_table_mu);
    for (auto& r : rows) g_table[r.first] = r.second;
    g_table_nonempty.store(!g_table.empty(), std::memory_order_release);
}

void clear_graph_replays(grgx_graph* g);

// Times the candidate shapes on each level of one traversal in `direction` and records the
// winners.  The values swept are zeros: the gathers, the edge walk and the arithmetic do not
// depend on them.
std::string autotune_impl(grgx_graph* g, int dtype, uint64_t rows, int direction, uint32_t flags) {
    GRGX_CHECK(dtype >= GRGX_F64 && dtype <= GRGX_BOOL, GRGX_ERR_API_MISUSE, "Unsupported dtype");
    GRGX_CHECK(direction == GRGX_DIRECTION_DOWN || direction == GRGX_DIRECTION_UP, GRGX_ERR_API_MISUSE,
               "Invalid traversal direction");
    GRGX_CHECK(rows > 0 && rows <= 2000000ull, GRGX_ERR_API_MISUSE, "matmul() requires non-zero dimensions.");
    DevicePlan* dp = ensure_device_plan(g);
    const Layout L = choose_layout(dtype, static_cast<long long>(rows), (flags & GRGX_FLAG_F32_PLAIN) != 0,
                                   (flags & GRGX_FLAG_F64_NATIVE) != 0);
    const bool down = (direction == GRGX_DIRECTION_DOWN);
    // the CSRs a call of this shape sweeps; for UP both forms when the split form is possible,
    // so the faster one is recorded for this graph
    // (for DOWN too: the height-0 level in parent blocks, the levels above it as usual)
    struct Pass {
        const DevCSR* c;
        int mode;
        const char* name;
        long long stateBase;
        bool skipLast;  // the CSR's last level is left to the next pass
    };
    std::vector<std::vector<Pass>> forms;
    const long long h0 = static_cast<long long>(dp->level_begin.size() > 1 ? dp->level_begin[1] : 0);
    // (on the chunking calls of this row width run on)
    if (down) {
        if (down_split_possible(dp)) ensure_down_split(g, dp);
        const SweepCSRs cs = sweep_csrs(dp, L);
        forms.push_back({{cs.down, 0, "level", 0, false}});
        if (cs.down0b->n_rows > 0)
            forms.push_back({{cs.down, 0, "split: level", 0, true},
                             {cs.down0b, 1, "split: height-0 parent block", 0, false}});
    } else {
        if (up_split_possible(dp)) ensure_up_split(g, dp);
        const SweepCSRs cs = sweep_csrs(dp, L);
        forms.push_back({{cs.up, 0, "level", 0, false}});
        if (cs.up0b->n_rows > 0)
            forms.push_back({{cs.up0b, 1, "split: height-0 block", dp->split_src, false},
                             {cs.up_int, 2, "split: level", dp->split_src, false}});
    }
    long long maxPieces = 0, maxHeavy = 0;
    for (const auto& f : forms)
        for (const Pass& ps : f) {
            maxPieces = std::max(maxPieces, ps.c->n_pieces);
            maxHeavy = std::max(maxHeavy, ps.c->n_heavy);
        }
    const bool needState = forms.size() > 1;
    const int maxT = max_tiles(L);
    const size_t n = g->host->num_nodes;
    cudaStream_t s = nullptr;
    GRGX_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    void *vals = nullptr, *partials = nullptr, *state = nullptr;
    unsigned* counters = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    std::ostringstream rep;
    auto release = [&] {
        if (vals) cudaFree(vals);
        if (partials) cudaFree(partials);
        if (state) cudaFree(state);
        if (counters) cudaFree(counters);
        if (e0) cudaEventDestroy(e0);
        if (e1) cudaEventDestroy(e1);
        cudaStreamDestroy(s);
    };
    try {
        const size_t valBytes = n * static_cast<size_t>(L.stride) * L.ssize;
        GRGX_CUDA(cudaMalloc(&vals, std::max<size_t>(valBytes, 16)));
        GRGX_CUDA(cudaMemsetAsync(vals, 0, valBytes, s));
        GRGX_CUDA(cudaMalloc(&partials, std::max<size_t>(static_cast<size_t>(maxPieces) * L.stride * L.asize, 16)));
        if (needState) {
            const size_t stateRows = down ? static_cast<size_t>(h0) : n - static_cast<size_t>(dp->split_src);
            const size_t stateBytes = stateRows * L.stride * std::max(L.asize, 8);
            GRGX_CUDA(cudaMalloc(&state, std::max<size_t>(stateBytes, 16)));
            GRGX_CUDA(cudaMemsetAsync(state, 0, stateBytes, s));
        }
        const size_t counterBytes = static_cast<size_t>(maxHeavy + 1) * maxT * sizeof(unsigned);
        GRGX_CUDA(cudaMalloc(&counters, counterBytes));
        GRGX_CUDA(cudaEventCreate(&e0));
        GRGX_CUDA(cudaEventCreate(&e1));
        unsigned* tickets = counters;
        unsigned* work = counters + maxHeavy * maxT;
        const int rmw = down ? 1 : 0;
        const DevCSR* cur = nullptr;
        int curMode = 0;
        long long curBase = 0;
        auto time_shape = [&](size_t lvl, const LevelShape& sh) {
            float best = 1e30f;
            for (int rep_i = 0; rep_i < 3; rep_i++) {
                GRGX_CUDA(cudaMemsetAsync(counters, 0, counterBytes, s));
                GRGX_CUDA(cudaEventRecord(e0, s));
                launch_level(L, *cur, lvl, vals, vals, curMode == 1 ? 0 : rmw, partials, tickets, work, s, nullptr, 0,
                             &sh, maxT, curMode ? state : nullptr, curBase, curMode ? curMode : 1);
                GRGX_CUDA(cudaEventRecord(e1, s));
                GRGX_CUDA(cudaEventSynchronize(e1));
                GRGX_CUDA(cudaGetLastError());
                float ms = 0;
                GRGX_CUDA(cudaEventElapsedTime(&ms, e0, e1));
                if (rep_i > 0) best = std::min(best, ms);  // the first launch warms up
            }
            return best;
        };
        const std::vector<int> gs = candidate_g(L);
        std::vector<double> formBest;
        for (const auto& form : forms) {
            long long totalEdges = 0;
            for (const Pass& ps : form) totalEdges += ps.c->n_edges;
            double totDefault = 0, totBest = 0;
            for (const Pass& ps : form) {
                cur = ps.c;
                curMode = ps.mode;
                curBase = ps.stateBase;
                const DevCSR& c = *ps.c;
                for (size_t lvl = 0; lvl + (ps.skipLast ? 1 : 0) < c.lb.size(); lvl++) {
                    if (c.le[lvl] <= c.lb[lvl]) continue;
                    const LevelShape def = default_shape(L);
                    const float tDef = time_shape(lvl, def);
                    totDefault += tDef;
                    // levels under 0.5% of the traversal's edges keep the default
                    if (c.level_edges[lvl] * 200 < totalEdges) {
                        totBest += tDef;
                        continue;
                    }
                    LevelShape best = def;
                    float tBest = tDef;
                    // greedy: the deep variant at the default lanes, then fewer lanes per row with
                    // the better variant while each halving keeps winning by 2%
                    if (has_deep(L)) {
                        const LevelShape deep{def.g, def.ntiles, 1};
                        const float t = time_shape(lvl, deep);
                        if (t < 0.98f * tBest) {
                            tBest = t;
                            best = deep;
                        }
                    }
                    for (size_t i = 1; i < gs.size(); i++) {
                        const LevelShape sh{gs[i], tiles_for(L, gs[i]), best.variant};
                        const float t = time_shape(lvl, sh);
                        if (!(t < 0.98f * tBest)) break;
                        tBest = t;
                        best = sh;
                    }
                    totBest += tBest;
                    {
                        std::lock_guard<std::mutex> lk(g_table_mu);
                        g_table[key_for(L, c.level_rows[lvl], c.level_edges[lvl])] = best;
                        g_table_nonempty.store(true, std::memory_order_release);
                    }
                    char line[256];
                    std::snprintf(line, sizeof(line),
                                  "%s %zu rows %lld edges %lld: g %d tiles %d variant %d, %.4f ms (default g %d "
                                  "variant 0: %.4f ms)\n",
                                  ps.name, lvl, c.level_rows[lvl], c.level_edges[lvl], best.g, best.ntiles,
                                  best.variant, tBest, def.g, tDef);
                    rep << line;
                }
            }
            char tail[160];
            const bool splitForm = (&form != &forms[0]);
            std::snprintf(tail, sizeof(tail), "%s %.4f ms tuned, %.4f ms default\n",
                          forms.size() > 1 ? (splitForm ? "split sweep" : "unsplit sweep") : "sweep", totBest,
                          totDefault);
            rep << tail;
            formBest.push_back(totBest);
        }
        if (forms.size() > 1) {
            const bool split = formBest[1] < 0.98 * formBest[0];
            if (down) {
                set_down_split_choice(g, dp, L, split);
                rep << (split ? "DOWN runs in split form for this shape\n" : "DOWN runs unsplit for this shape\n");
            } else {
                set_up_split_choice(g, dp, L, split);
                rep << (split ? "UP runs in split form for this shape\n" : "UP runs unsplit for this shape\n");
            }
        }
    } catch (...) {
        release();
        throw;
    }
    release();
    clear_graph_replays(g);
    return rep.str();
}

}  // namespace grgx
