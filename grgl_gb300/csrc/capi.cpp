// The C ABI (include/grgx.h): exception-free wrappers over the host graph, the plan and the
// matmul orchestration.
#include <algorithm>
#include <cstring>
#include <string>

#include "grgx_internal.h"

namespace grgx {
DevicePlan* ensure_device_plan(grgx_graph* g);
uint64_t device_plan_bytes(const grgx_graph* g);
uint64_t device_plan_levels(const grgx_graph* g);
void matmul_impl(grgx_graph* g, int dtype, const void* input, uint64_t in_cols, uint64_t rows, int direction,
                 void* output, uint64_t output_size, int emit_all, int by_indiv, const void* init, int init_kind,
                 void* miss, uint32_t flags, void* stream);
void set_timing(int enabled);
grgx_timing last_timing();
std::vector<grgx_timing> collect_timings();
double measure_l2_bandwidth(uint64_t bytes, int reps);
void pool_usage(int device, uint64_t* used, uint64_t* reserved);
void matmul_noalloc_impl(grgx_graph* g, int dtype, const void* input, uint64_t in_cols, uint64_t rows, int direction,
                         void* output, uint64_t output_size, void* stream);
void matmul_batch_impl(grgx_graph* g, const grgx_request* reqs, uint64_t n, uint64_t maxCols, uint32_t flags,
                       void* stream);
void matmul_standardized_impl(grgx_graph* g, int dtype, const void* input, uint64_t in_cols, uint64_t rows,
                              int direction, void* output, uint64_t output_size, uint32_t flags, void* stream);
void matmul_gram_impl(grgx_graph* g, int dtype, const void* input, uint64_t in_cols, uint64_t rows, int first,
                      void* output, uint64_t output_size, int standardized, uint32_t flags, void* stream);
void set_up_split(long long block, unsigned long long thresholdBytes);
void set_down_split_mode(int mode);
void set_staged(bool on);
void* host_alloc(uint64_t bytes);
void host_free(void* b);
std::string autotune_impl(grgx_graph* g, int dtype, uint64_t rows, int direction, uint32_t flags);
std::string autotune_export();
void autotune_import(const std::string& text);
void autotune_clear();

namespace {
thread_local std::string t_error;

template <typename F> grgx_status guarded(F&& f) {
    try {
        f();
        t_error.clear();
        return GRGX_OK;
    } catch (const Error& e) {
        t_error = e.what();
        return static_cast<grgx_status>(e.code);
    } catch (const std::bad_alloc&) {
        t_error = "host out of memory";
        return GRGX_ERR_OUT_OF_MEMORY;
    } catch (const std::exception& e) {
        t_error = e.what();
        return GRGX_ERR_CUDA;
    }
}

uint64_t count_levels(const HostGraph& g) {
    // Heights without building the plan (ordered graphs: one pass).
    std::vector<uint32_t> h(g.num_nodes, 0);
    uint32_t mx = 0;
    for (uint64_t v = 0; v < g.num_nodes; v++) {
        uint32_t x = 0;
        for (uint64_t e = g.down_off[v]; e < g.down_off[v + 1]; e++) {
            const uint32_t c = g.down_adj[e];
            if (c >= v) return 0;  // not ordered: unknown until the plan is built
            x = std::max(x, h[c] + 1);
        }
        h[v] = x;
        mx = std::max(mx, x);
    }
    return g.num_nodes ? mx + 1 : 0;
}
}  // namespace

void set_last_error(const std::string& msg) { t_error = msg; }

}  // namespace grgx

using namespace grgx;

extern "C" {

const char* grgx_last_error(void) { return t_error.c_str(); }

const char* grgx_version(void) { return "grgx 0.1 (sm_103a)"; }

grgx_status grgx_graph_load(const char* path, grgx_graph** out) {
    return guarded([&] {
        GRGX_CHECK(path && out, GRGX_ERR_API_MISUSE, "null argument");
        auto g = new grgx_graph();
        try {
            g->host = load_grg_file(path);
        } catch (...) {
            delete g;
            throw;
        }
        *out = g;
    });
}

grgx_status grgx_graph_from_csr(uint64_t num_nodes, uint64_t num_samples, uint64_t ploidy, const uint64_t* down_off,
                                const uint32_t* down_adj, uint64_t num_mutations, const uint32_t* mut_node,
                                const uint32_t* miss_node, const uint32_t* coals, grgx_graph** out) {
    return guarded([&] {
        GRGX_CHECK(out && down_off && (num_mutations == 0 || mut_node), GRGX_ERR_API_MISUSE, "null argument");
        GRGX_CHECK(num_nodes <= MAX_NODES && num_samples <= num_nodes, GRGX_ERR_API_MISUSE, "invalid node counts");
        GRGX_CHECK(ploidy > 0, GRGX_ERR_API_MISUSE, "ploidy must be positive");
        auto h = std::make_unique<HostGraph>();
        h->num_nodes = num_nodes;
        h->num_samples = num_samples;
        h->ploidy = ploidy;
        h->num_mutations = num_mutations;
        h->down_off.assign(down_off, down_off + num_nodes + 1);
        GRGX_CHECK(h->down_off[0] == 0, GRGX_ERR_API_MISUSE, "down_off[0] must be 0");
        for (uint64_t v = 0; v < num_nodes; v++)
            GRGX_CHECK(h->down_off[v + 1] >= h->down_off[v], GRGX_ERR_API_MISUSE, "down_off must be nondecreasing");
        const uint64_t E = h->down_off[num_nodes];
        GRGX_CHECK(E == 0 || down_adj, GRGX_ERR_API_MISUSE, "null argument");
        h->down_adj.assign(down_adj, down_adj + E);
        for (uint32_t c : h->down_adj) GRGX_CHECK(c < num_nodes, GRGX_ERR_API_MISUSE, "edge target out of range");
        h->mut_node.assign(mut_node, mut_node + num_mutations);
        for (uint32_t m : h->mut_node)
            GRGX_CHECK(m == INVALID_NODE || m < num_nodes, GRGX_ERR_API_MISUSE, "mutation node out of range");
        if (miss_node) {
            h->miss_node.assign(miss_node, miss_node + num_mutations);
            for (uint32_t m : h->miss_node)
                GRGX_CHECK(m == INVALID_NODE || m < num_nodes, GRGX_ERR_API_MISUSE, "missingness node out of range");
        }
        if (coals) h->coals.assign(coals, coals + (num_nodes - num_samples));
        auto g = new grgx_graph();
        g->host = std::move(h);
        *out = g;
    });
}

grgx_status grgx_graph_generate(uint64_t num_samples, uint64_t num_mutations, uint64_t seed, uint32_t window,
                                int threads, grgx_graph** out) {
    return guarded([&] {
        GRGX_CHECK(out && num_samples >= 2 && window >= 1, GRGX_ERR_API_MISUSE, "invalid generator arguments");
        auto g = new grgx_graph();
        try {
            g->host = generate_window_tree(num_samples, num_mutations, seed, window, threads);
        } catch (...) {
            delete g;
            throw;
        }
        *out = g;
    });
}

grgx_status grgx_graph_subset(const grgx_graph* g, const uint32_t* mutation_ids, uint64_t n, grgx_graph** out) {
    return guarded([&] {
        GRGX_CHECK(g && out && (n == 0 || mutation_ids), GRGX_ERR_API_MISUSE, "null argument");
        const HostGraph& h = const_cast<grgx_graph*>(g)->host_edges();
        std::vector<uint8_t> keep(h.num_nodes, 0);
        for (uint64_t s = 0; s < h.num_samples; s++) keep[s] = 1;
        std::vector<uint32_t> stack;
        auto seed = [&](uint32_t v) {
            if (v != INVALID_NODE && !keep[v]) {
                keep[v] = 1;
                stack.push_back(v);
            }
        };
        for (uint64_t i = 0; i < n; i++) {
            GRGX_CHECK(mutation_ids[i] < h.num_mutations, GRGX_ERR_API_MISUSE,
                       "Invalid MutationID: " + std::to_string(mutation_ids[i]));
            seed(h.mut_node[mutation_ids[i]]);
            if (!h.miss_node.empty()) seed(h.miss_node[mutation_ids[i]]);
        }
        while (!stack.empty()) {
            const uint32_t v = stack.back();
            stack.pop_back();
            for (uint64_t e = h.down_off[v]; e < h.down_off[v + 1]; e++) seed(h.down_adj[e]);
        }
        std::vector<uint32_t> remap(h.num_nodes, INVALID_NODE);
        uint64_t cnt = 0;
        for (uint64_t v = 0; v < h.num_nodes; v++)
            if (keep[v]) remap[v] = static_cast<uint32_t>(cnt++);
        auto sub = std::make_unique<HostGraph>();
        sub->num_nodes = cnt;
        sub->num_samples = h.num_samples;
        sub->ploidy = h.ploidy;
        sub->phased = h.phased;
        sub->num_mutations = n;
        sub->down_off.assign(1, 0);
        for (uint64_t v = 0; v < h.num_nodes; v++) {
            if (!keep[v]) continue;
            for (uint64_t e = h.down_off[v]; e < h.down_off[v + 1]; e++) sub->down_adj.push_back(remap[h.down_adj[e]]);
            sub->down_off.push_back(sub->down_adj.size());
        }
        sub->mut_node.resize(n);
        for (uint64_t i = 0; i < n; i++) {
            const uint32_t v = h.mut_node[mutation_ids[i]];
            sub->mut_node[i] = (v == INVALID_NODE) ? INVALID_NODE : remap[v];
        }
        if (!h.miss_node.empty()) {
            sub->miss_node.resize(n);
            for (uint64_t i = 0; i < n; i++) {
                const uint32_t v = h.miss_node[mutation_ids[i]];
                sub->miss_node[i] = (v == INVALID_NODE) ? INVALID_NODE : remap[v];
            }
        }
        if (!h.coals.empty()) {
            for (uint64_t v = h.num_samples; v < h.num_nodes; v++)
                if (keep[v]) sub->coals.push_back(v - h.num_samples < h.coals.size() ? h.coals[v - h.num_samples]
                                                                                    : COAL_NOT_SET);
        }
        if (!h.mut_pos.empty())
            for (uint64_t i = 0; i < n; i++) sub->mut_pos.push_back(h.mut_pos[mutation_ids[i]]);
        auto gg = new grgx_graph();
        gg->host = std::move(sub);
        *out = gg;
    });
}

grgx_status grgx_graph_save(const grgx_graph* g, const char* path) {
    return guarded([&] {
        GRGX_CHECK(g && path, GRGX_ERR_API_MISUSE, "null argument");
        save_grg_file(const_cast<grgx_graph*>(g)->host_edges(), path);
    });
}

void grgx_graph_destroy(grgx_graph* g) {
    if (!g) return;
    try {
        delete g;
    } catch (...) {
    }
}

grgx_status grgx_graph_info_get(const grgx_graph* g, grgx_graph_info* out) {
    return guarded([&] {
        GRGX_CHECK(g && out, GRGX_ERR_API_MISUSE, "null argument");
        const HostGraph& h = *g->host;
        std::memset(out, 0, sizeof(*out));
        out->num_nodes = h.num_nodes;
        out->num_edges = h.num_edges();
        out->num_samples = h.num_samples;
        out->num_mutations = h.num_mutations;
        out->ploidy = h.ploidy;
        // an encoded graph's levels are known once its plan is built
        out->num_levels = g->dev ? device_plan_levels(g) : (h.encoded() ? 0 : count_levels(h));
        out->has_missing = h.miss_node.empty() ? 0 : 1;
        bool coals = h.coals.size() >= h.num_nodes - h.num_samples;
        for (uint64_t i = 0; coals && i < h.num_nodes - h.num_samples; i++) coals = (h.coals[i] != COAL_NOT_SET);
        out->has_coals = coals ? 1 : 0;
        out->device_bytes = device_plan_bytes(g);
    });
}

grgx_status grgx_graph_export(const grgx_graph* g, uint64_t* down_off, uint32_t* down_adj, uint32_t* mut_node,
                              uint32_t* miss_node, uint32_t* coals) {
    return guarded([&] {
        GRGX_CHECK(g, GRGX_ERR_API_MISUSE, "null argument");
        const HostGraph& h = (down_off || down_adj) ? const_cast<grgx_graph*>(g)->host_edges() : *g->host;
        if (down_off) std::memcpy(down_off, h.down_off.data(), h.down_off.size() * sizeof(uint64_t));
        if (down_adj && !h.down_adj.empty())
            std::memcpy(down_adj, h.down_adj.data(), h.down_adj.size() * sizeof(uint32_t));
        if (mut_node && !h.mut_node.empty())
            std::memcpy(mut_node, h.mut_node.data(), h.mut_node.size() * sizeof(uint32_t));
        if (miss_node) {
            for (uint64_t m = 0; m < h.num_mutations; m++)
                miss_node[m] = h.miss_node.empty() ? INVALID_NODE : h.miss_node[m];
        }
        if (coals) {
            for (uint64_t i = 0; i < h.num_nodes - h.num_samples; i++)
                coals[i] = (i < h.coals.size()) ? h.coals[i] : COAL_NOT_SET;
        }
    });
}

grgx_status grgx_graph_upload(grgx_graph* g) {
    return guarded([&] {
        GRGX_CHECK(g, GRGX_ERR_API_MISUSE, "null argument");
        ensure_device_plan(g);
    });
}

grgx_status grgx_matmul(grgx_graph* g, grgx_dtype dtype, const void* input, uint64_t input_cols, uint64_t input_rows,
                        grgx_direction direction, void* output, uint64_t output_size, int emit_all_nodes,
                        int by_individual, const void* init, grgx_init init_kind, void* miss, uint32_t flags,
                        void* stream) {
    return guarded([&] {
        GRGX_CHECK(g && input && output, GRGX_ERR_API_MISUSE, "null argument");
        matmul_impl(g, dtype, input, input_cols, input_rows, direction, output, output_size, emit_all_nodes,
                    by_individual, init, init_kind, miss, flags, stream);
    });
}

grgx_status grgx_matmul_standardized(grgx_graph* g, grgx_dtype dtype, const void* input, uint64_t input_cols,
                                     uint64_t input_rows, grgx_direction direction, void* output,
                                     uint64_t output_size, uint32_t flags, void* stream) {
    return guarded([&] {
        GRGX_CHECK(g && input && output, GRGX_ERR_API_MISUSE, "null argument");
        matmul_standardized_impl(g, dtype, input, input_cols, input_rows, direction, output, output_size, flags,
                                 stream);
    });
}

grgx_status grgx_matmul_batch(grgx_graph* g, const grgx_request* requests, uint64_t n, uint64_t max_cols,
                              uint32_t flags, void* stream) {
    return guarded([&] {
        GRGX_CHECK(g, GRGX_ERR_API_MISUSE, "null argument");
        matmul_batch_impl(g, requests, n, max_cols, flags, stream);
    });
}

grgx_status grgx_matmul_noalloc(grgx_graph* g, grgx_dtype dtype, const void* input, uint64_t input_cols,
                                uint64_t input_rows, grgx_direction direction, void* output, uint64_t output_size,
                                void* stream) {
    return guarded([&] {
        GRGX_CHECK(g && input && output, GRGX_ERR_API_MISUSE, "null argument");
        matmul_noalloc_impl(g, dtype, input, input_cols, input_rows, direction, output, output_size, stream);
    });
}

grgx_status grgx_pool_usage(int device, uint64_t* used, uint64_t* reserved) {
    return guarded([&] { pool_usage(device, used, reserved); });
}

grgx_status grgx_measure_l2_bandwidth(uint64_t bytes, int reps, double* gbps) {
    return guarded([&] {
        GRGX_CHECK(gbps, GRGX_ERR_API_MISUSE, "null argument");
        *gbps = measure_l2_bandwidth(bytes, reps);
    });
}

namespace {
// Copies `text` (NUL-terminated, truncated to `len`) and reports the size it needs.
void copy_text(const std::string& text, char* buf, uint64_t len, uint64_t* needed) {
    if (needed) *needed = text.size() + 1;
    if (buf && len > 0) {
        const size_t k = std::min<size_t>(text.size(), static_cast<size_t>(len - 1));
        std::memcpy(buf, text.data(), k);
        buf[k] = '\0';
    }
}
}  // namespace

grgx_status grgx_autotune(grgx_graph* g, grgx_dtype dtype, uint64_t rows, grgx_direction direction, uint32_t flags,
                          char* report, uint64_t report_len, uint64_t* report_needed) {
    return guarded([&] {
        GRGX_CHECK(g, GRGX_ERR_API_MISUSE, "null argument");
        copy_text(autotune_impl(g, dtype, rows, direction, flags), report, report_len, report_needed);
    });
}

grgx_status grgx_autotune_export(char* buf, uint64_t len, uint64_t* needed) {
    return guarded([&] { copy_text(autotune_export(), buf, len, needed); });
}

grgx_status grgx_autotune_import(const char* text) {
    return guarded([&] {
        GRGX_CHECK(text, GRGX_ERR_API_MISUSE, "null argument");
        autotune_import(text);
    });
}

void grgx_autotune_clear(void) { autotune_clear(); }

grgx_status grgx_matmul_gram(grgx_graph* g, grgx_dtype dtype, const void* input, uint64_t input_cols,
                             uint64_t input_rows, grgx_direction first, void* output, uint64_t output_size,
                             int standardized, uint32_t flags, void* stream) {
    return guarded([&] {
        GRGX_CHECK(g && input && output, GRGX_ERR_API_MISUSE, "null argument");
        matmul_gram_impl(g, dtype, input, input_cols, input_rows, first, output, output_size, standardized, flags,
                         stream);
    });
}

grgx_status grgx_host_alloc(uint64_t bytes, void** out) {
    return guarded([&] {
        GRGX_CHECK(out, GRGX_ERR_API_MISUSE, "null argument");
        *out = host_alloc(bytes);
    });
}

void grgx_host_free(void* p) { host_free(p); }

void grgx_set_timing(int enabled) { set_timing(enabled); }

// Test hook (not part of the public header): uploads with the plan built on the host instead of
// the device, so the two builders can be compared.
extern "C" grgx_status grgx_graph_upload_host_plan(grgx_graph* g) {
    return guarded([&] {
        GRGX_CHECK(g, GRGX_ERR_API_MISUSE, "null argument");
        g->host_plan = true;
        ensure_device_plan(g);
    });
}

// Test hook (not part of the public header): one array of the plan the host builder lays out
// for `g` (plan.cpp: the renumbering, the level ranges, the UP/DOWN/seed rows, offsets and
// chunks -- the stages the device builder shares), so that its invariants can be checked
// without a GPU.  Names: "level_begin", "old2new", "new2old", "mut_new", "miss_new",
// "down_row_of", and "<csr>.<field>" for csr in up/down/seed/miss and field in rows/off/adj/
// chunks/heavy/level_chunk_begin/level_chunk_end (and up_fine/down_fine, the finer chunking of
// up/down: chunks, heavy and the level ranges only).  The arrays stay valid until the graph is
// destroyed.
extern "C" grgx_status grgx_debug_host_plan(grgx_graph* g, const char* name, const void** data,
                                            uint64_t* bytes) {
    return guarded([&] {
        GRGX_CHECK(g && name && data && bytes, GRGX_ERR_API_MISUSE, "null argument");
        {
            std::lock_guard<std::mutex> lk(g->mu);
            if (!g->inspect_plan) g->inspect_plan = grgx::build_plan(g->host_edges());
        }
        const grgx::HostPlan& p = *g->inspect_plan;
        bool found = false;
        auto put = [&](const auto& v) {
            *data = v.data();
            *bytes = static_cast<uint64_t>(v.size() * sizeof(v[0]));
            found = true;
        };
        const std::string n(name);
        if (n == "level_begin") put(p.level_begin);
        else if (n == "old2new") put(p.old2new);
        else if (n == "new2old") put(p.new2old);
        else if (n == "mut_new") put(p.mut_new);
        else if (n == "miss_new") put(p.miss_new);
        else if (n == "down_row_of") put(p.down_row_of);
        const std::pair<const char*, const grgx::PullCSR*> csrs[] = {
            {"up.", &p.up},           {"down.", &p.down},           {"seed.", &p.seed},
            {"miss.", &p.miss},       {"up_fine.", &p.up_fine},     {"down_fine.", &p.down_fine}};
        for (const auto& c : csrs) {
            if (n.rfind(c.first, 0) != 0) continue;
            const std::string f = n.substr(std::string(c.first).size());
            const grgx::PullCSR& P = *c.second;
            if (f == "rows") put(P.rows);
            else if (f == "off") put(P.off);
            else if (f == "adj") put(P.adj);
            else if (f == "chunks") put(P.chunks);
            else if (f == "heavy") put(P.heavy);
            else if (f == "level_chunk_begin") put(P.level_chunk_begin);
            else if (f == "level_chunk_end") put(P.level_chunk_end);
        }
        GRGX_CHECK(found, GRGX_ERR_API_MISUSE, "unknown plan array: " + n);
    });
}

// Test hook (not part of the public header): the block of height-0 ids used by split copies
// built from now on (0 keeps it) and the height-0 row bytes above which UP runs in split form.
extern "C" void grgx_debug_up_split(long long block, unsigned long long threshold_bytes) {
    grgx::set_up_split(block, threshold_bytes);
}

// Test hook (not part of the public header): DOWN split form by rule (0), always (1) or never
// (2); single-column split passes staged in shared memory (1) or gathered from global memory (0).
extern "C" void grgx_debug_split_forms(int down_mode, int staged) {
    grgx::set_down_split_mode(down_mode);
    grgx::set_staged(staged != 0);
}

grgx_status grgx_collect_timings(grgx_timing* out, uint64_t capacity, uint64_t* count) {
    return guarded([&] {
        GRGX_CHECK(count && (capacity == 0 || out), GRGX_ERR_API_MISUSE, "null argument");
        const std::vector<grgx_timing> t = collect_timings();
        GRGX_CHECK(t.size() <= capacity, GRGX_ERR_API_MISUSE, "timing buffer too small");
        for (size_t i = 0; i < t.size(); i++) out[i] = t[i];
        *count = t.size();
    });
}

grgx_status grgx_last_timing(grgx_timing* out) {
    return guarded([&] {
        GRGX_CHECK(out, GRGX_ERR_API_MISUSE, "null argument");
        *out = last_timing();
    });
}

}  // extern "C"
