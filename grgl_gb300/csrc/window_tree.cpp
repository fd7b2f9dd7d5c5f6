// Seeded window-tree GRG generator (the synthetic workload producer).
//
// For window w (variants [w*W, min((w+1)*W, M))) the generator draws, from a SplitMix64
// stream seeded with seed ^ w:
//   * a Kingman coalescent tree over all N samples: with k lineages the waiting time is
//     Exp(k(k-1)/2) and a uniformly random pair merges;
//   * one branch per variant, chosen with probability proportional to branch length; the
//     variant's carriers are the leaves below that branch (a ~1/f frequency spectrum).
// The tree is then collapsed to its mutated nodes, as a GRG built straight from a tree does
// (the idea of src/ts2grg.cpp): a mutated internal branch becomes a GRG node, a mutated leaf
// branch maps its mutation onto the sample node itself, and every GRG node's children are its
// nearest mutated descendants plus the samples with no mutated node in between.  Several
// variants on one branch share a node.
//
// Node ids: samples 0..N-1, then each window's mutated internal nodes in tree-creation order
// (children before parents), windows in order -- so the graph is topologically ordered and
// every child list is ascending.  Floating point is limited to +,-,*,/ and a series
// logarithm, compiled without FMA contraction, so every platform builds the same graph.
#include <algorithm>
#include <cstring>
#include <thread>

#include "grgx_internal.h"

namespace grgx {
namespace {

struct SplitMix64 {
    uint64_t s;
    explicit SplitMix64(uint64_t seed) : s(seed) {}
    uint64_t next() {
        uint64_t z = (s += 0x9e3779b97f4a7c15ull);
        z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
        z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
        return z ^ (z >> 31);
    }
    double uniform() { return static_cast<double>(next() >> 11) * (1.0 / 9007199254740992.0); }  // [0, 1)
    uint64_t below(uint64_t k) { return static_cast<uint64_t>((static_cast<unsigned __int128>(next()) * k) >> 64); }
};

// Natural log from range reduction x = m * 2^e (m in [sqrt(1/2), sqrt(2))) and the series
// ln m = 2 atanh(z), z = (m-1)/(m+1), |z| < 0.172; 12 terms reach double precision.
double series_log(double x) {
    int e = 0;
    double m = x;
    while (m > 1.4142135623730951) {
        m *= 0.5;
        e++;
    }
    while (m < 0.7071067811865476) {
        m *= 2.0;
        e--;
    }
    const double z = (m - 1.0) / (m + 1.0);
    const double z2 = z * z;
    double term = z, sum = 0.0;
    for (int k = 1; k <= 25; k += 2) {
        sum += term / static_cast<double>(k);
        term *= z2;
    }
    return static_cast<double>(e) * 0.6931471805599453 + 2.0 * sum;
}

struct WindowOut {
    uint32_t num_nodes = 0;              // mutated internal nodes (new GRG nodes)
    std::vector<uint32_t> off;           // num_nodes + 1
    std::vector<uint32_t> adj;           // children: sample id (< N) or N + local index
    std::vector<uint32_t> mut_local;     // per variant: sample id, or N + local index
};

void simulate_window(uint64_t N, uint64_t seed, uint64_t w, uint32_t nvar, WindowOut& out,
                     std::vector<uint32_t>& lin, std::vector<uint32_t>& parent, std::vector<double>& time,
                     std::vector<double>& cum, std::vector<int32_t>& local, std::vector<uint32_t>& nma) {
    SplitMix64 rng(seed ^ w);
    const uint64_t T = 2 * N - 1;  // tree nodes: leaves 0..N-1, internal N..2N-2 (root = 2N-2)
    lin.resize(N);
    parent.assign(T, 0xffffffffu);
    time.assign(T, 0.0);
    for (uint64_t i = 0; i < N; i++) lin[i] = static_cast<uint32_t>(i);
    double t = 0.0;
    uint64_t next = N;
    for (uint64_t k = N; k > 1; k--) {
        const double rate = 0.5 * static_cast<double>(k) * static_cast<double>(k - 1);
        t += -series_log(1.0 - rng.uniform()) / rate;
        const uint64_t i = rng.below(k);
        uint64_t j = rng.below(k - 1);
        if (j >= i) j++;
        const uint32_t p = static_cast<uint32_t>(next++);
        parent[lin[i]] = p;
        parent[lin[j]] = p;
        time[p] = t;
        lin[i] = p;
        lin[j] = lin[k - 1];
    }
    const uint64_t root = T - 1;
    // Branch-length prefix sums over the non-root nodes, in node order.
    cum.resize(root);
    double acc = 0.0;
    for (uint64_t v = 0; v < root; v++) {
        acc += time[parent[v]] - time[v];
        cum[v] = acc;
    }
    // Mutations: branch chosen in proportion to length.
    std::vector<uint32_t> branch(nvar);
    for (uint32_t j = 0; j < nvar; j++) {
        const double u = rng.uniform() * acc;
        uint64_t b = static_cast<uint64_t>(std::upper_bound(cum.begin(), cum.end(), u) - cum.begin());
        if (b >= root) b = root - 1;
        branch[j] = static_cast<uint32_t>(b);
    }
    // Mutated internal nodes get local ids in tree-node order (children before parents).
    local.assign(T, -1);
    std::vector<uint8_t> mutated(T, 0);
    for (uint32_t j = 0; j < nvar; j++) mutated[branch[j]] = 1;
    uint32_t cnt = 0;
    for (uint64_t v = N; v < T; v++)
        if (mutated[v]) local[v] = static_cast<int32_t>(cnt++);
    out.num_nodes = cnt;
    // Nearest mutated strict ancestor, parents first (descending node order).
    nma.assign(T, 0xffffffffu);
    for (uint64_t vv = root; vv > 0; vv--) {
        const uint64_t v = vv - 1;
        const uint32_t p = parent[v];
        nma[v] = mutated[p] ? p : nma[p];
    }
    // Children: samples (ascending) then mutated internal nodes (ascending).
    out.off.assign(cnt + 1, 0);
    for (uint64_t s = 0; s < N; s++) {
        if (mutated[s]) {
            if (nma[s] != 0xffffffffu) out.off[local[nma[s]] + 1]++;
        } else if (nma[s] != 0xffffffffu) {
            out.off[local[nma[s]] + 1]++;
        }
    }
    for (uint64_t v = N; v < root; v++)
        if (mutated[v] && nma[v] != 0xffffffffu) out.off[local[nma[v]] + 1]++;
    for (uint32_t i = 0; i < cnt; i++) out.off[i + 1] += out.off[i];
    out.adj.resize(out.off[cnt]);
    std::vector<uint32_t> fill(out.off.begin(), out.off.end() - 1);
    for (uint64_t s = 0; s < N; s++)
        if (nma[s] != 0xffffffffu) out.adj[fill[local[nma[s]]]++] = static_cast<uint32_t>(s);
    for (uint64_t v = N; v < root; v++)
        if (mutated[v] && nma[v] != 0xffffffffu) out.adj[fill[local[nma[v]]]++] = static_cast<uint32_t>(N + local[v]);
    out.mut_local.resize(nvar);
    for (uint32_t j = 0; j < nvar; j++) {
        const uint32_t b = branch[j];
        out.mut_local[j] = (b < N) ? b : static_cast<uint32_t>(N + local[b]);
    }
}

}  // namespace

std::unique_ptr<HostGraph> generate_window_tree(uint64_t N, uint64_t M, uint64_t seed, uint32_t W, int threads) {
    GRGX_CHECK(N >= 2 && N < 0x40000000ull, GRGX_ERR_API_MISUSE, "num_samples must be in [2, 2^30)");
    GRGX_CHECK(W >= 1, GRGX_ERR_API_MISUSE, "window must be positive");
    if (threads <= 0) threads = static_cast<int>(std::max(1u, std::thread::hardware_concurrency()));
    const uint64_t nwin = (M + W - 1) / W;
    auto g = std::make_unique<HostGraph>();
    g->num_samples = N;
    g->ploidy = 2;
    g->num_mutations = M;
    g->mut_node.assign(M, INVALID_NODE);
    g->mut_pos.resize(M);
    for (uint64_t m = 0; m < M; m++) g->mut_pos[m] = m + 1;  // window w, variant j: w*W + j + 1
    g->down_off.assign(N + 1, 0);
    g->down_adj.reserve(nwin * (N + W));

    const uint64_t batch = static_cast<uint64_t>(threads) * 2;
    std::vector<WindowOut> outs(batch);
    uint64_t nextNode = N;
    for (uint64_t w0 = 0; w0 < nwin; w0 += batch) {
        const uint64_t w1 = std::min(nwin, w0 + batch);
        std::vector<std::thread> pool;
        const uint64_t per = (w1 - w0 + threads - 1) / threads;
        for (int t = 0; t < threads; t++) {
            const uint64_t a = w0 + t * per, b = std::min(w1, a + per);
            if (a >= b) break;
            pool.emplace_back([&, a, b] {
                std::vector<uint32_t> lin, parent, nma;
                std::vector<double> time, cum;
                std::vector<int32_t> local;
                for (uint64_t w = a; w < b; w++) {
                    const uint32_t nvar = static_cast<uint32_t>(std::min<uint64_t>(W, M - w * W));
                    simulate_window(N, seed, w, nvar, outs[w - w0], lin, parent, time, cum, local, nma);
                }
            });
        }
        for (auto& th : pool) th.join();
        for (uint64_t w = w0; w < w1; w++) {
            WindowOut& o = outs[w - w0];
            const uint64_t base = nextNode;
            GRGX_CHECK(base + o.num_nodes <= MAX_NODES, GRGX_ERR_UNSUPPORTED, "generated graph exceeds the node limit");
            for (uint32_t i = 0; i < o.num_nodes; i++) {
                for (uint32_t e = o.off[i]; e < o.off[i + 1]; e++) {
                    const uint32_t c = o.adj[e];
                    g->down_adj.push_back(c < N ? c : static_cast<uint32_t>(base + (c - N)));
                }
                g->down_off.push_back(g->down_adj.size());
            }
            for (uint64_t j = 0; j < o.mut_local.size(); j++) {
                const uint32_t x = o.mut_local[j];
                g->mut_node[w * W + j] = x < N ? x : static_cast<uint32_t>(base + (x - N));
            }
            nextNode += o.num_nodes;
            WindowOut().adj.swap(o.adj);
        }
    }
    g->num_nodes = nextNode;
    g->down_adj.shrink_to_fit();
    return g;
}

}  // namespace grgx
