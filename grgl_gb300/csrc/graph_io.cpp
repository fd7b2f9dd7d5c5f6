// .grg file reader: the subset of GRGL's immutable load that the matmul path needs.  The edge
// buckets stay encoded (as the reference's CSR storage keeps them, csr_storage.h:407-429)
// until the device plan decodes them on the GPU or a host consumer materialises them.
//
// Layout read here (src/serialize.cpp:815-890 readImmutableGrg, :697-758 readGrgCommon,
// include/grgl/common.h:181-202 header):
//   128-byte header (magic, version, ploidy, population count, sample/mutation/node/edge
//   counts, bp range, flags)
//   u64 edge byte count, then each node's children as one vbyte bucket: a varint count
//   followed by varint deltas of the ascending child ids (csr_storage.h:407-429)
//   node bucket offsets: u32 x (nodes+1) for format <= 5.1, else u64 x (nodes+1)
//   mutation -> node ids: u32 x mutations
//   mutation records: 24 bytes each (mutation.h:271-283); records whose allele storage word
//   has bit 0 set keep their alleles in a trailing varint-length string
//   population names (strings), then u16 population ids per sample, if populations > 0
//   coalescence counts: u32 x (nodes - samples)
//   individual ids, if flag 0x1: u64 byte count, bytes, offsets (u32 or u64) x (indivs+1)
//   missingness nodes, if flag 0x4: u32 x mutations
// The varint format is LEB128-style: 7 data bits per byte, high bit = more bytes follow
// (third-party/libvbyte/vbyte.cc:98-147).
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <thread>

#include "grgx_internal.h"

namespace grgx {
namespace {

constexpr uint64_t FILE_MAGIC = 0xE9366C64DDC8C5B0ull;  // common.h:181
constexpr uint16_t FILE_MAJOR = 5;                      // common.h:182
constexpr uint64_t FLAG_HAS_INDIV_IDS = 0x1;            // common.h:174
constexpr uint64_t FLAG_UNPHASED = 0x2;                 // common.h:176
constexpr uint64_t FLAG_HAS_MISSING = 0x4;              // common.h:179

#pragma pack(push, 1)
struct FileHeader {
    uint64_t magic;
    uint16_t versionMajor;
    uint16_t versionMinor;
    uint16_t ploidy;
    uint16_t populationCount;
    uint64_t sampleCount;
    uint64_t mutationCount;
    uint64_t nodeCount;
    uint64_t edgeCount;
    uint64_t rangeStart;
    uint64_t rangeEnd;
    uint64_t flags;
    uint64_t unused[7];
};
#pragma pack(pop)
static_assert(sizeof(FileHeader) == 128, "header size");

struct Reader {
    std::ifstream in;
    explicit Reader(const std::string& p) : in(p, std::ios::binary) {}
    void read(void* dst, size_t bytes) {
        in.read(reinterpret_cast<char*>(dst), static_cast<std::streamsize>(bytes));
        GRGX_CHECK(in.good() && static_cast<size_t>(in.gcount()) == bytes, GRGX_ERR_BAD_FILE,
                   "Malformed GRG file");
    }
    template <typename T> T scalar() {
        T v{};
        read(&v, sizeof(T));
        return v;
    }
    template <typename T> std::vector<T> array(size_t n) {
        std::vector<T> v(n);
        if (n) read(v.data(), n * sizeof(T));
        return v;
    }
    void skip(uint64_t bytes) {
        in.seekg(static_cast<std::streamoff>(bytes), std::ios::cur);
        GRGX_CHECK(in.good(), GRGX_ERR_BAD_FILE, "Malformed GRG file");
    }
    uint32_t varint32() {
        uint32_t value = 0;
        for (int shift = 0; shift < 35; shift += 7) {
            uint8_t b = scalar<uint8_t>();
            value |= static_cast<uint32_t>(b & 0x7fu) << shift;
            if (!(b & 0x80u)) return value;
        }
        throw Error(GRGX_ERR_BAD_FILE, "Malformed GRG file");
    }
    void skip_string() { skip(varint32()); }
};

inline size_t decode_varint(const uint8_t* p, const uint8_t* end, uint32_t* out) {
    uint32_t value = 0;
    size_t i = 0;
    for (int shift = 0; shift < 35; shift += 7, i++) {
        GRGX_CHECK(p + i < end, GRGX_ERR_BAD_FILE, "Malformed GRG file");
        const uint8_t b = p[i];
        value |= static_cast<uint32_t>(b & 0x7fu) << shift;
        if (!(b & 0x80u)) {
            *out = value;
            return i + 1;
        }
    }
    throw Error(GRGX_ERR_BAD_FILE, "Malformed GRG file");
}

}  // namespace

std::unique_ptr<HostGraph> load_grg_file(const std::string& path) {
    Reader r(path);
    GRGX_CHECK(r.in.good(), GRGX_ERR_BAD_FILE, "Could not read " + path);
    FileHeader h{};
    r.read(&h, sizeof(h));
    GRGX_CHECK(h.magic == FILE_MAGIC, GRGX_ERR_BAD_FILE, "Invalid file header");
    GRGX_CHECK(h.versionMajor == FILE_MAJOR, GRGX_ERR_BAD_FILE, "Incompatible file major version");
    GRGX_CHECK(h.ploidy != 0, GRGX_ERR_BAD_FILE, "Malformed GRG file: ploidy was 0");
    GRGX_CHECK(h.nodeCount <= MAX_NODES && h.sampleCount <= h.nodeCount, GRGX_ERR_BAD_FILE, "Malformed GRG file");
    const bool smallIdx = (h.versionMajor < 5) || (h.versionMajor == 5 && h.versionMinor <= 1);

    auto g = std::make_unique<HostGraph>();
    g->num_nodes = h.nodeCount;
    g->num_samples = h.sampleCount;
    g->num_mutations = h.mutationCount;
    g->ploidy = h.ploidy;
    g->phased = !(h.flags & FLAG_UNPHASED);

    const uint64_t edgeBytes = r.scalar<uint64_t>();
    std::vector<uint8_t> buckets = r.array<uint8_t>(edgeBytes);
    std::vector<uint64_t> nodeIdx(h.nodeCount + 1);
    if (smallIdx) {
        std::vector<uint32_t> small = r.array<uint32_t>(h.nodeCount + 1);
        for (size_t i = 0; i < small.size(); i++) nodeIdx[i] = small[i];
    } else {
        nodeIdx = r.array<uint64_t>(h.nodeCount + 1);
    }
    for (uint64_t v = 0; v < h.nodeCount; v++)
        GRGX_CHECK(nodeIdx[v] <= nodeIdx[v + 1] && nodeIdx[v + 1] <= edgeBytes, GRGX_ERR_BAD_FILE,
                   "Malformed GRG file");
    g->enc_buckets = std::move(buckets);
    g->enc_index = std::move(nodeIdx);
    g->enc_edges = h.edgeCount;

    g->mut_node = r.array<uint32_t>(h.mutationCount);
    for (uint32_t& n : g->mut_node)
        GRGX_CHECK(n == INVALID_NODE || n < h.nodeCount, GRGX_ERR_BAD_FILE, "Malformed GRG file");
    // Mutation records: 8 bytes allele storage, 8 position, 4 time, 2 alt index, 2 unused.
    std::vector<uint8_t> muts = r.array<uint8_t>(h.mutationCount * 24);
    g->mut_pos.resize(h.mutationCount);
    uint64_t deferred = 0;
    for (uint64_t m = 0; m < h.mutationCount; m++) {
        const uint8_t* rec = muts.data() + m * 24;
        if (rec[0] & 0x1u) deferred++;
        uint64_t pos;
        std::memcpy(&pos, rec + 8, 8);
        g->mut_pos[m] = pos;
    }
    for (uint64_t i = 0; i < deferred; i++) r.skip_string();
    if (h.populationCount > 0) {
        for (uint64_t i = 0; i < h.populationCount; i++) r.skip_string();
        r.skip(h.sampleCount * sizeof(uint16_t));
    }
    g->coals = r.array<uint32_t>(h.nodeCount - h.sampleCount);
    if (h.flags & FLAG_HAS_INDIV_IDS) {
        const uint64_t idBytes = r.scalar<uint64_t>();
        r.skip(idBytes);
        const uint64_t indivs = h.sampleCount / h.ploidy;
        r.skip((indivs + 1) * (smallIdx ? 4 : 8));
    }
    if (h.flags & FLAG_HAS_MISSING) {
        g->miss_node = r.array<uint32_t>(h.mutationCount);
        for (uint32_t& n : g->miss_node)
            GRGX_CHECK(n == INVALID_NODE || n < h.nodeCount, GRGX_ERR_BAD_FILE, "Malformed GRG file");
    }
    return g;
}

namespace {
void put_varint(std::vector<uint8_t>& out, uint32_t v) {
    while (v >= 0x80u) {
        out.push_back(static_cast<uint8_t>(v | 0x80u));
        v >>= 7;
    }
    out.push_back(static_cast<uint8_t>(v));
}
}  // namespace

// Writes format 5.3 in the layout the reader above takes (the reference writer's order,
// serialize.cpp:517-669): header; edge bucket bytes and buckets (count + deltas of the ascending
// children, an empty bucket for a node without children); u64 bucket offsets; mutation nodes;
// 24-byte mutation records (REF "A", ALT "C" stored inline, time not set); coalescence counts;
// missingness nodes when present.  Children must be ascending within each node.
void save_grg_file(const HostGraph& g, const std::string& path) {
    const uint64_t n = g.num_nodes, M = g.num_mutations;
    // buckets encoded in parallel over node ranges balanced by edge count, then concatenated
    const uint64_t E = g.down_adj.size();
    const unsigned hw = std::thread::hardware_concurrency();
    const int T = (E < (1u << 22)) ? 1 : static_cast<int>(std::min(64u, hw ? hw : 4u));
    std::vector<uint64_t> nb(T + 1, n);
    nb[0] = 0;
    for (int t = 1; t < T; t++)
        nb[t] = static_cast<uint64_t>(std::lower_bound(g.down_off.begin(), g.down_off.end(), E * t / T) -
                                      g.down_off.begin());
    std::vector<std::vector<uint8_t>> part(T);
    std::vector<uint64_t> index(n + 1, 0);
    std::vector<int> bad(T, 0);
    auto encode = [&](int t) {
        std::vector<uint8_t>& out = part[t];
        for (uint64_t v = nb[t]; v < nb[t + 1]; v++) {
            index[v] = out.size();  // relative to the part; rebased below
            const uint64_t b = g.down_off[v], e = g.down_off[v + 1];
            if (b < e) {
                put_varint(out, static_cast<uint32_t>(e - b));
                uint32_t prev = 0;
                for (uint64_t x = b; x < e; x++) {
                    const uint32_t c = g.down_adj[x];
                    if (x != b && c < prev) bad[t] = 1;
                    put_varint(out, c - prev);
                    prev = c;
                }
            }
        }
    };
    std::vector<std::thread> pool;
    for (int t = 1; t < T; t++) pool.emplace_back(encode, t);
    encode(0);
    for (auto& th : pool) th.join();
    for (int t = 0; t < T; t++) GRGX_CHECK(!bad[t], GRGX_ERR_API_MISUSE, "children must be ascending to be saved");
    uint64_t base = 0;
    for (int t = 0; t < T; t++) {
        for (uint64_t v = nb[t]; v < nb[t + 1]; v++) index[v] += base;
        base += part[t].size();
    }
    index[n] = base;
    FileHeader h{};
    h.magic = FILE_MAGIC;
    h.versionMajor = FILE_MAJOR;
    h.versionMinor = 3;
    h.ploidy = static_cast<uint16_t>(g.ploidy);
    h.populationCount = 0;
    h.sampleCount = g.num_samples;
    h.mutationCount = M;
    h.nodeCount = n;
    h.edgeCount = g.down_adj.size();
    uint64_t lo = UINT64_MAX, hi = 0;
    for (uint64_t p : g.mut_pos) {
        lo = std::min(lo, p);
        hi = std::max(hi, p + 1);
    }
    h.rangeStart = g.mut_pos.empty() ? 0 : lo;
    h.rangeEnd = g.mut_pos.empty() ? 0 : hi;
    h.flags = (g.phased ? 0 : FLAG_UNPHASED) | (g.miss_node.empty() ? 0 : FLAG_HAS_MISSING);
    std::ofstream out(path, std::ios::binary | std::ios::trunc);
    GRGX_CHECK(out.good(), GRGX_ERR_API_MISUSE, "Could not write " + path);
    auto put = [&](const void* p, size_t bytes) {
        out.write(static_cast<const char*>(p), static_cast<std::streamsize>(bytes));
    };
    put(&h, sizeof(h));
    const uint64_t edgeBytes = base;
    put(&edgeBytes, sizeof(edgeBytes));
    for (int t = 0; t < T; t++) put(part[t].data(), part[t].size());
    put(index.data(), index.size() * sizeof(uint64_t));
    put(g.mut_node.data(), g.mut_node.size() * sizeof(uint32_t));
    for (uint64_t m = 0; m < M; m++) {
        uint8_t rec[24] = {0};
        rec[1] = 'A';  // byte 0 stays 0: alleles stored inline
        rec[2] = 'C';
        const uint64_t pos = m < g.mut_pos.size() ? g.mut_pos[m] : m + 1;
        const uint32_t timeNotSet = 0x3FFFFFFFu;
        const uint16_t altIndex = 1;
        std::memcpy(rec + 8, &pos, 8);
        std::memcpy(rec + 16, &timeNotSet, 4);
        std::memcpy(rec + 20, &altIndex, 2);
        put(rec, sizeof(rec));
    }
    std::vector<uint32_t> coals(n - g.num_samples, COAL_NOT_SET);
    for (size_t i = 0; i < coals.size() && i < g.coals.size(); i++) coals[i] = g.coals[i];
    put(coals.data(), coals.size() * sizeof(uint32_t));
    if (!g.miss_node.empty()) put(g.miss_node.data(), g.miss_node.size() * sizeof(uint32_t));
    out.flush();
    GRGX_CHECK(out.good(), GRGX_ERR_API_MISUSE, "Writing GRG failed");
}

void materialize_edges(HostGraph& g) {
    if (!g.encoded()) return;
    const uint64_t n = g.num_nodes;
    std::vector<uint64_t> off(n + 1, 0);
    std::vector<uint32_t> adj;
    adj.reserve(g.enc_edges);
    const uint8_t* base = g.enc_buckets.data();
    const uint8_t* end = base + g.enc_buckets.size();
    for (uint64_t v = 0; v < n; v++) {
        const uint64_t b0 = g.enc_index[v], b1 = g.enc_index[v + 1];
        if (b0 < b1) {
            const uint8_t* p = base + b0;
            uint32_t count = 0;
            p += decode_varint(p, end, &count);
            uint32_t prev = 0;
            for (uint32_t i = 0; i < count; i++) {
                uint32_t delta = 0;
                p += decode_varint(p, end, &delta);
                prev += delta;
                GRGX_CHECK(prev < n, GRGX_ERR_BAD_FILE, "Malformed GRG file");
                adj.push_back(prev);
            }
        }
        off[v + 1] = adj.size();
    }
    GRGX_CHECK(adj.size() == g.enc_edges, GRGX_ERR_BAD_FILE, "Malformed GRG file");
    g.down_off = std::move(off);
    g.down_adj = std::move(adj);
    std::vector<uint8_t>().swap(g.enc_buckets);
    std::vector<uint64_t>().swap(g.enc_index);
    g.enc_edges = 0;
}

}  // namespace grgx
