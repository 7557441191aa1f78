// fbk_compact.cu — unitig compaction from the device-resident solid table
// (src/graph/build.rs:330-594).
//
// The reference walks, in hash-map order, every out-edge of every boundary directed
// k-mer (in-degree != 1 or out-degree != 1), extending through 1-in-1-out nodes and
// marking the edges it used so the walk from the other end of the same unitig is
// skipped; then it walks the remaining all-1-in-1-out cycles; then it links unitigs
// whose ends overlap by k or k-1 bases.  Here:
//   1. a node index (open addressing over the converted rows) is built on the device;
//   2. every (boundary node, direction, out-edge) start walks its path on the device,
//      one thread per start, with no shared marks: a unitig reachable from both ends
//      is kept from the end whose (row, direction, edge) is smaller — the same set of
//      unitigs, decided without ordering;
//   3. a second walk writes the bases of the kept paths and marks their nodes, and a
//      per-unitig pass stores min(sequence, reverse complement) as the reference does;
//   4. the 1-in-1-out nodes no path visited (isolated cycles, few) and the overlap
//      edges are handled on the host, as build.rs:450-594 does.
// A unitig's coverage is the mean node coverage of its path without the last node
// (build.rs:379-435); which end a path starts from therefore changes its coverage
// when the end nodes differ, exactly as the reference's map order does.
#include <algorithm>
#include <array>
#include <cstring>
#include <string>
#include <unordered_map>
#include <vector>

#include "fbk_device.cuh"
#include "fbk_internal.h"

using namespace fbk;

namespace {

constexpr uint64_t CIDX_SALT = 0x3c6ef372fe94f82bULL;

// ---- multi-word k-mer integers (big-endian words, value = the MSB-first k-mer) ----
template <int NW>
__host__ __device__ __forceinline__ void kshl2_push(Key<NW>& x, uint32_t b, uint32_t k) {
    // ((x << 2) | b) masked to 2k bits (KmerInt::roll_next, forward half)
#pragma unroll
    for (int i = 0; i < NW; ++i) x.w[i] = (x.w[i] << 2) | (i + 1 < NW ? (x.w[i + 1] >> 62) : 0ULL);
    x.w[NW - 1] |= b;
    const uint32_t bits = 2 * k;
#pragma unroll
    for (int i = 0; i < NW; ++i) {
        const int lo = 64 * (NW - 1 - i);  // lowest bit of word i
        if ((int)bits <= lo) x.w[i] = 0;
        else if ((int)bits < lo + 64) x.w[i] &= (1ULL << (bits - lo)) - 1;
    }
}
template <int NW>
__host__ __device__ __forceinline__ void kshr2_put(Key<NW>& x, uint32_t c, uint32_t k) {
    // (x >> 2) | (c << 2(k-1))  (KmerInt::roll_next, reverse half)
#pragma unroll
    for (int i = NW - 1; i >= 0; --i) x.w[i] = (x.w[i] >> 2) | (i > 0 ? (x.w[i - 1] << 62) : 0ULL);
    const uint32_t pos = 2 * (k - 1);
    x.w[NW - 1 - pos / 64] |= (uint64_t)c << (pos % 64);
}
template <int NW>
__host__ __device__ __forceinline__ uint32_t kbase(const Key<NW>& x, uint32_t i, uint32_t k) {
    // base i from the 5' end (i = 0: most significant)
    const uint32_t pos = 2 * (k - 1 - i);
    return (uint32_t)(x.w[NW - 1 - pos / 64] >> (pos % 64)) & 3u;
}
template <int NW>
__host__ __device__ __forceinline__ Key<NW> krc(const Key<NW>& x, uint32_t k) {
    Key<NW> r;
#pragma unroll
    for (int i = 0; i < NW; ++i) r.w[i] = 0;
    for (uint32_t i = 0; i < k; ++i) {
        // base i of rc = complement of base k-1-i of x
        const uint32_t c = 3u - kbase<NW>(x, k - 1 - i, k);
        const uint32_t pos = 2 * (k - 1 - i);
        r.w[NW - 1 - pos / 64] |= (uint64_t)c << (pos % 64);
    }
    return r;
}
template <int NW>
__host__ __device__ __forceinline__ bool kless(const Key<NW>& a, const Key<NW>& b) {
    for (int i = 0; i < NW; ++i)
        if (a.w[i] != b.w[i]) return a.w[i] < b.w[i];
    return false;
}
template <int NW>
__host__ __device__ __forceinline__ bool keq(const Key<NW>& a, const Key<NW>& b) {
    for (int i = 0; i < NW; ++i)
        if (a.w[i] != b.w[i]) return false;
    return true;
}
template <int NW>
__host__ __device__ __forceinline__ uint64_t kfold(const Key<NW>& a) {
    uint64_t f = 0;
    for (int i = 0; i < NW; ++i) f ^= a.w[i];
    return f;
}

struct Rows {
    const uint64_t* keys;
    const uint16_t* cov;
    const uint8_t* mask;
    uint64_t n;
    const uint32_t* idx;  // node index: row + 1, 0 = empty
    uint64_t cap;         // power of two
};

template <int NW>
__device__ __forceinline__ Key<NW> row_key(const Rows& R, uint64_t r) {
    Key<NW> x;
#pragma unroll
    for (int i = 0; i < NW; ++i) x.w[i] = R.keys[r * NW + i];
    return x;
}

template <int NW>
__device__ __forceinline__ int64_t find_row(const Rows& R, const Key<NW>& x) {
    uint64_t s = smix(kfold<NW>(x) ^ CIDX_SALT) & (R.cap - 1);
    for (uint64_t probe = 0; probe < R.cap; ++probe) {
        const uint32_t v = R.idx[s];
        if (v == 0) return -1;
        if (keq<NW>(row_key<NW>(R, v - 1), x)) return (int64_t)(v - 1);
        s = (s + 1) & (R.cap - 1);
    }
    return -1;
}

template <int NW>
__global__ void k_cidx_build(const uint64_t* __restrict__ keys, uint64_t n, uint32_t* idx, uint64_t cap, uint32_t* status) {
    for (uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += (uint64_t)gridDim.x * blockDim.x) {
        Key<NW> x;
#pragma unroll
        for (int i = 0; i < NW; ++i) x.w[i] = keys[r * NW + i];
        uint64_t s = smix(kfold<NW>(x) ^ CIDX_SALT) & (cap - 1);
        bool done = false;
        for (uint64_t probe = 0; probe < cap && !done; ++probe) {
            done = atomicCAS(&idx[s], 0u, (uint32_t)(r + 1)) == 0u;
            s = (s + 1) & (cap - 1);
        }
        if (!done) atomicOr(status, ST_TABLE_FULL);
    }
}

__device__ __forceinline__ uint32_t pc4(uint32_t v) { return __popc(v & 15u); }

// Walk starts per row: every out-edge of both directions of a boundary row.
__global__ void k_walk_count(const uint8_t* __restrict__ mask, uint64_t n, uint32_t* cnt) {
    for (uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t m = mask[r];
        const bool boundary = pc4(m) != 1 || pc4(m >> 4) != 1;
        cnt[r] = boundary ? pc4(m) + pc4(m >> 4) : 0;
    }
}
// Start list from the exclusive prefix of the counts: start = row << 4 | dir << 3 | edge.
__global__ void k_walk_starts(const uint8_t* __restrict__ mask, uint64_t n, const uint64_t* __restrict__ pre, uint64_t* starts) {
    for (uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t m = mask[r];
        if (pc4(m) == 1 && pc4(m >> 4) == 1) continue;
        uint64_t o = pre[r];
        for (uint32_t dir = 0; dir < 2; ++dir) {
            const uint32_t out = dir ? (m >> 4) & 15u : m & 15u;
            for (uint32_t b = 0; b < 4; ++b)
                if ((out >> b) & 1u) starts[o++] = (r << 4) | (dir << 3) | b;
        }
    }
}

// One walk (build.rs:349-445 without the marks).  Returns the bases (k + steps), the
// coverage sum and points, and whether this start keeps the unitig.  When `seq` is
// given, writes the bases in walk orientation and marks the visited rows.
template <int NW>
__device__ void walk(const Rows& R, uint32_t k, uint64_t start, uint64_t max_steps, uint64_t& len, unsigned long long& cov_sum,
                     uint64_t& points, bool& keep, uint8_t* seq, uint8_t* visited, uint32_t* status) {
    const uint64_t r0 = start >> 4;
    const uint32_t dir0 = (uint32_t)(start >> 3) & 1u, b0 = (uint32_t)start & 7u;
    const Key<NW> u = row_key<NW>(R, r0);
    Key<NW> f = dir0 ? krc<NW>(u, k) : u;
    Key<NW> rv = dir0 ? u : krc<NW>(u, k);
    if (seq) {
        for (uint32_t i = 0; i < k; ++i) seq[i] = "ACGT"[kbase<NW>(f, i, k)];
        visited[r0] = 1;
    }
    uint32_t rc_p = 3u - kbase<NW>(f, 0, k);
    kshl2_push<NW>(f, b0, k);
    kshr2_put<NW>(rv, 3u - b0, k);
    len = k + 1;
    if (seq) seq[k] = "ACGT"[b0];
    cov_sum = R.cov[r0];
    points = 1;
    keep = true;
    for (uint64_t step = 0;; ++step) {
        const bool c_rc = kless<NW>(rv, f);
        const Key<NW> can = c_rc ? rv : f;
        const int64_t rc = find_row<NW>(R, can);
        if (rc < 0) return;  // the path ends at a k-mer with no node: no walk comes back
        const uint32_t m = R.mask[rc];
        const uint32_t c_out = c_rc ? (m >> 4) & 15u : m & 15u;
        const uint32_t c_in = c_rc ? m & 15u : (m >> 4) & 15u;
        if (__popc(c_in) != 1 || __popc(c_out) != 1) {
            // boundary end: the walk from (rc, !c_rc, rc_p) covers the same unitig
            const uint32_t back = c_rc ? m & 15u : (m >> 4) & 15u;  // out-edges of the opposite direction
            if ((back >> rc_p) & 1u) {
                const uint64_t other = ((uint64_t)rc << 4) | ((uint64_t)(c_rc ? 0u : 1u) << 3) | rc_p;
                keep = start <= other;
            }
            if (seq) visited[rc] = 1;
            return;
        }
        if (step >= max_steps) {
            atomicOr(status, ST_SPIN_TIMEOUT);  // a path longer than the node count: impossible for valid rows
            return;
        }
        if (seq) visited[rc] = 1;
        const uint32_t nb = __ffs(c_out) - 1;
        rc_p = 3u - kbase<NW>(f, 0, k);
        kshl2_push<NW>(f, nb, k);
        kshr2_put<NW>(rv, 3u - nb, k);
        if (seq) seq[len] = "ACGT"[nb];
        len++;
        cov_sum += R.cov[rc];
        points++;
    }
}

template <int NW>
__global__ void k_walk_measure(Rows R, uint32_t k, const uint64_t* __restrict__ starts, uint64_t n_starts, uint64_t* len_out,
                               unsigned long long* cov_out, uint64_t* pts_out, uint32_t* status) {
    for (uint64_t s = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; s < n_starts; s += (uint64_t)gridDim.x * blockDim.x) {
        uint64_t len, pts;
        unsigned long long cs;
        bool keep;
        walk<NW>(R, k, starts[s], R.n + 1, len, cs, pts, keep, nullptr, nullptr, status);
        len_out[s] = keep ? len : 0;
        cov_out[s] = cs;
        pts_out[s] = pts;
    }
}

template <int NW>
__global__ void k_walk_write(Rows R, uint32_t k, const uint64_t* __restrict__ starts, uint64_t n_starts,
                             const uint64_t* __restrict__ len, const uint64_t* __restrict__ off, uint8_t* seqs, uint8_t* visited,
                             uint32_t* status) {
    for (uint64_t s = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; s < n_starts; s += (uint64_t)gridDim.x * blockDim.x) {
        if (!len[s]) continue;
        uint64_t l, pts;
        unsigned long long cs;
        bool keep;
        walk<NW>(R, k, starts[s], R.n + 1, l, cs, pts, keep, seqs + off[s], visited, status);
    }
}

// min(sequence, reverse complement), in place (build.rs:438-439).
__global__ void k_canon_seq(uint8_t* seqs, const uint64_t* __restrict__ off, const uint64_t* __restrict__ len, uint64_t n) {
    for (uint64_t s = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; s < n; s += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t L = len[s];
        if (!L) continue;
        uint8_t* q = seqs + off[s];
        auto comp = [](uint8_t c) -> uint8_t { return c == 'A' ? 'T' : c == 'C' ? 'G' : c == 'G' ? 'C' : 'A'; };
        int cmp = 0;
        for (uint64_t i = 0; i < L && !cmp; ++i) {
            const uint8_t a = comp(q[L - 1 - i]), b = q[i];
            cmp = a < b ? -1 : a > b ? 1 : 0;
        }
        if (cmp < 0) {
            for (uint64_t i = 0; i < L / 2; ++i) {
                const uint8_t a = q[i], b = q[L - 1 - i];
                q[i] = comp(b);
                q[L - 1 - i] = comp(a);
            }
            if (L & 1) q[L / 2] = comp(q[L / 2]);
        }
    }
}

// Rows that are 1-in-1-out and on no path: candidates for isolated cycles.
__global__ void k_cycle_candidates(const uint8_t* __restrict__ mask, const uint8_t* __restrict__ visited, uint64_t n, uint8_t* flag) {
    for (uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t m = mask[r];
        flag[r] = (!visited[r] && pc4(m) == 1 && pc4(m >> 4) == 1) ? 1 : 0;
    }
}

// ---- host side ---------------------------------------------------------------
struct HUnitig {
    std::string seq;
    float cov;
    bool circular;
};

template <int NW>
struct HKeyHash {
    size_t operator()(const std::array<uint64_t, NW>& a) const {
        uint64_t f = 0;
        for (int i = 0; i < NW; ++i) f ^= a[i];
        return (size_t)smix(f);
    }
};

// build.rs:450-555 over the candidate rows (host).
template <int NW>
void host_cycles(uint32_t k, const std::vector<uint64_t>& keys, const std::vector<uint16_t>& cov, const std::vector<uint8_t>& mask,
                 std::vector<HUnitig>& out) {
    using A = std::array<uint64_t, NW>;
    struct N {
        uint16_t cov;
        uint8_t mask, visited;
    };
    std::unordered_map<A, N, HKeyHash<NW>> map;
    std::vector<A> order;
    for (size_t i = 0; i < cov.size(); ++i) {
        A a;
        for (int j = 0; j < NW; ++j) a[j] = keys[i * NW + j];
        map[a] = N{cov[i], mask[i], 0};
        order.push_back(a);
    }
    auto toK = [](const A& a) {
        Key<NW> x;
        for (int j = 0; j < NW; ++j) x.w[j] = a[j];
        return x;
    };
    auto toA = [](const Key<NW>& x) {
        A a;
        for (int j = 0; j < NW; ++j) a[j] = x.w[j];
        return a;
    };
    for (const A& a : order) {
        auto it = map.find(a);
        const N n0 = it->second;
        const uint32_t fo = n0.mask & 15u, fi = (n0.mask >> 4) & 15u;
        if (__builtin_popcount(fo) != 1 || __builtin_popcount(fi) != 1) continue;
        const uint32_t b = __builtin_ctz(fo);
        if ((n0.visited >> b) & 1u) continue;
        it->second.visited |= (uint8_t)(1u << b);
        const Key<NW> start = toK(a);
        std::string path(k, 'A');
        for (uint32_t i = 0; i < k; ++i) path[i] = "ACGT"[kbase<NW>(start, i, k)];
        Key<NW> f = start, rv = krc<NW>(start, k);
        const uint32_t rc_first = 3u - kbase<NW>(f, 0, k);
        kshl2_push<NW>(f, b, k);
        kshr2_put<NW>(rv, 3u - b, k);
        bool c_rc = kless<NW>(rv, f);
        Key<NW> cur = c_rc ? rv : f;
        auto mark = [&](const Key<NW>& x, uint32_t bit) {
            auto m = map.find(toA(x));
            if (m != map.end()) m->second.visited |= (uint8_t)(1u << bit);
        };
        mark(cur, !c_rc ? rc_first + 4 : rc_first);
        path.push_back("ACGT"[b]);
        uint64_t total = n0.cov, points = 1;
        while (!keq<NW>(cur, start)) {
            auto m = map.find(toA(cur));
            if (m == map.end()) break;
            const N nc = m->second;
            const uint32_t c_out = !c_rc ? nc.mask & 15u : (nc.mask >> 4) & 15u;
            const uint32_t c_in = !c_rc ? (nc.mask >> 4) & 15u : nc.mask & 15u;
            if (__builtin_popcount(c_in) != 1 || __builtin_popcount(c_out) != 1) break;
            const uint32_t nb = __builtin_ctz(c_out);
            const uint32_t ebit = !c_rc ? nb : nb + 4;
            if ((nc.visited >> ebit) & 1u) break;
            m->second.visited |= (uint8_t)(1u << ebit);
            const uint32_t rc_p = 3u - kbase<NW>(f, 0, k);
            kshl2_push<NW>(f, nb, k);
            kshr2_put<NW>(rv, 3u - nb, k);
            c_rc = kless<NW>(rv, f);
            cur = c_rc ? rv : f;
            mark(cur, !c_rc ? rc_p + 4 : rc_p);
            path.push_back("ACGT"[nb]);
            total += nc.cov;
            points++;
        }
        if (keq<NW>(cur, start) && path.size() > k) {
            if (path.compare(path.size() - k, k, path, 0, k) == 0) path.resize(path.size() - k);
            else if (path.compare(path.size() - (k - 1), k - 1, path, 0, k - 1) == 0) path.resize(path.size() - (k - 1));
            out.push_back(HUnitig{path, std::max(1.0f, (float)total / (float)points), true});
        }
    }
}

std::string rc_string(const std::string& s) {
    std::string r(s.size(), 'A');
    for (size_t i = 0; i < s.size(); ++i) {
        const char c = s[s.size() - 1 - i];
        r[i] = c == 'A' ? 'T' : c == 'C' ? 'G' : c == 'G' ? 'C' : 'A';
    }
    return r;
}

}  // namespace

struct fbk_unitigs {
    std::vector<HUnitig> u;
    // edges: from id, from side (0 forward, 1 reverse strand), to id, to rc, overlap, support
    std::vector<std::array<uint32_t, 6>> edges;
    uint64_t bases = 0, linear_walks = 0, cycle_candidates = 0;
};

namespace {

// build.rs:557-594: edges by exact k and k-1 overlap; cdbg.rs:113-122 merges repeats.
void link_unitigs(uint32_t k, fbk_unitigs* U) {
    const uint32_t n = (uint32_t)U->u.size();
    std::vector<std::vector<std::array<uint32_t, 4>>> side[2];
    side[0].resize(n);
    side[1].resize(n);
    auto add = [&](uint32_t id, int s, uint32_t t, uint32_t trc, uint32_t ov, uint32_t sup) {
        for (auto& e : side[s][id])
            if (e[0] == t && e[1] == trc && e[2] == ov) {
                e[3] = std::min<uint32_t>(65535, e[3] + sup);
                return;
            }
        side[s][id].push_back({t, trc, ov, sup});
    };
    for (uint32_t id = 0; id < n; ++id)
        if (U->u[id].circular) add(id, 0, id, 0, k - 1, 10);  // build.rs:546-547
    for (uint32_t ov : {k, k - 1}) {
        if (ov == 0) continue;
        std::unordered_map<std::string, std::vector<std::pair<uint32_t, uint32_t>>> prefix;
        std::vector<std::string> rcs(n);
        for (uint32_t id = 0; id < n; ++id) {
            const std::string& f = U->u[id].seq;
            rcs[id] = rc_string(f);
            if (f.size() >= ov) {
                prefix[f.substr(0, ov)].push_back({id, 0});
                prefix[rcs[id].substr(0, ov)].push_back({id, 1});
            }
        }
        for (uint32_t id = 0; id < n; ++id) {
            const std::string& f = U->u[id].seq;
            if (f.size() < ov) continue;
            auto a = prefix.find(f.substr(f.size() - ov));
            if (a != prefix.end())
                for (auto& t : a->second)
                    if (t.first != id || U->u[id].circular) add(id, 0, t.first, t.second, ov, 10);
            const std::string& r = rcs[id];
            auto c = prefix.find(r.substr(r.size() - ov));
            if (c != prefix.end())
                for (auto& t : c->second)
                    if (t.first != id || U->u[id].circular) add(id, 1, t.first, t.second, ov, 10);
        }
    }
    for (uint32_t id = 0; id < n; ++id)
        for (int s = 0; s < 2; ++s)
            for (auto& e : side[s][id]) U->edges.push_back({id, (uint32_t)s, e[0], e[1], e[2], e[3]});
}

template <int NW>
fbk_status compact_impl(fbk_table* t, fbk_unitigs* U) {
    fbk_ctx* ctx = t->ctx;
    const uint64_t n = t->n_solid;
    const uint32_t k = t->k;
    if (k < 2) return set_err(ctx, FBK_ERR_INVALID, "compaction needs k >= 2");
    if (n == 0) return FBK_OK;
    if (n >= (1ULL << 31)) return set_err(ctx, FBK_ERR_INVALID, "compaction: more than 2^31 solid rows");
    Launch L = launch_cfg(ctx, 256, 0);
    uint64_t cap = 1;
    while (cap < 2 * n) cap <<= 1;
    struct Bufs {
        fbk_ctx* c;
        std::vector<void*> p;
        void* get(uint64_t b) {
            void* q = dev_alloc(c, b);
            if (q) p.push_back(q);
            return q;
        }
        ~Bufs() {
            cudaStreamSynchronize(c->stream);
            for (void* q : p) dev_free(c, q);
        }
    } B{ctx, {}};
    uint32_t* idx = (uint32_t*)B.get(cap * 4);
    uint32_t* cnt = (uint32_t*)B.get(n * 4);
    uint8_t* visited = (uint8_t*)B.get(n);
    if (!idx || !cnt || !visited) return set_err(ctx, FBK_ERR_OOM, "compaction index");
    CK(ctx, cudaMemsetAsync(idx, 0, cap * 4, ctx->stream));
    CK(ctx, cudaMemsetAsync(visited, 0, n, ctx->stream));
    CK(ctx, cudaMemsetAsync(ctx->d_status, 0, 4, ctx->stream));
    TIMED(ctx, "compact_index", (k_cidx_build<NW><<<L.grid, L.block, 0, L.stream>>>(t->out_keys, n, idx, cap, ctx->d_status),
                                 cudaGetLastError()));
    TIMED(ctx, "compact_count", (k_walk_count<<<L.grid, L.block, 0, L.stream>>>(t->out_mask, n, cnt), cudaGetLastError()));
    // prefix of the per-row start counts (host: one pass over n u32)
    std::vector<uint32_t> hc(n);
    CK(ctx, cudaMemcpyAsync(hc.data(), cnt, n * 4, cudaMemcpyDeviceToHost, ctx->stream));
    CK(ctx, cudaStreamSynchronize(ctx->stream));
    std::vector<uint64_t> pre(n);
    uint64_t n_starts = 0;
    for (uint64_t r = 0; r < n; ++r) {
        pre[r] = n_starts;
        n_starts += hc[r];
    }
    U->linear_walks = n_starts;
    Rows R{t->out_keys, t->out_cov, t->out_mask, n, idx, cap};
    std::vector<uint64_t> hlen(n_starts), hoff(n_starts);
    std::vector<unsigned long long> hcs(n_starts);
    std::vector<uint64_t> hpts(n_starts);
    uint8_t* seqs = nullptr;
    uint64_t total = 0;
    if (n_starts) {
        uint64_t* d_pre = (uint64_t*)B.get(n * 8);
        uint64_t* starts = (uint64_t*)B.get(n_starts * 8);
        uint64_t* len = (uint64_t*)B.get(n_starts * 8);
        unsigned long long* cs = (unsigned long long*)B.get(n_starts * 8);
        uint64_t* pts = (uint64_t*)B.get(n_starts * 8);
        uint64_t* off = (uint64_t*)B.get(n_starts * 8);
        if (!d_pre || !starts || !len || !cs || !pts || !off) return set_err(ctx, FBK_ERR_OOM, "compaction walks");
        CK(ctx, cudaMemcpyAsync(d_pre, pre.data(), n * 8, cudaMemcpyHostToDevice, ctx->stream));
        TIMED(ctx, "compact_starts", (k_walk_starts<<<L.grid, L.block, 0, L.stream>>>(t->out_mask, n, d_pre, starts), cudaGetLastError()));
        TIMED(ctx, "compact_walk", (k_walk_measure<NW><<<L.grid, L.block, 0, L.stream>>>(R, k, starts, n_starts, len, cs, pts,
                                                                                          ctx->d_status),
                                    cudaGetLastError()));
        CK(ctx, cudaMemcpyAsync(hlen.data(), len, n_starts * 8, cudaMemcpyDeviceToHost, ctx->stream));
        CK(ctx, cudaMemcpyAsync(hcs.data(), cs, n_starts * 8, cudaMemcpyDeviceToHost, ctx->stream));
        CK(ctx, cudaMemcpyAsync(hpts.data(), pts, n_starts * 8, cudaMemcpyDeviceToHost, ctx->stream));
        CK(ctx, cudaStreamSynchronize(ctx->stream));
        for (uint64_t s = 0; s < n_starts; ++s) {
            hoff[s] = total;
            total += hlen[s];
        }
        seqs = (uint8_t*)B.get(std::max<uint64_t>(total, 1));
        if (!seqs) return set_err(ctx, FBK_ERR_OOM, "compaction sequences");
        CK(ctx, cudaMemcpyAsync(off, hoff.data(), n_starts * 8, cudaMemcpyHostToDevice, ctx->stream));
        TIMED(ctx, "compact_write", (k_walk_write<NW><<<L.grid, L.block, 0, L.stream>>>(R, k, starts, n_starts, len, off, seqs, visited,
                                                                                         ctx->d_status),
                                     cudaGetLastError()));
        TIMED(ctx, "compact_canon", (k_canon_seq<<<L.grid, L.block, 0, L.stream>>>(seqs, off, len, n_starts), cudaGetLastError()));
    }
    uint32_t bits = 0;
    fbk_status st = ctx_check_status(ctx, &bits);
    if (st) return st;
    if (bits) return set_err(ctx, FBK_ERR_INVALID, "compaction: node index full or a path longer than the node count");
    std::vector<uint8_t> hseq(total);
    if (total) CK(ctx, cudaMemcpyAsync(hseq.data(), seqs, total, cudaMemcpyDeviceToHost, ctx->stream));
    // isolated cycles: candidate rows to the host
    uint8_t* flag = (uint8_t*)B.get(n);
    if (!flag) return set_err(ctx, FBK_ERR_OOM, "compaction cycle flags");
    TIMED(ctx, "compact_cycles", (k_cycle_candidates<<<L.grid, L.block, 0, L.stream>>>(t->out_mask, visited, n, flag), cudaGetLastError()));
    std::vector<uint8_t> hflag(n);
    CK(ctx, cudaMemcpyAsync(hflag.data(), flag, n, cudaMemcpyDeviceToHost, ctx->stream));
    CK(ctx, cudaStreamSynchronize(ctx->stream));
    for (uint64_t s = 0; s < n_starts; ++s) {
        if (!hlen[s]) continue;
        HUnitig h;
        h.seq.assign((const char*)hseq.data() + hoff[s], hlen[s]);
        h.cov = std::max(1.0f, (float)hcs[s] / (float)hpts[s]);
        h.circular = false;
        U->bases += hlen[s];
        U->u.push_back(std::move(h));
    }
    std::vector<uint64_t> ck;
    std::vector<uint16_t> cc;
    std::vector<uint8_t> cm;
    std::vector<uint64_t> rows;
    for (uint64_t r = 0; r < n; ++r)
        if (hflag[r]) rows.push_back(r);
    U->cycle_candidates = rows.size();
    if (!rows.empty()) {
        // the candidates are gathered from a host copy of the rows (cycles are rare)
        std::vector<uint64_t> all_k(n * NW);
        std::vector<uint16_t> all_c(n);
        std::vector<uint8_t> all_m(n);
        CK(ctx, cudaMemcpyAsync(all_k.data(), t->out_keys, n * 8 * NW, cudaMemcpyDeviceToHost, ctx->stream));
        CK(ctx, cudaMemcpyAsync(all_c.data(), t->out_cov, n * 2, cudaMemcpyDeviceToHost, ctx->stream));
        CK(ctx, cudaMemcpyAsync(all_m.data(), t->out_mask, n, cudaMemcpyDeviceToHost, ctx->stream));
        CK(ctx, cudaStreamSynchronize(ctx->stream));
        ck.resize(rows.size() * NW);
        cc.resize(rows.size());
        cm.resize(rows.size());
        for (size_t i = 0; i < rows.size(); ++i) {
            for (int j = 0; j < NW; ++j) ck[i * NW + j] = all_k[rows[i] * NW + j];
            cc[i] = all_c[rows[i]];
            cm[i] = all_m[rows[i]];
        }
        const size_t before = U->u.size();
        host_cycles<NW>(k, ck, cc, cm, U->u);
        for (size_t i = before; i < U->u.size(); ++i) U->bases += U->u[i].seq.size();
    }
    link_unitigs(k, U);
    return FBK_OK;
}

}  // namespace

extern "C" {

FBK_API fbk_status fbk_compact(fbk_table* t, fbk_unitigs** out) {
    if (!t || !out) return FBK_ERR_INVALID;
    *out = nullptr;
    fbk_ctx* ctx = t->ctx;
    CK(ctx, cudaSetDevice(ctx->device));
    auto* U = new fbk_unitigs();
    fbk_status st = t->nw == 1 ? compact_impl<1>(t, U) : t->nw == 2 ? compact_impl<2>(t, U) : compact_impl<4>(t, U);
    if (st) {
        delete U;
        return st;
    }
    *out = U;
    return FBK_OK;
}

FBK_API fbk_status fbk_unitigs_info(const fbk_unitigs* u, uint64_t* n_unitigs, uint64_t* total_bases, uint64_t* n_edges) {
    if (!u) return FBK_ERR_INVALID;
    if (n_unitigs) *n_unitigs = u->u.size();
    if (total_bases) *total_bases = u->bases;
    if (n_edges) *n_edges = u->edges.size();
    return FBK_OK;
}

FBK_API fbk_status fbk_unitigs_export(const fbk_unitigs* u, uint8_t* ascii, uint64_t* offsets, float* cov, uint8_t* circular) {
    if (!u || !offsets) return FBK_ERR_INVALID;
    uint64_t p = 0;
    offsets[0] = 0;
    for (size_t i = 0; i < u->u.size(); ++i) {
        if (ascii) memcpy(ascii + p, u->u[i].seq.data(), u->u[i].seq.size());
        p += u->u[i].seq.size();
        offsets[i + 1] = p;
        if (cov) cov[i] = u->u[i].cov;
        if (circular) circular[i] = u->u[i].circular;
    }
    return FBK_OK;
}

FBK_API fbk_status fbk_unitigs_edges(const fbk_unitigs* u, uint32_t* edges, uint64_t cap, uint64_t* n_out) {
    if (!u || !n_out) return FBK_ERR_INVALID;
    const uint64_t n = std::min<uint64_t>(cap, u->edges.size());
    if (n && !edges) return FBK_ERR_INVALID;
    for (uint64_t i = 0; i < n; ++i) memcpy(edges + 6 * i, u->edges[i].data(), 24);
    *n_out = u->edges.size();
    return FBK_OK;
}

FBK_API fbk_status fbk_unitigs_release(fbk_unitigs* u) {
    delete u;
    return FBK_OK;
}

}  // extern "C"
