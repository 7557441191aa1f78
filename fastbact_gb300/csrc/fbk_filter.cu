// fbk_filter.cu — the multi-k upgrade's input filter (src/graph/local_multik.rs:259-333)
// on the device.
//
// filter_active_reads keeps the reads that touch unitig ends, branching junctions
// or unresolved regions: it indexes the canonical ntHash (k' = min(k, 31)) of every
// k'-mer of short (< 2000 bp), circular or branching unitigs and of the first and
// last 350 k'-mers of the other unitigs, then keeps a read when the ntHash at offset
// 0, (len - k') / 2 or len - k' is indexed; a pair is kept when either read is.
// Here the index is an open-addressing set of u64 hashes built on the device from the
// packed unitigs, and one thread tests each read of the device bank.
#include <algorithm>
#include <cstring>
#include <vector>

#include "fbk_device.cuh"
#include "fbk_internal.h"

using namespace fbk;

namespace {

constexpr uint64_t HSET_EMPTY = ~0ULL;

__global__ void k_hset_insert(const uint64_t* __restrict__ data, const uint64_t* __restrict__ win, uint64_t n_win, uint32_t k,
                              unsigned long long* set, uint64_t cap, uint32_t* flags) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n_win; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t h = nthash_canonical_at(data, win[i], k);
        if (h == HSET_EMPTY) {  // the one value the set cannot hold is kept as a flag
            atomicOr(flags, 1u);
            continue;
        }
        uint64_t s = smix(h) & (cap - 1);
        for (uint64_t probe = 0; probe < cap; ++probe) {
            const unsigned long long old = atomicCAS(&set[s], HSET_EMPTY, (unsigned long long)h);
            if (old == HSET_EMPTY || old == h) break;
            s = (s + 1) & (cap - 1);
        }
    }
}

__device__ __forceinline__ bool hset_has(const unsigned long long* set, uint64_t cap, uint32_t flags, uint64_t h) {
    if (h == HSET_EMPTY) return flags & 1u;
    uint64_t s = smix(h) & (cap - 1);
    for (uint64_t probe = 0; probe < cap; ++probe) {
        const uint64_t v = set[s];
        if (v == h) return true;
        if (v == HSET_EMPTY) return false;
        s = (s + 1) & (cap - 1);
    }
    return false;
}

// local_multik.rs:296-307: ntHash at offsets 0, (len - k) / 2 and len - k.
__global__ void k_active_reads(BankDev b, uint32_t k, const unsigned long long* __restrict__ set, uint64_t cap,
                               const uint32_t* __restrict__ flags, uint8_t* active) {
    const uint32_t fl = *flags;
    for (uint64_t r = b.r_begin + (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; r < b.r_end; r += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t len = b.len[r];
        bool a = false;
        if (len >= k) {
            const uint64_t off = b.off[r];
            const uint32_t offs[3] = {0u, (len - k) / 2, len - k};
            for (int j = 0; j < 3 && !a; ++j) a = hset_has(set, cap, fl, nthash_canonical_at(b.data, off + offs[j], k));
        }
        active[r] = a ? 1 : 0;
    }
}

}  // namespace

extern "C" {

FBK_API fbk_status fbk_filter_active_reads(fbk_ctx* ctx, const fbk_bank* bank, const uint8_t* unitig_ascii,
                                           const uint64_t* unitig_offsets, const uint8_t* circular, const uint32_t* edges_fwd,
                                           const uint32_t* edges_rev, uint64_t n_unitigs, uint32_t graph_k, uint8_t* keep_out,
                                           uint64_t* n_kept) {
    if (!ctx || !bank || !unitig_offsets || !keep_out || (n_unitigs && (!unitig_ascii || !circular || !edges_fwd || !edges_rev)))
        return FBK_ERR_INVALID;
    if (bank->arena_reads.size() != 3) return set_err(ctx, FBK_ERR_INVALID, "filter_active_reads needs a three-arena ReadBank");
    if (graph_k < 1) return set_err(ctx, FBK_ERR_INVALID, "graph k must be >= 1");
    CK(ctx, cudaSetDevice(ctx->device));
    CK(ctx, bank_wait(ctx, bank));
    const uint32_t k = std::min<uint32_t>(graph_k, 31);
    const uint64_t WINDOW = 350;
    // pack the unitigs (ASCII_TO_2BIT: A0 C1 G2 T3, anything else 0) and list the windows
    std::vector<uint64_t> words(8, 0), win;
    uint64_t pos = 0;
    auto push_base = [&](uint8_t c) {
        const uint64_t code = c == 'C' || c == 'c' ? 1 : c == 'G' || c == 'g' ? 2 : c == 'T' || c == 't' ? 3 : 0;
        if ((pos >> 5) + 8 >= words.size()) words.resize(words.size() * 2 + 16, 0);
        words[pos >> 5] |= code << ((pos & 31) * 2);
        ++pos;
    };
    for (uint64_t u = 0; u < n_unitigs; ++u) {
        const uint64_t a = unitig_offsets[u], e = unitig_offsets[u + 1], len = e - a;
        const uint64_t base = pos;
        for (uint64_t i = a; i < e; ++i) push_base(unitig_ascii[i]);
        if (len < k) continue;
        const uint64_t nk = len - k + 1;
        if (len < 2000 || circular[u] || edges_fwd[u] > 1 || edges_rev[u] > 1) {
            for (uint64_t i = 0; i < nk; ++i) win.push_back(base + i);
        } else {
            const uint64_t left = std::min<uint64_t>(WINDOW, nk);
            for (uint64_t i = 0; i < left; ++i) win.push_back(base + i);
            const uint64_t right = std::min<uint64_t>(len > WINDOW ? len - WINDOW : 0, len - k);
            for (uint64_t i = right; i < nk; ++i) win.push_back(base + i);
        }
    }
    const uint64_t n_words = (pos + 31) / 32 + 8;
    uint64_t cap = 1024;
    while (cap < 2 * win.size()) cap <<= 1;
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
    uint64_t* d_words = (uint64_t*)B.get(n_words * 8);
    uint64_t* d_win = (uint64_t*)B.get(std::max<uint64_t>(win.size(), 1) * 8);
    unsigned long long* set = (unsigned long long*)B.get(cap * 8);
    uint32_t* flags = (uint32_t*)B.get(256);
    uint8_t* active = (uint8_t*)B.get(std::max<uint64_t>(bank->n_reads, 1));
    if (!d_words || !d_win || !set || !flags || !active) return set_err(ctx, FBK_ERR_OOM, "filter_active_reads buffers");
    words.resize(n_words, 0);
    CK(ctx, cudaMemcpyAsync(d_words, words.data(), n_words * 8, cudaMemcpyHostToDevice, ctx->stream));
    if (!win.empty()) CK(ctx, cudaMemcpyAsync(d_win, win.data(), win.size() * 8, cudaMemcpyHostToDevice, ctx->stream));
    CK(ctx, cudaMemsetAsync(set, 0xFF, cap * 8, ctx->stream));
    CK(ctx, cudaMemsetAsync(flags, 0, 4, ctx->stream));
    Launch L = launch_cfg(ctx, 256, 0);
    if (!win.empty())
        TIMED(ctx, "filter_index", (k_hset_insert<<<L.grid, L.block, 0, L.stream>>>(d_words, d_win, win.size(), k, set, cap, flags),
                                    cudaGetLastError()));
    if (bank->n_reads)
        TIMED(ctx, "filter_reads", (k_active_reads<<<L.grid, L.block, 0, L.stream>>>(bank_view(bank, 0, bank->n_reads, nullptr), k, set,
                                                                                    cap, flags, active),
                                    cudaGetLastError()));
    std::vector<uint8_t> act(bank->n_reads);
    if (bank->n_reads) CK(ctx, cudaMemcpyAsync(act.data(), active, bank->n_reads, cudaMemcpyDeviceToHost, ctx->stream));
    CK(ctx, cudaStreamSynchronize(ctx->stream));
    // local_multik.rs:309-329: merged reads on their own, pairs together
    const uint64_t M = bank->arena_reads[0], F = bank->arena_reads[1], R = bank->arena_reads[2];
    uint64_t kept = 0;
    for (uint64_t i = 0; i < M; ++i) kept += keep_out[i] = act[i];
    const uint64_t pe = std::min(F, R);
    for (uint64_t i = 0; i < F; ++i) keep_out[M + i] = 0;
    for (uint64_t i = 0; i < R; ++i) keep_out[M + F + i] = 0;
    for (uint64_t i = 0; i < pe; ++i) {
        const uint8_t kp = act[M + i] | act[M + F + i];
        keep_out[M + i] = keep_out[M + F + i] = kp;
        kept += 2 * kp;
    }
    if (n_kept) *n_kept = kept;
    return FBK_OK;
}

}  // extern "C"

// ===========================================================================
// index_terminal_kmers (src/resolve/mapper.rs:89-136): the canonical k-mers (folded to
// u64, KmerInt::to_u64) of the first and last 1000 k-mers of every unitig (all of them
// when it has at most 2000), kept when they occur exactly once, with the unitig strand
// (DirUnitigId(id, is_rc)) and the k-mer's position.  A device map counts every key;
// the value written by a key's only occurrence is the one kept.
// ===========================================================================
namespace {

struct TermWindow {
    uint64_t g;     // first base in the packed unitigs
    uint32_t unitig, pos;
};

template <int NW>
__global__ void k_term_insert(const uint64_t* __restrict__ data, const TermWindow* __restrict__ win, uint64_t n_win, uint32_t k,
                              unsigned long long* keys, uint32_t* cnt, uint64_t* vals, uint64_t cap, unsigned long long* full_fold) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n_win; i += (uint64_t)gridDim.x * blockDim.x) {
        const TermWindow w = win[i];
        Key<NW> can;
        bool rc;
        window_canonical<NW>(data, w.g, k, can, rc);
        const uint64_t h = key_fold<NW>(can);
        const uint64_t v = ((uint64_t)w.unitig << 33) | ((uint64_t)(rc ? 1 : 0) << 32) | w.pos;
        if (h == HSET_EMPTY) {  // the fold the map cannot hold as a key: counted in slot 0 of full_fold
            atomicAdd(&full_fold[0], 1ULL);
            full_fold[1] = v;
            continue;
        }
        uint64_t s = smix(h) & (cap - 1);
        for (uint64_t probe = 0; probe < cap; ++probe) {
            const unsigned long long old = atomicCAS(&keys[s], HSET_EMPTY, (unsigned long long)h);
            if (old == HSET_EMPTY || old == h) {
                atomicAdd(&cnt[s], 1u);
                vals[s] = v;
                break;
            }
            s = (s + 1) & (cap - 1);
        }
    }
}

}  // namespace

extern "C" {

FBK_API fbk_status fbk_index_terminal_kmers(fbk_ctx* ctx, const uint8_t* unitig_ascii, const uint64_t* unitig_offsets,
                                            uint64_t n_unitigs, uint32_t k, uint32_t key_bits, uint64_t* keys_out,
                                            uint32_t* unitig_out, uint8_t* is_rc_out, uint32_t* pos_out, uint64_t cap_out,
                                            uint64_t* n_out) {
    if (!ctx || !unitig_offsets || !n_out || (n_unitigs && !unitig_ascii)) return FBK_ERR_INVALID;
    const int nw = key_bits == 64 ? 1 : key_bits == 128 ? 2 : key_bits == 256 ? 4 : 0;
    if (!nw || k < 1 || k > (uint32_t)(32 * nw - 1)) return set_err(ctx, FBK_ERR_INVALID, "k out of range for key_bits");
    CK(ctx, cudaSetDevice(ctx->device));
    std::vector<uint64_t> words(8, 0);
    std::vector<TermWindow> win;
    uint64_t pos = 0;
    for (uint64_t u = 0; u < n_unitigs; ++u) {
        const uint64_t a = unitig_offsets[u], e = unitig_offsets[u + 1], len = e - a, base = pos;
        for (uint64_t i = a; i < e; ++i) {
            const uint8_t c = unitig_ascii[i];
            const uint64_t code = c == 'C' || c == 'c' ? 1 : c == 'G' || c == 'g' ? 2 : c == 'T' || c == 't' ? 3 : 0;
            if ((pos >> 5) + 8 >= words.size()) words.resize(words.size() * 2 + 16, 0);
            words[pos >> 5] |= code << ((pos & 31) * 2);
            ++pos;
        }
        if (len < k) continue;
        const uint64_t total = len - k + 1;
        if (total <= 2000) {
            for (uint64_t i = 0; i < total; ++i) win.push_back({base + i, (uint32_t)u, (uint32_t)i});
        } else {
            for (uint64_t i = 0; i < 1000; ++i) win.push_back({base + i, (uint32_t)u, (uint32_t)i});
            for (uint64_t i = total - 1000; i < total; ++i) win.push_back({base + i, (uint32_t)u, (uint32_t)i});
        }
    }
    const uint64_t n_words = (pos + 31) / 32 + 8;
    words.resize(n_words, 0);
    uint64_t cap = 1024;
    while (cap < 2 * win.size()) cap <<= 1;
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
    uint64_t* d_words = (uint64_t*)B.get(n_words * 8);
    TermWindow* d_win = (TermWindow*)B.get(std::max<uint64_t>(win.size(), 1) * sizeof(TermWindow));
    unsigned long long* keys = (unsigned long long*)B.get(cap * 8);
    uint32_t* cnt = (uint32_t*)B.get(cap * 4);
    uint64_t* vals = (uint64_t*)B.get(cap * 8);
    unsigned long long* ff = (unsigned long long*)B.get(64);
    if (!d_words || !d_win || !keys || !cnt || !vals || !ff) return set_err(ctx, FBK_ERR_OOM, "terminal k-mer index buffers");
    CK(ctx, cudaMemcpyAsync(d_words, words.data(), n_words * 8, cudaMemcpyHostToDevice, ctx->stream));
    if (!win.empty()) CK(ctx, cudaMemcpyAsync(d_win, win.data(), win.size() * sizeof(TermWindow), cudaMemcpyHostToDevice, ctx->stream));
    CK(ctx, cudaMemsetAsync(keys, 0xFF, cap * 8, ctx->stream));
    CK(ctx, cudaMemsetAsync(cnt, 0, cap * 4, ctx->stream));
    CK(ctx, cudaMemsetAsync(ff, 0, 64, ctx->stream));
    Launch L = launch_cfg(ctx, 256, 0);
    if (!win.empty()) {
        cudaError_t e = cudaSuccess;
        TimedLaunch tl;
        time_begin(ctx, "term_index", tl);
        if (nw == 1) k_term_insert<1><<<L.grid, L.block, 0, L.stream>>>(d_words, d_win, win.size(), k, keys, cnt, vals, cap, ff);
        else if (nw == 2) k_term_insert<2><<<L.grid, L.block, 0, L.stream>>>(d_words, d_win, win.size(), k, keys, cnt, vals, cap, ff);
        else k_term_insert<4><<<L.grid, L.block, 0, L.stream>>>(d_words, d_win, win.size(), k, keys, cnt, vals, cap, ff);
        e = cudaGetLastError();
        time_end(ctx, tl);
        if (e != cudaSuccess) return cuda_err(ctx, e, "term_index");
    }
    std::vector<unsigned long long> hk(cap);
    std::vector<uint32_t> hc(cap);
    std::vector<uint64_t> hv(cap);
    unsigned long long hff[2] = {0, 0};
    CK(ctx, cudaMemcpyAsync(hk.data(), keys, cap * 8, cudaMemcpyDeviceToHost, ctx->stream));
    CK(ctx, cudaMemcpyAsync(hc.data(), cnt, cap * 4, cudaMemcpyDeviceToHost, ctx->stream));
    CK(ctx, cudaMemcpyAsync(hv.data(), vals, cap * 8, cudaMemcpyDeviceToHost, ctx->stream));
    CK(ctx, cudaMemcpyAsync(hff, ff, 16, cudaMemcpyDeviceToHost, ctx->stream));
    CK(ctx, cudaStreamSynchronize(ctx->stream));
    std::vector<std::pair<uint64_t, uint64_t>> uniq;
    for (uint64_t s = 0; s < cap; ++s)
        if (hk[s] != HSET_EMPTY && hc[s] == 1) uniq.push_back({hk[s], hv[s]});
    if (hff[0] == 1) uniq.push_back({HSET_EMPTY, hff[1]});
    std::sort(uniq.begin(), uniq.end());
    const uint64_t n = std::min<uint64_t>(cap_out, uniq.size());
    for (uint64_t i = 0; i < n; ++i) {
        if (keys_out) keys_out[i] = uniq[i].first;
        if (unitig_out) unitig_out[i] = (uint32_t)(uniq[i].second >> 33);
        if (is_rc_out) is_rc_out[i] = (uint8_t)((uniq[i].second >> 32) & 1);
        if (pos_out) pos_out[i] = (uint32_t)uniq[i].second;
    }
    *n_out = uniq.size();
    return FBK_OK;
}

}  // extern "C"
