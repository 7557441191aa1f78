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
