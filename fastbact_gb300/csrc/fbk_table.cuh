// fbk_table.cuh — device pieces shared by the single-isolate and the multi-isolate
// build kernels: open-addressing probes of the solid table, the solidity-bitmap
// test, and the per-warp record staging of pass 2.
#pragma once
#include <cuda/atomic>

#include "fbk_device.cuh"
#include "fbk_kernels.cuh"

namespace fbk {

static constexpr uint64_t FP_SALT = 0xbb67ae8584caa73bULL;
static constexpr uint64_t TAG_READY = 1ULL << 63;
static constexpr uint64_t KEY_EMPTY = ~0ULL;

// ---------------------------------------------------------------------------
// Solid table probing from a precomputed home slot
// ---------------------------------------------------------------------------
// Home slot of a key: the high 64 bits of h * cap (any capacity), h = splitmix64 of
// the folded key with the sketch's row-0 seed — the hash the gate already computes
// for row 0, whose column is its low bits, so the record emit reuses it.
__device__ __forceinline__ uint64_t home_slot_h(uint64_t h_row0, uint64_t cap) { return __umul64hi(h_row0, cap); }
__device__ __forceinline__ uint64_t home_slot(uint64_t fold, uint64_t cap) {
    return home_slot_h(smix(fold ^ cms_seed(0)), cap);
}
// Record bucket of a key: the same hash scaled to the bucket count, so that bucket b
// holds the keys whose home slots lie in [b cap / P, (b + 1) cap / P) whatever the
// capacity.
__device__ __forceinline__ uint32_t bucket_of_h(uint64_t h_row0, uint32_t n_buckets) {
    return (uint32_t)__umul64hi(h_row0, n_buckets);
}
__device__ __forceinline__ uint32_t bucket_of(uint64_t fold, uint32_t n_buckets) {
    return bucket_of_h(smix(fold ^ cms_seed(0)), n_buckets);
}

__device__ __forceinline__ int64_t table_slot1(const TableDev& t, uint64_t key, uint64_t s, uint32_t* status) {
    for (uint32_t probe = 0; probe < t.max_probe; ++probe) {
        const uint64_t cur = __ldcg(&t.keys[s]);
        if (cur == key) return (int64_t)s;
        if (cur == KEY_EMPTY) {
            const uint64_t old = atomicCAS((unsigned long long*)&t.keys[s], KEY_EMPTY, key);
            if (old == KEY_EMPTY || old == key) return (int64_t)s;
        }
        s = s + 1 == t.cap ? 0 : s + 1;
    }
    atomicOr(status, ST_TABLE_FULL);
    return -1;
}

// 16-byte compare-and-swap (sm_90 and later): the 128-bit key of a slot goes from
// EMPTY (all ones: a k <= 63 key leaves its top two bits zero) to the key in one
// atomic step, so a slot never holds half a key and no publication wait is needed.
__device__ __forceinline__ void cas128(uint64_t* addr, uint64_t cmp_lo, uint64_t cmp_hi, uint64_t new_lo, uint64_t new_hi,
                                       uint64_t& old_lo, uint64_t& old_hi) {
    asm volatile(
        "{\n\t.reg .b128 c, n, d;\n\t"
        "mov.b128 c, {%2, %3};\n\t"
        "mov.b128 n, {%4, %5};\n\t"
        "atom.global.cas.b128 d, [%6], c, n;\n\t"
        "mov.b128 {%0, %1}, d;\n\t}"
        : "=l"(old_lo), "=l"(old_hi)
        : "l"(cmp_lo), "l"(cmp_hi), "l"(new_lo), "l"(new_hi), "l"(addr)
        : "memory");
}

// A slot goes from EMPTY to its key in one 16-byte CAS and never changes again, so a
// word read that is neither EMPTY nor ours proves the slot belongs to another key and
// needs no CAS.  Word 0 of a k <= 63 key is below 2^62, so word 0 != EMPTY proves the
// slot is claimed; word 1 can be all ones in a real key (a 32-base poly-T suffix), so a
// word 1 of EMPTY proves nothing and such slots, like every EMPTY-looking one, are
// decided by the CAS, which returns the slot's whole current value.  A key whose word 1
// is all ones is also confirmed by the CAS when it seems found, since a read of the two
// words could straddle another key's claim.
__device__ __forceinline__ int64_t table_slot2(const TableDev& t, const Key<2>& key, uint64_t s, uint32_t* status) {
    const bool w1_empty = key.w[1] == KEY_EMPTY;
    for (uint32_t probe = 0; probe < t.max_probe; ++probe) {
        uint64_t* a = t.keys + s * 2;
        const ulonglong2 c = __ldcg(reinterpret_cast<const ulonglong2*>(a));
        const bool other = (c.x != KEY_EMPTY && c.x != key.w[0]) || (c.y != KEY_EMPTY && c.y != key.w[1]);
        if (!other) {
            if (c.x == key.w[0] && c.y == key.w[1] && !w1_empty) return (int64_t)s;
            uint64_t o0, o1;
            cas128(a, KEY_EMPTY, KEY_EMPTY, key.w[0], key.w[1], o0, o1);
            if ((o0 == KEY_EMPTY && o1 == KEY_EMPTY) || (o0 == key.w[0] && o1 == key.w[1])) return (int64_t)s;
        }
        s = s + 1 == t.cap ? 0 : s + 1;
    }
    atomicOr(status, ST_TABLE_FULL);
    return -1;
}

template <int NW>
__device__ __forceinline__ int64_t table_slotw(const TableDev& t, const Key<NW>& key, uint64_t f, uint64_t s, uint32_t* status) {
    const uint64_t fp = (smix(f ^ FP_SALT) | 1ULL) & ~TAG_READY;
    // with the tag in word 0 (tag_stride == NW) the key's word 0 is zero and not stored
    const int w0 = t.tag_stride == NW ? 1 : 0;
    for (uint32_t probe = 0; probe < t.max_probe; ++probe) {
        unsigned long long* tp = (unsigned long long*)&t.tags[s * t.tag_stride];
        cuda::atomic_ref<unsigned long long, cuda::thread_scope_device> tag_ref(*tp);
        uint64_t tag = tag_ref.load(cuda::memory_order_acquire);
        if (tag == 0) {
            const uint64_t old = atomicCAS(tp, 0ULL, fp);
            if (old == 0) {
#pragma unroll
                for (int i = 0; i < NW; ++i)
                    if (i >= w0) __stcg(&t.keys[s * NW + i], key.w[i]);
                tag_ref.fetch_or(TAG_READY, cuda::memory_order_release);
                return (int64_t)s;
            }
            tag = old;
        }
        if ((tag & ~TAG_READY) == fp) {
            // Same fingerprint: wait (bounded) until the claiming thread has published
            // the key words, then compare them.
            uint32_t spins = 0;
            while (!(tag & TAG_READY)) {
                if (++spins > t.spin_limit) {
                    atomicOr(status, ST_SPIN_TIMEOUT);
                    return -1;
                }
                __nanosleep(64);
                tag = tag_ref.load(cuda::memory_order_acquire);
            }
            bool eq = true;
#pragma unroll
            for (int i = 0; i < NW; ++i)
                if (i >= w0) eq &= (__ldcg(&t.keys[s * NW + i]) == key.w[i]);
            if (eq) return (int64_t)s;
        }
        s = s + 1 == t.cap ? 0 : s + 1;
    }
    atomicOr(status, ST_TABLE_FULL);
    return -1;
}


// The ladder gate of pass 2 (fbk_k_ladder.cu) for one window, in two halves so that
// the four L2 loads can be in flight while other work runs: gate_issue hashes the key
// for the four rows and loads the top level's words, gate_resolve tests the bits.
struct GateLoads {
    uint32_t w[4];  // the loaded words of the four rows
    uint32_t bits;  // each row's bit within its word, 5 bits per row (one register, not four)
    uint64_t h0;    // row-0 hash, which also places the key in the table (home_slot_h)
};
__device__ __forceinline__ void gate_issue(const uint32_t* __restrict__ top, uint32_t log2w, uint64_t key, bool live, GateLoads& g) {
    const uint64_t wmask = (1ULL << log2w) - 1;
    g.bits = 0;
    uint64_t hr[4];
    cms_row_hashes(key, hr);
    g.h0 = hr[0];
#pragma unroll
    for (int row = 0; row < 4; ++row) {
        const uint32_t bit = ((uint32_t)row << log2w) + (uint32_t)(hr[row] & wmask);
        g.bits |= (bit & 31u) << (5 * row);
        g.w[row] = live ? __ldg(top + (bit >> 5)) : 0u;
    }
}
__device__ __forceinline__ bool gate_resolve(const GateLoads& g, bool live) {
    bool ok = live;
#pragma unroll
    for (int row = 0; row < 4; ++row) ok &= ((g.w[row] >> ((g.bits >> (5 * row)) & 31u)) & 1u) != 0;
    return ok;
}

__device__ __forceinline__ bool bm_bit(const uint32_t* __restrict__ bm, uint64_t g) {
    return (__ldg(&bm[g >> 5]) >> (g & 31)) & 1u;
}

// Writes a record (key, info byte) in the bucket's layout at dst.  WS_T >= 0 is the
// word shift known at compile time (it equals bk.ws); -1 reads it from bk.
template <int NW, int WS_T = -1>
__device__ __forceinline__ void rec_put(uint64_t* dst, const Key<NW>& key, uint32_t info, const BucketDev& bk) {
    const uint32_t ws = WS_T >= 0 ? (uint32_t)WS_T : bk.ws;
    const uint32_t base = bk.packed ? 0u : 1u;
    if (!bk.packed) dst[0] = info;
#pragma unroll
    for (int i = 0; i < NW; ++i)
        if ((uint32_t)i >= ws)
            dst[base + i - ws] = key.w[i] | ((bk.packed && (uint32_t)i == ws) ? ((uint64_t)info << 56) : 0ULL);
}
// Reads a record written by rec_put; returns its info byte.  Streaming loads (every
// record is read once), or with CACHED loads through L1 for a record read twice.
template <int NW, bool CACHED = false>
__device__ __forceinline__ uint64_t rec_word(const uint64_t* p) {
    if constexpr (CACHED) return __ldg(p);
    else return __ldcs(p);
}
template <int NW, bool CACHED = false>
__device__ __forceinline__ uint32_t rec_get(const uint64_t* src, Key<NW>& key, const BucketDev& bk) {
    const uint32_t ws = bk.ws, base = bk.packed ? 0u : 1u;
    uint32_t info = 0;
    if (!bk.packed) info = (uint32_t)rec_word<NW, CACHED>(src);
#pragma unroll
    for (int i = 0; i < NW; ++i) {
        uint64_t w = 0;
        if ((uint32_t)i >= ws) w = rec_word<NW, CACHED>(src + base + i - ws);
        if (bk.packed && (uint32_t)i == ws) {
            info = (uint32_t)(w >> 56);
            w &= (1ULL << 56) - 1;
        }
        key.w[i] = w;
    }
    return info;
}
// The key of a record only (the record filter's count).
template <int NW>
__device__ __forceinline__ void rec_key(const uint64_t* src, Key<NW>& key, const BucketDev& bk) {
    const uint32_t ws = bk.ws, base = bk.packed ? 0u : 1u;
#pragma unroll
    for (int i = 0; i < NW; ++i) {
        uint64_t w = 0;
        if ((uint32_t)i >= ws) w = __ldcg(src + base + i - ws);
        if (bk.packed && (uint32_t)i == ws) w &= (1ULL << 56) - 1;
        key.w[i] = w;
    }
}

// Records are staged per warp in shared memory (emit_buf(NW) of them) and flushed
// bucket by bucket: one atomic per (flush, bucket) reserves room for all of the
// warp's records of that bucket, which are then written as one run.
// Records staged per warp.  Staging 2-3.5 times as many per warp (9 KB of shared
// memory per warp) made the emit 3-40% slower: the shared memory comes out of the L1
// that serves the bank and gate loads.
__host__ __device__ constexpr uint32_t emit_buf(int) { return 128u; }
constexpr uint32_t EMIT_MAX_BUCKETS = 64;
// staging words per warp: records (NW + 1 words apart, bk.rw of them used), bucket
// bytes, ranks (u16), histogram (64 u32), reservation bases (64 u64), bucket-order
// permutation (u16)
#define EMIT_WARP_WORDS(NW) \
    (emit_buf(NW) * ((NW) + 1) + emit_buf(NW) / 8 + emit_buf(NW) / 4 + EMIT_MAX_BUCKETS / 2 + EMIT_MAX_BUCKETS + emit_buf(NW) / 4)

// Warp counting sort of the staged records by bucket: a shared-memory histogram
// (one atomic per record), one round of global reservations (lane j reserves for
// buckets j and j + 32), a warp scan of the counts that places every record in
// bucket order, then a copy in that order, so the records of a bucket leave as one
// contiguous run of stores.
template <int NW>
__device__ __forceinline__ void emit_flush(const BucketDev& bk, uint32_t stripe, uint32_t lane, uint64_t* buf, const uint8_t* bbuf,
                                           uint32_t n_buf, uint32_t* hist, unsigned long long* gbase, uint16_t* rank,
                                           uint16_t* perm) {
    constexpr uint32_t SW = NW + 1;  // staging stride in words
    const uint32_t RW = bk.rw;       // words per record (<= SW)
    const uint32_t nb = bk.n_buckets;  // <= EMIT_MAX_BUCKETS = 64
    for (uint32_t bu = lane; bu < nb; bu += 32) hist[bu] = 0;
    __syncwarp();
    for (uint32_t j = lane; j < n_buf; j += 32) rank[j] = (uint16_t)atomicAdd(&hist[bbuf[j]], 1u);
    __syncwarp();
    const uint32_t c0 = lane < nb ? hist[lane] : 0u, c1 = lane + 32 < nb ? hist[lane + 32] : 0u;
    if (c0) gbase[lane] = atomicAdd(bk.fill + (uint64_t)lane * bk.stripes + stripe, (unsigned long long)c0);
    if (c1) gbase[lane + 32] = atomicAdd(bk.fill + (uint64_t)(lane + 32) * bk.stripes + stripe, (unsigned long long)c1);
    uint32_t s0 = c0, s1 = c1;  // inclusive scans over the lanes
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        const uint32_t a = __shfl_up_sync(0xffffffffu, s0, off), b = __shfl_up_sync(0xffffffffu, s1, off);
        if (lane >= (uint32_t)off) {
            s0 += a;
            s1 += b;
        }
    }
    const uint32_t tot0 = __shfl_sync(0xffffffffu, s0, 31);
    __syncwarp();
    if (lane < nb) hist[lane] = s0 - c0;  // first bucket-order position of each bucket
    if (lane + 32 < nb) hist[lane + 32] = tot0 + s1 - c1;
    __syncwarp();
    for (uint32_t j = lane; j < n_buf; j += 32) perm[hist[bbuf[j]] + rank[j]] = (uint16_t)j;
    __syncwarp();
    if (RW <= 2) {
        // lane p writes the p-th record in bucket order: a store instruction covers one
        // word of 32 consecutive records of the runs
        for (uint32_t p = lane; p < n_buf; p += 32) {
            const uint32_t j = perm[p], bu = bbuf[j];
            const unsigned long long pos = gbase[bu] + (p - hist[bu]);
            if (pos < bk.stripe_cap) {
                uint64_t* dst = bk.recs + (((uint64_t)bu * bk.stripes + stripe) * bk.stripe_cap + pos) * RW;
                dst[0] = buf[j * SW];
                if (RW == 2) dst[1] = buf[j * SW + 1];
            } else {
                atomicOr(bk.overflow, 1u);
            }
        }
    } else {
        // records of 3 words or more: one word per lane, 32 consecutive words per store
        for (uint32_t w = lane; w < n_buf * RW; w += 32) {
            const uint32_t p = w / RW, i = w - p * RW;
            const uint32_t j = perm[p], bu = bbuf[j];
            const unsigned long long pos = gbase[bu] + (p - hist[bu]);
            if (pos < bk.stripe_cap) bk.recs[(((uint64_t)bu * bk.stripes + stripe) * bk.stripe_cap + pos) * RW + i] = buf[j * SW + i];
            else if (i == 0) atomicOr(bk.overflow, 1u);
        }
    }
    __syncwarp();
}

}  // namespace fbk
