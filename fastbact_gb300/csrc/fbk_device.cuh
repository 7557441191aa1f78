// fbk_device.cuh — device primitives of the k-mer counting front end (sm_103a).
//
// K-mers are read straight out of the 2-bit packed bank: the window of k bases that
// starts at base g is the 2k-bit field at bit 2g of the LSB-first stream
// (src/common/bitseq.rs:213-219).  From that field W:
//   rc  = ~W masked to 2k bits          (kmer.rs:99-101, 158-178, 260-305)
//   fwd = W with its 2-bit groups reversed, as the MSB-first integer of
//         KmerInt::from_ascii (kmer.rs:73-81, 132-140, 210-222)
// so every lane computes its own window with no rolling dependency; the values are
// identical to RollingKmer::roll_next's (kmer.rs:104-112, 181-189, 307-329).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace fbk {

// splitmix64 finaliser — src/common/sketch.rs:13-18
__host__ __device__ __forceinline__ uint64_t smix(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
    return z ^ (z >> 31);
}

// CMS row seeds — sketch.rs:122-127
__host__ __device__ __forceinline__ constexpr uint64_t cms_seed(int r) {
    return r == 0 ? 0x243f6a8885a308d3ULL : r == 1 ? 0x13198a2e03707344ULL : r == 2 ? 0xa4093822299f31d0ULL : 0x082efa98ec4e6c89ULL;
}

// The four row hashes smix(key ^ seed_r) of the sketch (sketch.rs:191-223).  The first
// xor-shift distributes over the xor with the seed, (x ^ s) ^ ((x ^ s) >> 30) =
// (x ^ (x >> 30)) ^ (s ^ (s >> 30)), so it is done once for the four rows and each row
// xors a folded seed.
__host__ __device__ __forceinline__ constexpr uint64_t cms_seed_folded(int r) {
    return cms_seed(r) ^ (cms_seed(r) >> 30);
}
__host__ __device__ __forceinline__ void cms_row_hashes(uint64_t key, uint64_t (&h)[4]) {
    const uint64_t x = key ^ (key >> 30);
#pragma unroll
    for (int r = 0; r < 4; ++r) {
        uint64_t z = (x ^ cms_seed_folded(r)) * 0xbf58476d1ce4e5b9ULL;
        z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
        h[r] = z ^ (z >> 31);
    }
}

// ntHash seeds — kmer.rs:385-391 (REV[c] == FWD[3-c])
__host__ __device__ __forceinline__ uint64_t nt_fwd(uint32_t c) {
    return (c & 2) ? ((c & 1) ? 0x295c504fac61002eULL : 0x20323ee046061444ULL)
                   : ((c & 1) ? 0x3193c18562a02b4cULL : 0x3c8bfbb395c60474ULL);
}
__host__ __device__ __forceinline__ uint64_t rotl64(uint64_t x, uint32_t r) {
    r &= 63;
    return (x << r) | (x >> ((64 - r) & 63));
}
__host__ __device__ __forceinline__ uint64_t rotr64(uint64_t x, uint32_t r) {
    r &= 63;
    return (x >> r) | (x << ((64 - r) & 63));
}

// Reverses the order of the 32 2-bit groups of x.
__device__ __forceinline__ uint64_t rev2(uint64_t x) {
    x = __brevll(x);
    return ((x >> 1) & 0x5555555555555555ULL) | ((x & 0x5555555555555555ULL) << 1);
}

// 64 bits of the packed stream starting at base g (bases g .. g+31).  The bank
// buffer carries 8 zero words of padding, so word g/32+1 always exists.
__device__ __forceinline__ uint64_t bits_at(const uint64_t* __restrict__ d, uint64_t g) {
    const uint64_t wi = g >> 5;
    const uint32_t sh = (uint32_t)(g & 31) << 1;
    const uint64_t lo = d[wi], hi = d[wi + 1];
    return (lo >> sh) | ((hi << (63 - sh)) << 1);
}
__device__ __forceinline__ uint32_t base_at(const uint64_t* __restrict__ d, uint64_t g) {
    return (uint32_t)(d[g >> 5] >> ((g & 31) << 1)) & 3u;
}

// Canonical k-mer of NW 64-bit words, big-endian (w[0] most significant), the word
// order of [u64; 4] in kmer.rs:199.
template <int NW>
struct Key {
    uint64_t w[NW];
};

template <int NW>
__device__ __forceinline__ bool key_less(const Key<NW>& a, const Key<NW>& b) {
#pragma unroll
    for (int i = 0; i < NW; ++i)
        if (a.w[i] != b.w[i]) return a.w[i] < b.w[i];
    return false;
}
template <int NW>
__device__ __forceinline__ bool key_eq(const Key<NW>& a, const Key<NW>& b) {
    bool e = true;
#pragma unroll
    for (int i = 0; i < NW; ++i) e &= (a.w[i] == b.w[i]);
    return e;
}
// KmerInt::to_u64 — kmer.rs:115-117 (u64), 192-194 (lo^hi), 332-334 (xor of 4 words)
template <int NW>
__device__ __forceinline__ uint64_t key_fold(const Key<NW>& a) {
    uint64_t f = 0;
#pragma unroll
    for (int i = 0; i < NW; ++i) f ^= a.w[i];
    return f;
}

// Mask for LSB-first word i of a 2k-bit field.
__device__ __forceinline__ uint64_t field_mask(uint32_t k, int i) {
    const int bits = (int)(2 * k) - 64 * i;
    return bits >= 64 ? ~0ULL : bits <= 0 ? 0ULL : ((1ULL << bits) - 1);
}

// Canonical k-mer (min(fwd, rc), rc chosen iff rc < fwd — build.rs:102,258) of the
// window starting at base g, for a word shift WS = (64*NW - 2k) / 64 known at compile
// time: the 2k-bit field covers NK = NW - WS words, so only NK + 1 packed words are
// read and reversed, and every register index is a constant.
template <int NW, int WS>
__device__ __forceinline__ void canonical_ws(const uint64_t* __restrict__ d, uint64_t g, uint32_t k, Key<NW>& can,
                                             bool& is_rc) {
    constexpr int NK = NW - WS;
    const uint64_t wi = g >> 5;
    const uint32_t sh = (uint32_t)(g & 31) << 1;
    // bases g .. g + 32 NK - 1 (the bank carries 8 zero words of padding)
    uint64_t D[NK + 1], W[NK], R[NK];
#pragma unroll
    for (int i = 0; i <= NK; ++i) D[i] = d[wi + i];
#pragma unroll
    for (int i = 0; i < NK; ++i) {
        W[i] = (D[i] >> sh) | ((D[i + 1] << (63 - sh)) << 1);
        R[i] = rev2(W[i]);
    }
    // fwd: full group reversal of the field (R), then a right shift by
    // s = 64*NW - 2k bits across big-endian words: word j takes R[j - WS] >> bs and
    // the low bits of R[j - WS - 1]
    const uint32_t bs = (64u * NW - 2u * k) & 63;
    Key<NW> fwd, rc;
#pragma unroll
    for (int j = 0; j < NW; ++j) {
        const uint64_t hi = j - WS >= 0 ? R[j - WS >= 0 ? j - WS : 0] : 0ULL;
        const uint64_t lo = j - WS - 1 >= 0 ? R[j - WS - 1 >= 0 ? j - WS - 1 : 0] : 0ULL;
        fwd.w[j] = (hi >> bs) | (bs ? (lo << (64 - bs)) : 0ULL);
    }
    // rc: ~W masked to 2k bits; LSB-first word i is big-endian word NW-1-i.
#pragma unroll
    for (int i = 0; i < NW; ++i) rc.w[NW - 1 - i] = i < NK ? (~W[i < NK ? i : 0]) & field_mask(k, i) : 0ULL;
    is_rc = key_less<NW>(rc, fwd);
    can = is_rc ? rc : fwd;
}

// Canonical k-mer of the window at g for any k <= 32*NW - 1: the word shift is the
// same for every window of a launch, so the branch below never diverges.
template <int NW>
__device__ __forceinline__ void window_canonical(const uint64_t* __restrict__ d, uint64_t g, uint32_t k, Key<NW>& can,
                                                 bool& is_rc) {
    const uint32_t ws = (64u * NW - 2u * k) >> 6;
    if constexpr (NW == 1) {
        canonical_ws<1, 0>(d, g, k, can, is_rc);
    } else if constexpr (NW == 2) {
        if (ws == 0) canonical_ws<2, 0>(d, g, k, can, is_rc);
        else canonical_ws<2, 1>(d, g, k, can, is_rc);
    } else {
        static_assert(NW == 4, "keys are 1, 2 or 4 words");
        if (ws == 0) canonical_ws<4, 0>(d, g, k, can, is_rc);
        else if (ws == 1) canonical_ws<4, 1>(d, g, k, can, is_rc);
        else if (ws == 2) canonical_ws<4, 2>(d, g, k, can, is_rc);
        else canonical_ws<4, 3>(d, g, k, can, is_rc);
    }
}

// Counter index of row r for key in a 4 x 2^log2w Count-Min Sketch (sketch.rs:193-195).
__device__ __forceinline__ uint64_t cms_index(uint64_t key, int r, uint32_t log2w) {
    const uint64_t col = smix(key ^ cms_seed(r)) & ((1ULL << log2w) - 1);
    return ((uint64_t)r << log2w) + col;
}

// One increment of N (row, column) counters kept as threshold ladders (t levels of
// bits, level j set by the (j+1)-th increment; see fbk_k_ladder.cu).  climb[i] is
// false for a counter whose top level is already set.  The N atomics of a level are
// issued together and waited on once, so a warp pays one L2 round trip per level
// below the top, not one per (counter, level); the top level's old value is not
// needed (a reduction with no return).
template <int N>
__device__ __forceinline__ void ladder_climb(uint32_t* __restrict__ lad, uint64_t level_words, uint32_t t,
                                             const uint32_t (&wd)[N], const uint32_t (&mk)[N], bool (&climb)[N]) {
    for (uint32_t j = 0; j + 1 < t; ++j) {
        uint32_t* lv = lad + (uint64_t)j * level_words;
        uint32_t old[N];
#pragma unroll
        for (int i = 0; i < N; ++i) old[i] = climb[i] ? atomicOr(lv + wd[i], mk[i]) : 0u;
#pragma unroll
        for (int i = 0; i < N; ++i) climb[i] = (old[i] & mk[i]) != 0;
    }
    uint32_t* lv = lad + (uint64_t)(t - 1) * level_words;
#pragma unroll
    for (int i = 0; i < N; ++i)
        if (climb[i]) atomicOr(lv + wd[i], mk[i]);
}

// HyperLogLog register index and rank — sketch.rs:49-63 (p = 14 there).
__device__ __forceinline__ void hll_idx_rho(uint64_t h, uint32_t p, uint32_t& idx, uint32_t& rho) {
    idx = (uint32_t)(h >> (64 - p));
    const uint64_t w = h & ((1ULL << (64 - p)) - 1);
    rho = w == 0 ? (64 - p + 1) : ((uint32_t)__clzll(w) - p + 1);
}

// Canonical ntHash of the window of k bases at g (nthash_fwd/rev, kmer.rs:394-423).
// Equal to RollingNtHash's rolled value for the same window (kmer.rs:447-464).
__device__ __forceinline__ uint64_t nthash_canonical_at(const uint64_t* __restrict__ d, uint64_t g, uint32_t k) {
    uint64_t hf = 0, hr = 0;
    for (uint32_t j = 0; j < k; ++j) {
        const uint32_t c = base_at(d, g + j);
        hf ^= rotl64(nt_fwd(c), (k - 1 - j) & 63);
        hr ^= rotl64(nt_fwd(3 - c), j & 63);
    }
    return hf < hr ? hf : hr;
}

// Canonical ntHash of windows lo .. hi-1 of the read at base off, handed to f(i, h):
// the first computed as above, each next one rolled from it (kmer.rs:447-464) —
//   fwd(i+1) = rotl(fwd(i) ^ rotl(F[c_i], k-1), 1) ^ F[c_{i+k}]
//   rev(i+1) = rotr(rev(i) ^ R[c_i] ^ rotl(R[c_{i+k}], k), 1),   R[c] = F[3-c]
// exact identities of the XOR-of-rotations definition, so every value equals
// nthash_canonical_at's.
template <class Fn>
__device__ __forceinline__ void nthash_run(const uint64_t* __restrict__ d, uint64_t off, uint32_t k, uint32_t lo, uint32_t hi,
                                           Fn&& f) {
    if (lo >= hi) return;
    uint64_t hf = 0, hr = 0;
    for (uint32_t j = 0; j < k; ++j) {
        const uint32_t c = base_at(d, off + lo + j);
        hf ^= rotl64(nt_fwd(c), (k - 1 - j) & 63);
        hr ^= rotl64(nt_fwd(3 - c), j & 63);
    }
    f(lo, hf < hr ? hf : hr);
    for (uint32_t i = lo + 1; i < hi; ++i) {
        const uint32_t co = base_at(d, off + i - 1), ci = base_at(d, off + i - 1 + k);
        hf = rotl64(hf ^ rotl64(nt_fwd(co), k - 1), 1) ^ nt_fwd(ci);
        hr = rotr64(hr ^ nt_fwd(3 - co) ^ rotl64(nt_fwd(3 - ci), k), 1);
        f(i, hf < hr ? hf : hr);
    }
}

// Device status bits, read by the host after each phase.
enum : uint32_t {
    ST_TABLE_FULL = 1u,
    ST_SPIN_TIMEOUT = 2u,
    ST_BAD_INPUT = 4u,
};

}  // namespace fbk
