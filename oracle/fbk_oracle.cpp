// fbk_oracle.cpp — ORACLE: CPU restatement of fastBact's k-mer counting front end.
//
// TEST INFRASTRUCTURE ONLY.  Nothing in the product (the fastbact_gb300 package and
// its libfbk.so) links, loads or calls this file.  It is used by tests/ to check the
// device results, by __graft_entry__.smoke() to check its one small run, and by
// bench.py as the timed CPU baseline ("kind": "port") and as the reference arm.
//
// The reference (Caizhaohui/fastBact v0.1.0) is pure Rust.  No Rust toolchain and
// no vendored crates exist where this project is built, so the reference cannot be
// compiled or run; this file restates its algorithm function by function, each one
// citing the Rust file:line it follows (paths relative to the fastBact repository).
// Parity pin: the reference ships no golden hash/sketch vectors; this restatement is
// pinned against every known-answer test its own test modules hold for the path
// (bitseq.rs:433-506, kmer.rs:543-664, sketch.rs:262-407, estimator.rs:448-546,
// build.rs:604-687 structural inputs) plus the published SplitMix64 output vectors.
// The tests in tests/test_oracle_kat.py carry those checks.
//
// Build: oracle/build_oracle.sh (g++ -O2 -ffp-contract=off, no fast-math: the f64
// estimator math must round exactly like Rust's f64, which calls the same libm).

#include <algorithm>
#include <array>
#include <type_traits>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

namespace orc {

typedef unsigned __int128 u128;

// ---------------------------------------------------------------------------
// splitmix64 finaliser — src/common/sketch.rs:13-18
// ---------------------------------------------------------------------------
static inline uint64_t splitmix64(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
    return z ^ (z >> 31);
}

// ---------------------------------------------------------------------------
// 2-bit codec — src/common/bitseq.rs:67-87
// ---------------------------------------------------------------------------
struct Ascii2Bit {
    uint8_t t[256];
    Ascii2Bit() {
        for (int i = 0; i < 256; ++i) t[i] = 0;  // non-ACGT -> 0 (A), bitseq.rs:76
        t['A'] = t['a'] = 0;
        t['C'] = t['c'] = 1;
        t['G'] = t['g'] = 2;
        t['T'] = t['t'] = 3;
    }
};
static const Ascii2Bit A2B;
static const uint8_t COMPLEMENT_2BIT[4] = {3, 2, 1, 0};          // bitseq.rs:84
static const uint8_t TWO_BIT_TO_ASCII[4] = {'A', 'C', 'G', 'T'};  // bitseq.rs:87

// rev_comp_word — bitseq.rs:120-138
static inline uint64_t rev_comp_word(uint64_t word, unsigned num_bases) {
    if (num_bases == 0) return 0;
    uint64_t w = __builtin_bswap64(word);
    w = ((w & 0x0f0f0f0f0f0f0f0fULL) << 4) | ((w & 0xf0f0f0f0f0f0f0f0ULL) >> 4);
    w = ((w & 0x3333333333333333ULL) << 2) | ((w & 0xccccccccccccccccULL) >> 2);
    w = ~w;
    if (num_bases < 32) {
        unsigned shift = (32 - num_bases) * 2;
        uint64_t mask = (1ULL << (num_bases * 2)) - 1;
        return (w >> shift) & mask;
    }
    return w;
}

// BitSeqArena layout (bitseq.rs:145-222): base i of the arena stream lives at bits
// 2*(i%32) of data[i/32]; offsets[id] is the base index of sequence id.
struct Arena {
    const uint64_t* data;
    uint64_t n_words;
    const uint64_t* offsets;
    const uint32_t* lengths;
    uint64_t n_seqs;
};

// extract_ascii_into — bitseq.rs:286-299
static inline void extract_ascii_into(const Arena& a, uint64_t id, std::vector<uint8_t>& buf) {
    buf.clear();
    uint64_t len = a.lengths[id];
    uint64_t start = a.offsets[id];
    for (uint64_t i = 0; i < len; ++i) {
        uint64_t g = start + i;
        uint64_t code = (a.data[g >> 5] >> ((g & 31) << 1)) & 3;
        buf.push_back(TWO_BIT_TO_ASCII[code]);
    }
}

// ---------------------------------------------------------------------------
// KmerInt — src/common/kmer.rs:18-335
// ---------------------------------------------------------------------------
struct K64 {
    uint64_t v;
    static const unsigned MAX_K = 31;  // kmer.rs:66
    static K64 from_ascii(const uint8_t* s, unsigned k) {  // kmer.rs:73-81
        uint64_t val = 0;
        for (unsigned i = 0; i < k; ++i) val = (val << 2) | A2B.t[s[i]];
        return K64{val};
    }
    K64 rev_comp(unsigned k) const { return K64{rev_comp_word(v, k)}; }  // kmer.rs:99-101
    static void roll_next(K64& fwd, K64& rev, uint8_t base, unsigned k) {  // kmer.rs:104-112
        uint64_t b = base & 3;
        uint64_t comp_b = (uint64_t)COMPLEMENT_2BIT[b] << (2 * (k - 1));
        uint64_t mask = k >= 32 ? ~0ULL : ((1ULL << (2 * k)) - 1);
        fwd.v = ((fwd.v << 2) | b) & mask;
        rev.v = (rev.v >> 2) | comp_b;
    }
    uint64_t to_u64() const { return v; }  // kmer.rs:115-117
    bool operator<(const K64& o) const { return v < o.v; }
    bool operator==(const K64& o) const { return v == o.v; }
    void words(uint64_t* out) const { out[0] = v; }
    static const int NW = 1;
};

struct K128 {
    u128 v;
    static const unsigned MAX_K = 63;  // kmer.rs:125
    static K128 from_ascii(const uint8_t* s, unsigned k) {  // kmer.rs:132-140
        u128 val = 0;
        for (unsigned i = 0; i < k; ++i) val = (val << 2) | (u128)A2B.t[s[i]];
        return K128{val};
    }
    K128 rev_comp(unsigned k) const {  // kmer.rs:158-178
        if (k == 0) return K128{0};
        uint64_t hi = (uint64_t)(v >> 64), lo = (uint64_t)v;
        uint64_t rc_hi = rev_comp_word(hi, 32), rc_lo = rev_comp_word(lo, 32);
        u128 full = ((u128)rc_lo << 64) | (u128)rc_hi;
        if (k < 64) {
            unsigned shift = (64 - k) * 2;
            u128 mask = (((u128)1) << (2 * k)) - 1;
            return K128{(full >> shift) & mask};
        }
        return K128{full};
    }
    static void roll_next(K128& fwd, K128& rev, uint8_t base, unsigned k) {  // kmer.rs:181-189
        u128 b = base & 3;
        u128 comp_b = ((u128)COMPLEMENT_2BIT[(unsigned)b]) << (2 * (k - 1));
        u128 mask = k >= 64 ? ~(u128)0 : ((((u128)1) << (2 * k)) - 1);
        fwd.v = ((fwd.v << 2) | b) & mask;
        rev.v = (rev.v >> 2) | comp_b;
    }
    uint64_t to_u64() const { return (uint64_t)v ^ (uint64_t)(v >> 64); }  // kmer.rs:192-194
    bool operator<(const K128& o) const { return v < o.v; }
    bool operator==(const K128& o) const { return v == o.v; }
    // Words in big-endian order (most significant first), matching K256.
    void words(uint64_t* out) const { out[0] = (uint64_t)(v >> 64); out[1] = (uint64_t)v; }
    static const int NW = 2;
};

struct K256 {
    uint64_t w[4];  // big-endian: w[0] most significant (kmer.rs:199)
    static const unsigned MAX_K = 127;
    static void mask_to(uint64_t* words, unsigned k) {  // masking loop, kmer.rs:246-256 / 292-302
        unsigned total_bits = 2 * k;
        for (int j = 0; j < 4; ++j) {
            unsigned word_min_bit = (3 - j) * 64;
            if (total_bits <= word_min_bit) words[j] = 0;
            else if (total_bits < word_min_bit + 64) {
                unsigned bits_in_word = total_bits - word_min_bit;
                words[j] &= (1ULL << bits_in_word) - 1;
            }
        }
    }
    static K256 from_ascii(const uint8_t* s, unsigned k) {  // kmer.rs:210-222
        K256 r{{0, 0, 0, 0}};
        for (unsigned i = 0; i < k; ++i) {
            uint64_t code = A2B.t[s[i]];
            r.w[0] = (r.w[0] << 2) | (r.w[1] >> 62);
            r.w[1] = (r.w[1] << 2) | (r.w[2] >> 62);
            r.w[2] = (r.w[2] << 2) | (r.w[3] >> 62);
            r.w[3] = (r.w[3] << 2) | code;
        }
        return r;
    }
    K256 push_base(uint8_t base, unsigned k) const {  // kmer.rs:236-258
        uint64_t code = base & 3;
        K256 r{{(w[0] << 2) | (w[1] >> 62), (w[1] << 2) | (w[2] >> 62), (w[2] << 2) | (w[3] >> 62),
                (w[3] << 2) | code}};
        mask_to(r.w, k);
        return r;
    }
    K256 rev_comp(unsigned k) const {  // kmer.rs:260-305
        if (k == 0) return K256{{0, 0, 0, 0}};
        uint64_t full[4] = {rev_comp_word(w[3], 32), rev_comp_word(w[2], 32), rev_comp_word(w[1], 32),
                            rev_comp_word(w[0], 32)};
        if (k == 128) return K256{{full[0], full[1], full[2], full[3]}};
        unsigned s = (128 - k) * 2, w_shift = s / 64, b_shift = s % 64;
        K256 r{{0, 0, 0, 0}};
        for (unsigned i = 0; i < 4; ++i) {
            if (i + w_shift < 4) {
                r.w[i + w_shift] |= full[i] >> b_shift;
                if (b_shift > 0 && i + w_shift + 1 < 4) r.w[i + w_shift + 1] |= full[i] << (64 - b_shift);
            }
        }
        mask_to(r.w, k);
        return r;
    }
    static void roll_next(K256& fwd, K256& rev, uint8_t base, unsigned k) {  // kmer.rs:307-329
        K256 nf = fwd.push_base(base, k);
        uint64_t comp_b = COMPLEMENT_2BIT[base & 3];
        K256 nr{{rev.w[0] >> 2, (rev.w[1] >> 2) | (rev.w[0] << 62), (rev.w[2] >> 2) | (rev.w[1] << 62),
                 (rev.w[3] >> 2) | (rev.w[2] << 62)}};
        unsigned bit_pos = 2 * (k - 1);
        unsigned word_idx = 3 - bit_pos / 64;
        nr.w[word_idx] |= comp_b << (bit_pos % 64);
        fwd = nf;
        rev = nr;
    }
    uint64_t to_u64() const { return w[0] ^ w[1] ^ w[2] ^ w[3]; }  // kmer.rs:332-334
    bool operator<(const K256& o) const {  // derived Ord on [u64;4]: lexicographic
        for (int i = 0; i < 4; ++i)
            if (w[i] != o.w[i]) return w[i] < o.w[i];
        return false;
    }
    bool operator==(const K256& o) const {
        return w[0] == o.w[0] && w[1] == o.w[1] && w[2] == o.w[2] && w[3] == o.w[3];
    }
    void words(uint64_t* out) const { for (int i = 0; i < 4; ++i) out[i] = w[i]; }
    static const int NW = 4;
};

// ---------------------------------------------------------------------------
// ntHash — src/common/kmer.rs:385-477
// ---------------------------------------------------------------------------
static const uint64_t NT_HASH_FWD[4] = {0x3c8bfbb395c60474ULL, 0x3193c18562a02b4cULL,
                                        0x20323ee046061444ULL, 0x295c504fac61002eULL};
static const uint64_t NT_HASH_REV[4] = {0x295c504fac61002eULL, 0x20323ee046061444ULL,
                                        0x3193c18562a02b4cULL, 0x3c8bfbb395c60474ULL};
static inline uint64_t rotl(uint64_t x, unsigned r) { r &= 63; return r ? (x << r) | (x >> (64 - r)) : x; }
static inline uint64_t rotr(uint64_t x, unsigned r) { r &= 63; return r ? (x >> r) | (x << (64 - r)) : x; }

static uint64_t nthash_fwd(const uint8_t* s, unsigned k) {  // kmer.rs:394-404
    uint64_t h = 0;
    for (unsigned i = 0; i < k; ++i) h ^= rotl(NT_HASH_FWD[A2B.t[s[i]]], (k - 1 - i) % 64);
    return h;
}
static uint64_t nthash_rev(const uint8_t* s, unsigned k) {  // kmer.rs:407-416
    uint64_t h = 0;
    for (unsigned i = 0; i < k; ++i) h ^= rotl(NT_HASH_REV[A2B.t[s[i]]], i % 64);
    return h;
}
struct RollingNtHash {  // kmer.rs:427-477
    unsigned k;
    uint64_t h_fwd, h_rev;
    RollingNtHash(const uint8_t* s, unsigned kk) : k(kk), h_fwd(nthash_fwd(s, kk)), h_rev(nthash_rev(s, kk)) {}
    uint64_t roll(uint8_t out_base, uint8_t in_base) {  // kmer.rs:447-464
        unsigned oc = A2B.t[out_base], ic = A2B.t[in_base];
        unsigned k_mod = k % 64, km1_mod = (k - 1) % 64;
        h_fwd = rotl(h_fwd, 1) ^ rotl(NT_HASH_FWD[oc], k_mod) ^ NT_HASH_FWD[ic];
        h_rev = rotr(h_rev, 1) ^ rotr(NT_HASH_REV[oc], 1) ^ rotl(NT_HASH_REV[ic], km1_mod);
        return canonical();
    }
    uint64_t canonical() const { return h_fwd < h_rev ? h_fwd : h_rev; }  // kmer.rs:468-470
};

// ---------------------------------------------------------------------------
// Rust `f64 as u64` (saturating, NaN -> 0)
// ---------------------------------------------------------------------------
static inline uint64_t f64_to_u64_sat(double x) {
    if (!(x > 0.0)) return 0;  // NaN, negatives, -0
    if (x >= 18446744073709551616.0) return UINT64_MAX;
    return (uint64_t)x;
}
static inline uint64_t f64_to_usize_sat(double x) { return f64_to_u64_sat(x); }

// ---------------------------------------------------------------------------
// HyperLogLog — src/common/sketch.rs:24-115 (p = 14 in the reference; p is a
// parameter here so the p = 16 stress configuration has a restatement too)
// ---------------------------------------------------------------------------
struct HLL {
    unsigned p;
    std::vector<uint8_t> reg;
    explicit HLL(unsigned pp) : p(pp), reg((size_t)1 << pp, 0) {}
    void add_hash(uint64_t h) {  // sketch.rs:49-63
        size_t idx = (size_t)(h >> (64 - p));
        uint64_t w = h & ((1ULL << (64 - p)) - 1);
        uint8_t rho = w == 0 ? (uint8_t)(64 - p + 1) : (uint8_t)(__builtin_clzll(w) - p + 1);
        if (rho > reg[idx]) reg[idx] = rho;
    }
    void merge(const HLL& o) {  // sketch.rs:73-80
        for (size_t i = 0; i < reg.size(); ++i)
            if (o.reg[i] > reg[i]) reg[i] = o.reg[i];
    }
    double estimate() const { return estimate_regs(reg.data(), p); }
    static double estimate_regs(const uint8_t* r, unsigned p) {  // sketch.rs:83-114
        size_t n = (size_t)1 << p;
        double m = (double)n;
        double alpha_m = 0.7213 / (1.0 + 1.079 / m);
        double sum = 0.0;
        size_t zeros = 0;
        for (size_t i = 0; i < n; ++i) {
            sum += std::ldexp(1.0, -(int)r[i]);  // 2.0f64.powi(-val): exact power of two
            if (r[i] == 0) zeros++;
        }
        double raw = alpha_m * m * m / sum;
        if (raw <= 2.5 * m) {
            if (zeros > 0) return m * std::log(m / (double)zeros);
            return raw;
        } else if (raw <= (1.0 / 30.0) * 18446744073709551616.0) {
            return raw;
        }
        double two64 = 18446744073709551616.0;
        return -two64 * std::log(1.0 - raw / two64);
    }
};

// ---------------------------------------------------------------------------
// CountMinSketch — src/common/sketch.rs:121-253.  counter_bits == 4 is the
// reference layout (two nibbles per byte, saturating at 15, byte (r*w+col)>>1,
// high nibble for odd counter index).  counter_bits == 16 is the u16 variant
// (saturating at 65535); for every threshold t <= 15 it decides identically
// because min_r min(15, n_r) == min(15, min_r n_r).
// ---------------------------------------------------------------------------
static const uint64_t CMS_SEEDS[4] = {0x243f6a8885a308d3ULL, 0x13198a2e03707344ULL,
                                      0xa4093822299f31d0ULL, 0x082efa98ec4e6c89ULL};  // sketch.rs:122-127

static inline uint64_t next_pow2_u64(uint64_t x) {
    if (x <= 1) return 1;
    return 1ULL << (64 - __builtin_clzll(x - 1));
}

struct CMS {
    uint64_t width, mask;
    int bits;
    std::vector<std::atomic<uint8_t>> nib;     // counter_bits == 4
    std::vector<std::atomic<uint16_t>> c16;    // counter_bits == 16
    CMS(uint64_t w, int counter_bits) : bits(counter_bits) {  // sketch.rs:140-157
        if ((w & (w - 1)) != 0) w = next_pow2_u64(w);
        width = w;
        mask = w - 1;
        if (bits == 4) {
            std::vector<std::atomic<uint8_t>> t(4 * w / 2);
            for (auto& x : t) x.store(0, std::memory_order_relaxed);
            nib.swap(t);
        } else {
            std::vector<std::atomic<uint16_t>> t(4 * w);
            for (auto& x : t) x.store(0, std::memory_order_relaxed);
            c16.swap(t);
        }
    }
    static uint64_t width_for_genome_size(uint64_t g) {  // sketch.rs:165-168
        uint64_t target = next_pow2_u64(g * 16);
        if (target < (1ULL << 21)) target = 1ULL << 21;
        if (target > (1ULL << 27)) target = 1ULL << 27;
        return target;
    }
    void add(uint64_t key) {  // sketch.rs:191-223
        for (int r = 0; r < 4; ++r) {
            uint64_t col = splitmix64(key ^ CMS_SEEDS[r]) & mask;
            uint64_t ci = (uint64_t)r * width + col;
            if (bits == 4) {
                std::atomic<uint8_t>& a = nib[ci >> 1];
                bool hi = (ci & 1) == 1;
                uint8_t cur = a.load(std::memory_order_relaxed);
                for (;;) {
                    uint8_t cnt = hi ? (cur >> 4) & 0x0F : cur & 0x0F;
                    if (cnt >= 15) break;
                    uint8_t nc = cnt + 1;
                    uint8_t nv = hi ? (uint8_t)((cur & 0x0F) | (nc << 4)) : (uint8_t)((cur & 0xF0) | nc);
                    if (a.compare_exchange_weak(cur, nv, std::memory_order_relaxed)) break;
                }
            } else {
                std::atomic<uint16_t>& a = c16[ci];
                uint16_t cur = a.load(std::memory_order_relaxed);
                for (;;) {
                    if (cur == 0xFFFF) break;
                    if (a.compare_exchange_weak(cur, (uint16_t)(cur + 1), std::memory_order_relaxed)) break;
                }
            }
        }
    }
    uint32_t estimate(uint64_t key) const {  // sketch.rs:227-246
        uint32_t mn = bits == 4 ? 15u : 0xFFFFu;
        for (int r = 0; r < 4; ++r) {
            uint64_t col = splitmix64(key ^ CMS_SEEDS[r]) & mask;
            uint64_t ci = (uint64_t)r * width + col;
            uint32_t cnt;
            if (bits == 4) {
                uint8_t cur = nib[ci >> 1].load(std::memory_order_relaxed);
                cnt = (ci & 1) ? (cur >> 4) & 0x0F : cur & 0x0F;
            } else {
                cnt = c16[ci].load(std::memory_order_relaxed);
            }
            if (cnt < mn) mn = cnt;
            if (mn == 0) return 0;
        }
        return mn;
    }
    uint32_t add_and_estimate(uint64_t key) { add(key); return estimate(key); }  // sketch.rs:250-253
};

// ---------------------------------------------------------------------------
// Worker pool: dynamic chunking over an index range (stands in for rayon's
// work-stealing `into_par_iter`, src/graph/build.rs:94,246).
// ---------------------------------------------------------------------------
template <class F>
static void parallel_chunks(uint64_t n, uint64_t chunk, int threads, F f) {
    if (threads <= 1 || n <= chunk) {
        for (uint64_t s = 0; s < n; s += chunk) f(s, std::min(n, s + chunk));
        return;
    }
    std::atomic<uint64_t> next(0);
    std::vector<std::thread> ts;
    for (int t = 0; t < threads; ++t)
        ts.emplace_back([&]() {
            for (;;) {
                uint64_t s = next.fetch_add(chunk);
                if (s >= n) break;
                f(s, std::min(n, s + chunk));
            }
        });
    for (auto& t : ts) t.join();
}

static int resolve_threads(int t) {
    if (t > 0) return t;
    unsigned h = std::thread::hardware_concurrency();
    return h ? (int)h : 1;
}

// ---------------------------------------------------------------------------
// Shard map: open addressing, stands in for FxHashMap<K, KmerAcc> (hashbrown).
// Iteration order is irrelevant: results are compared as sets sorted by key.
// ---------------------------------------------------------------------------
struct KmerAcc {  // build.rs:145-149
    uint16_t cov;
    uint16_t edge_counts[8];
};

static inline uint16_t sat_add_u16(uint16_t a, uint32_t b) {
    uint32_t s = (uint32_t)a + b;
    return s > 0xFFFF ? 0xFFFF : (uint16_t)s;
}

template <class K>
struct ShardMap {
    std::vector<K> keys;
    std::vector<KmerAcc> vals;
    std::vector<uint8_t> used;
    uint64_t n = 0, cap = 0;
    static uint64_t h(const K& k) { return splitmix64(k.to_u64() * 0x9E3779B97F4A7C15ULL + 0x632BE59BD9B4E019ULL); }
    void grow() {
        uint64_t nc = cap ? cap * 2 : 1024;
        std::vector<K> ok;
        std::vector<KmerAcc> ov;
        std::vector<uint8_t> ou;
        ok.swap(keys); ov.swap(vals); ou.swap(used);
        keys.assign(nc, K{});
        vals.assign(nc, KmerAcc{});
        used.assign(nc, 0);
        cap = nc;
        n = 0;
        for (uint64_t i = 0; i < ou.size(); ++i)
            if (ou[i]) *slot(ok[i]) = ov[i];
    }
    KmerAcc* slot(const K& k) {  // entry(k).or_default()
        if ((n + 1) * 10 > cap * 7) grow();
        uint64_t m = cap - 1, p = h(k) & m;
        for (;;) {
            if (!used[p]) { used[p] = 1; keys[p] = k; vals[p] = KmerAcc{}; n++; return &vals[p]; }
            if (keys[p] == k) return &vals[p];
            p = (p + 1) & m;
        }
    }
};

// Solid table after conversion (build.rs:295-328) plus the raw accumulators.
template <class K>
struct SolidTable {
    std::vector<ShardMap<K>> shards;
    SolidTable() : shards(64) {}
};

static inline unsigned shard_idx(uint64_t key_u64) { return (unsigned)(splitmix64(key_u64) & 63); }  // build.rs:152-154

// Bank iteration order: merged, pe_forward, pe_reverse (build.rs:90).
struct Bank {
    Arena a[3];
};

// ---------------------------------------------------------------------------
// Pass 1 — build.rs:90-116 (+ prior contigs ×10, build.rs:118-138)
// ---------------------------------------------------------------------------
template <class K>
static void pass1(const Bank& bank, unsigned k, CMS& cms, int threads, const uint64_t* keep_mask_pairs,
                  const uint32_t* pair_idx_per_arena[3]) {
    for (int ai = 0; ai < 3; ++ai) {
        const Arena& arena = bank.a[ai];
        parallel_chunks(arena.n_seqs, 1024, threads, [&](uint64_t s, uint64_t e) {
            std::vector<uint8_t> buf;
            buf.reserve(300);
            for (uint64_t id = s; id < e; ++id) {
                if (keep_mask_pairs && pair_idx_per_arena[ai]) {
                    uint64_t pi = pair_idx_per_arena[ai][id];
                    if (!((keep_mask_pairs[pi >> 6] >> (pi & 63)) & 1)) continue;
                }
                if (arena.lengths[id] < k) continue;
                extract_ascii_into(arena, id, buf);
                const uint8_t* seq = buf.data();
                K fwd = K::from_ascii(seq, k);
                K rev = fwd.rev_comp(k);
                cms.add((rev < fwd ? rev : fwd).to_u64());
                for (size_t i = k; i < buf.size(); ++i) {
                    K::roll_next(fwd, rev, A2B.t[seq[i]], k);
                    cms.add((rev < fwd ? rev : fwd).to_u64());
                }
            }
        });
    }
}

template <class K>
static void pass1_contigs(const uint8_t* ascii, const uint64_t* offs, uint64_t n_contigs, unsigned k, CMS& cms) {
    for (uint64_t c = 0; c < n_contigs; ++c) {
        const uint8_t* s = ascii + offs[c];
        uint64_t len = offs[c + 1] - offs[c];
        if (len < k) continue;
        K fwd = K::from_ascii(s, k);
        K rev = fwd.rev_comp(k);
        K can = rev < fwd ? rev : fwd;
        for (int t = 0; t < 10; ++t) cms.add(can.to_u64());
        for (uint64_t i = k; i < len; ++i) {
            K::roll_next(fwd, rev, A2B.t[s[i]], k);
            can = rev < fwd ? rev : fwd;
            for (int t = 0; t < 10; ++t) cms.add(can.to_u64());
        }
    }
}

// ---------------------------------------------------------------------------
// Pass 2 — build.rs:141-289: CMS-gated transitions into 64 mutex shards with
// per-thread buffers flushed at 2048 entries.
// ---------------------------------------------------------------------------
template <class K>
static void pass2(const Bank& bank, unsigned k, const CMS& cms, unsigned t_solid, SolidTable<K>& tab, int threads,
                  const uint64_t* keep_mask_pairs, const uint32_t* pair_idx_per_arena[3],
                  const uint8_t* contig_ascii, const uint64_t* contig_offs, uint64_t n_contigs) {
    std::vector<std::mutex> mutexes(64);
    // Prior contigs: +100 cov, +1000 edge (build.rs:203-240)
    for (uint64_t c = 0; c < n_contigs; ++c) {
        const uint8_t* s = contig_ascii + contig_offs[c];
        uint64_t len = contig_offs[c + 1] - contig_offs[c];
        if (len < k + 1) continue;
        K u_fwd = K::from_ascii(s, k), u_rev = u_fwd.rev_comp(k);
        bool u_rc = u_rev < u_fwd;
        K u_can = u_rc ? u_rev : u_fwd;
        for (uint64_t i = 0; i + k + 1 <= len; ++i) {
            uint8_t base = A2B.t[s[i + k]];
            K v_fwd = u_fwd, v_rev = u_rev;
            K::roll_next(v_fwd, v_rev, base, k);
            bool v_rc = v_rev < v_fwd;
            K v_can = v_rc ? v_rev : v_fwd;
            uint8_t edge_u = !u_rc ? base : base + 4;
            KmerAcc* e = tab.shards[shard_idx(u_can.to_u64())].slot(u_can);
            e->cov = sat_add_u16(e->cov, 100);
            e->edge_counts[edge_u] = sat_add_u16(e->edge_counts[edge_u], 1000);
            uint8_t p = A2B.t[s[i]], rc_p = 3 - p;
            uint8_t edge_v = !v_rc ? rc_p + 4 : rc_p;
            e = tab.shards[shard_idx(v_can.to_u64())].slot(v_can);
            e->cov = sat_add_u16(e->cov, 100);
            e->edge_counts[edge_v] = sat_add_u16(e->edge_counts[edge_v], 1000);
            u_fwd = v_fwd; u_rev = v_rev; u_can = v_can; u_rc = v_rc;
        }
    }
    for (int ai = 0; ai < 3; ++ai) {
        const Arena& arena = bank.a[ai];
        parallel_chunks(arena.n_seqs, 4096, threads, [&](uint64_t s, uint64_t e) {
            std::vector<uint8_t> buf;
            buf.reserve(300);
            std::vector<std::vector<std::pair<K, uint8_t>>> tbuf(64);
            auto flush = [&](unsigned si) {
                if (tbuf[si].empty()) return;
                std::lock_guard<std::mutex> g(mutexes[si]);
                for (auto& pe : tbuf[si]) {
                    KmerAcc* a = tab.shards[si].slot(pe.first);
                    a->cov = sat_add_u16(a->cov, 1);
                    a->edge_counts[pe.second] = sat_add_u16(a->edge_counts[pe.second], 1);
                }
                tbuf[si].clear();
            };
            auto push = [&](unsigned si, const K& km, uint8_t edge) {
                tbuf[si].push_back(std::make_pair(km, edge));
                if (tbuf[si].size() >= 2048) flush(si);
            };
            for (uint64_t id = s; id < e; ++id) {
                if (keep_mask_pairs && pair_idx_per_arena[ai]) {
                    uint64_t pi = pair_idx_per_arena[ai][id];
                    if (!((keep_mask_pairs[pi >> 6] >> (pi & 63)) & 1)) continue;
                }
                if (arena.lengths[id] < k + 1) continue;
                extract_ascii_into(arena, id, buf);
                const uint8_t* seq = buf.data();
                uint64_t L = buf.size();
                K u_fwd = K::from_ascii(seq, k), u_rev = u_fwd.rev_comp(k);
                bool u_rc = u_rev < u_fwd;
                K u_can = u_rc ? u_rev : u_fwd;
                uint32_t u_cnt = cms.estimate(u_can.to_u64());
                for (uint64_t i = 0; i + k + 1 <= L; ++i) {
                    uint8_t base = A2B.t[seq[i + k]];
                    K v_fwd = u_fwd, v_rev = u_rev;
                    K::roll_next(v_fwd, v_rev, base, k);
                    bool v_rc = v_rev < v_fwd;
                    K v_can = v_rc ? v_rev : v_fwd;
                    uint32_t v_cnt = cms.estimate(v_can.to_u64());
                    if (u_cnt >= t_solid && v_cnt >= t_solid) {
                        uint8_t edge_u = !u_rc ? base : base + 4;
                        push(shard_idx(u_can.to_u64()), u_can, edge_u);
                        uint8_t p = A2B.t[seq[i]], rc_p = 3 - p;
                        uint8_t edge_v = !v_rc ? rc_p + 4 : rc_p;
                        push(shard_idx(v_can.to_u64()), v_can, edge_v);
                    }
                    u_fwd = v_fwd; u_rev = v_rev; u_can = v_can; u_rc = v_rc; u_cnt = v_cnt;
                }
            }
            for (unsigned si = 0; si < 64; ++si) flush(si);
        });
    }
}

// Export of the accumulator map (all keys) and of the SolidKmerNode conversion
// (build.rs:302-328): mask bit e iff edge_counts[e] >= min_trans_cov, keep iff mask != 0,
// cov = max(1, acc.cov / 2).  Rows are sorted by key (big-endian word order).
template <class K>
struct Row {
    K key;
    KmerAcc acc;
};

template <class K>
static std::vector<Row<K>> collect_sorted(const SolidTable<K>& tab) {
    std::vector<Row<K>> rows;
    for (auto& sh : tab.shards)
        for (uint64_t i = 0; i < sh.cap; ++i)
            if (sh.used[i]) rows.push_back(Row<K>{sh.keys[i], sh.vals[i]});
    std::sort(rows.begin(), rows.end(), [](const Row<K>& a, const Row<K>& b) { return a.key < b.key; });
    return rows;
}

// ---------------------------------------------------------------------------
// Estimator — src/ingest/estimator.rs:104-440
// ---------------------------------------------------------------------------
static void compute_dynamic_kmers(uint64_t median_len, int64_t target_max_k, std::vector<uint64_t>& out) {
    // estimator.rs:104-161
    out.clear();
    uint64_t min_k = median_len < 75 ? 21 : 31;
    uint64_t effective_len = (median_len * 16) / 10;
    uint64_t auto_max = f64_to_usize_sat((double)effective_len * 0.85);
    uint64_t max_k = target_max_k >= 0 ? (uint64_t)target_max_k : auto_max;
    if (max_k < min_k) max_k = min_k;  // clamp(min_k, 127)
    if (max_k > 127) max_k = 127;
    if (max_k % 2 == 0) max_k -= 1;
    if (max_k <= min_k) { out.push_back(min_k); return; }
    if (median_len >= 100) {
        uint64_t mid_k = 63;
        if (max_k > mid_k + 10) { out.push_back(min_k); out.push_back(mid_k); out.push_back(max_k); }
        else if (max_k > min_k) { out.push_back(min_k); out.push_back(max_k); }
        else out.push_back(min_k);
        return;
    }
    uint64_t steps = 2;
    uint64_t step = (max_k - min_k) / steps;
    if (step % 2 == 1) step += 1;
    if (step < 6) step = 6;
    for (uint64_t kk = min_k; kk <= max_k; kk += step) out.push_back(kk);
    uint64_t last = out.back();
    if (last != max_k && max_k > last) {
        if (max_k - last >= 10) out.push_back(max_k);
        else out.back() = max_k;
    }
    out.erase(std::unique(out.begin(), out.end()), out.end());
}


// ---------------------------------------------------------------------------
// Plain 4-line FASTQ reading (stands in for needletail 0.5.1, called through
// open_fastx, trim_merge.rs:241-258).  Line endings (\n or \r\n) are stripped;
// the record id is the header line without '@'.  Gzip input is not restated.
// ---------------------------------------------------------------------------
struct FastqReader {
    FILE* f = nullptr;
    std::string hdr, seq, plus, qual;
    explicit FastqReader(const char* path) { f = fopen(path, "rb"); }
    ~FastqReader() { if (f) fclose(f); }
    bool getline(std::string& s) {
        s.clear();
        int c;
        bool any = false;
        while ((c = fgetc(f)) != EOF) {
            any = true;
            if (c == '\n') break;
            s.push_back((char)c);
        }
        if (!s.empty() && s.back() == '\r') s.pop_back();
        return any;
    }
    // 1 = record, 0 = end of input, -1 = malformed record
    int next(std::string& err) {
        for (;;) {
            if (!getline(hdr)) return 0;
            if (!hdr.empty()) break;  // tolerate blank lines between records
        }
        if (hdr[0] != '@') { err = "expected '@' at the start of a FASTQ record"; return -1; }
        if (!getline(seq)) { err = "truncated FASTQ record (missing sequence line)"; return -1; }
        if (!getline(plus) || plus.empty() || plus[0] != '+') { err = "truncated FASTQ record (missing '+' line)"; return -1; }
        if (!getline(qual)) { err = "truncated FASTQ record (missing quality line)"; return -1; }
        if (qual.size() != seq.size()) { err = "sequence and quality lengths differ"; return -1; }
        hdr.erase(0, 1);
        return 1;
    }
};

// extract_read_id_prefix — estimator.rs:89-99
static std::string read_id_prefix(const std::string& id) {
    size_t ws = id.size();
    for (size_t i = 0; i < id.size(); ++i)
        if (id[i] == ' ' || id[i] == '\t' || id[i] == '\n' || id[i] == '\r' || id[i] == '\f') { ws = i; break; }
    std::string s = id.substr(0, ws);
    if (s.size() >= 2 && s[s.size() - 2] == '/' && (s.back() == '1' || s.back() == '2')) s.resize(s.size() - 2);
    return s;
}

}  // namespace orc

// ===========================================================================
// extern "C" surface for ctypes (tests, smoke(), CPU baseline timing)
// ===========================================================================
using namespace orc;

#define ORC_API extern "C" __attribute__((visibility("default")))

typedef struct {
    const uint64_t* data;
    uint64_t n_words;
    const uint64_t* offsets;
    const uint32_t* lengths;
    uint64_t n_seqs;
} orc_arena;

typedef struct {
    uint64_t exact_read_pairs;
    uint64_t total_bases_r1;
    uint64_t total_bases_r2;
    uint64_t total_bases;
    uint64_t min_read_len;
    uint64_t max_read_len;
    double mean_read_len;
    uint64_t median_read_len;
} orc_count_stats;

typedef struct {
    uint64_t genome_size;
    uint64_t exact_read_pairs;
    uint64_t total_bases;
    uint64_t median_read_len;
    uint64_t max_read_len;
    double estimated_cov;
    double subsample_factor;
    uint64_t kmers[8];
    uint64_t n_kmers;
    int32_t confidence;  // 0 High, 1 LowCoverageWarning, 2 Unreliable
    int32_t _pad;
    uint64_t u_ge_1;
    uint64_t u_ge_2;
    double sample_kmer_depth;
    uint64_t pairs_sampled;  // diagnostic: pairs consumed before the loop ended
    uint64_t m_sample;       // diagnostic
} orc_genome_estimate;

ORC_API uint64_t orc_splitmix64(uint64_t z) { return splitmix64(z); }
ORC_API uint64_t orc_rev_comp_word(uint64_t w, unsigned n) { return rev_comp_word(w, n); }
ORC_API uint64_t orc_cms_width_for_genome_size(uint64_t g) { return CMS::width_for_genome_size(g); }

// K-mer integer helpers; words are big-endian (most significant first), nw = 1, 2, 4.

ORC_API int orc_kmer_from_ascii(int key_bits, const uint8_t* s, unsigned k, uint64_t* out) {
    if (key_bits == 64) K64::from_ascii(s, k).words(out);
    else if (key_bits == 128) K128::from_ascii(s, k).words(out);
    else if (key_bits == 256) K256::from_ascii(s, k).words(out);
    else return -1;
    return 0;
}

template <class K>
static K from_words(const uint64_t* w);
template <>
K64 from_words<K64>(const uint64_t* w) { return K64{w[0]}; }
template <>
K128 from_words<K128>(const uint64_t* w) { return K128{((u128)w[0] << 64) | (u128)w[1]}; }
template <>
K256 from_words<K256>(const uint64_t* w) { return K256{{w[0], w[1], w[2], w[3]}}; }

ORC_API int orc_kmer_rev_comp(int key_bits, const uint64_t* in, unsigned k, uint64_t* out) {
    if (key_bits == 64) from_words<K64>(in).rev_comp(k).words(out);
    else if (key_bits == 128) from_words<K128>(in).rev_comp(k).words(out);
    else if (key_bits == 256) from_words<K256>(in).rev_comp(k).words(out);
    else return -1;
    return 0;
}

ORC_API uint64_t orc_kmer_to_u64(int key_bits, const uint64_t* in) {
    if (key_bits == 64) return from_words<K64>(in).to_u64();
    if (key_bits == 128) return from_words<K128>(in).to_u64();
    return from_words<K256>(in).to_u64();
}

// Rolling canonical k-mers along an ASCII sequence (RollingKmer, kmer.rs:344-378).
// out receives (len-k+1) canonical keys of nw words each, plus an is_rc flag per window.
template <class K>
static void rolling_canon(const uint8_t* s, uint64_t len, unsigned k, uint64_t* out, uint8_t* is_rc) {
    K fwd = K::from_ascii(s, k), rev = fwd.rev_comp(k);
    uint64_t n = len - k + 1;
    for (uint64_t i = 0; i < n; ++i) {
        if (i > 0) K::roll_next(fwd, rev, A2B.t[s[i + k - 1]], k);
        bool rc = rev < fwd;
        (rc ? rev : fwd).words(out + i * K::NW);
        if (is_rc) is_rc[i] = rc;
    }
}

ORC_API int orc_rolling_canonicals(int key_bits, const uint8_t* s, uint64_t len, unsigned k, uint64_t* out, uint8_t* is_rc) {
    if (len < k || k == 0) return 0;
    if (key_bits == 64) rolling_canon<K64>(s, len, k, out, is_rc);
    else if (key_bits == 128) rolling_canon<K128>(s, len, k, out, is_rc);
    else if (key_bits == 256) rolling_canon<K256>(s, len, k, out, is_rc);
    else return -1;
    return (int)(len - k + 1);
}

ORC_API uint64_t orc_nthash_fwd(const uint8_t* s, unsigned k) { return nthash_fwd(s, k); }
ORC_API uint64_t orc_nthash_rev(const uint8_t* s, unsigned k) { return nthash_rev(s, k); }
ORC_API uint64_t orc_nthash_canonical(const uint8_t* s, unsigned k) {  // kmer.rs:419-423
    uint64_t f = nthash_fwd(s, k), r = nthash_rev(s, k);
    return f < r ? f : r;
}
// Canonical ntHash of every window, produced by RollingNtHash::new + roll.
ORC_API int orc_nthash_rolling_all(const uint8_t* s, uint64_t len, unsigned k, uint64_t* out) {
    if (len < k || k == 0) return 0;
    RollingNtHash h(s, k);
    out[0] = h.canonical();
    for (uint64_t i = k; i < len; ++i) out[i - k + 1] = h.roll(s[i - k], s[i]);
    return (int)(len - k + 1);
}

// HyperLogLog handles
ORC_API void* orc_hll_new(unsigned p) { return new HLL(p); }
ORC_API void orc_hll_free(void* h) { delete (HLL*)h; }
ORC_API void orc_hll_add_hash(void* h, uint64_t x) { ((HLL*)h)->add_hash(x); }
ORC_API void orc_hll_add_hashes(void* h, const uint64_t* xs, uint64_t n) { for (uint64_t i = 0; i < n; ++i) ((HLL*)h)->add_hash(xs[i]); }
ORC_API void orc_hll_add_canonical_hashes(void* h, const uint64_t* xs, uint64_t n) {  // sketch.rs:68-70
    for (uint64_t i = 0; i < n; ++i) ((HLL*)h)->add_hash(splitmix64(xs[i]));
}
ORC_API void orc_hll_merge(void* h, const void* o) { ((HLL*)h)->merge(*(const HLL*)o); }
ORC_API double orc_hll_estimate(const void* h) { return ((const HLL*)h)->estimate(); }
ORC_API double orc_hll_estimate_regs(const uint8_t* regs, unsigned p) { return HLL::estimate_regs(regs, p); }
ORC_API void orc_hll_registers(const void* h, uint8_t* out) {
    const HLL* x = (const HLL*)h;
    memcpy(out, x->reg.data(), x->reg.size());
}

// CountMinSketch handles
ORC_API void* orc_cms_new(uint64_t width, int counter_bits) {
    if (counter_bits != 4 && counter_bits != 16) return nullptr;
    return new CMS(width, counter_bits);
}
ORC_API void orc_cms_free(void* c) { delete (CMS*)c; }
ORC_API uint64_t orc_cms_width(const void* c) { return ((const CMS*)c)->width; }
ORC_API void orc_cms_add(void* c, uint64_t key) { ((CMS*)c)->add(key); }
ORC_API void orc_cms_add_many(void* c, const uint64_t* keys, uint64_t n) { for (uint64_t i = 0; i < n; ++i) ((CMS*)c)->add(keys[i]); }
ORC_API uint32_t orc_cms_estimate(const void* c, uint64_t key) { return ((const CMS*)c)->estimate(key); }
ORC_API uint32_t orc_cms_add_and_estimate(void* c, uint64_t key) { return ((CMS*)c)->add_and_estimate(key); }
// Raw table bytes: nibble layout (4*w/2 bytes) or u16 counters (4*w*2 bytes, little endian).
ORC_API uint64_t orc_cms_nbytes(const void* c) {
    const CMS* x = (const CMS*)c;
    return x->bits == 4 ? 4 * x->width / 2 : 4 * x->width * 2;
}
// Loads raw table bytes in the export layout (test plumbing for merged sketches of
// sharded counts; the reference has no counterpart).
ORC_API void orc_cms_import(void* c, const uint8_t* in) {
    CMS* x = (CMS*)c;
    if (x->bits == 4) {
        for (size_t i = 0; i < x->nib.size(); ++i) x->nib[i].store(in[i], std::memory_order_relaxed);
    } else {
        for (size_t i = 0; i < x->c16.size(); ++i)
            x->c16[i].store((uint16_t)(in[2 * i] | (in[2 * i + 1] << 8)), std::memory_order_relaxed);
    }
}
ORC_API void orc_cms_export(const void* c, uint8_t* out) {
    const CMS* x = (const CMS*)c;
    if (x->bits == 4) {
        for (size_t i = 0; i < x->nib.size(); ++i) out[i] = x->nib[i].load(std::memory_order_relaxed);
    } else {
        for (size_t i = 0; i < x->c16.size(); ++i) {
            uint16_t v = x->c16[i].load(std::memory_order_relaxed);
            out[2 * i] = (uint8_t)(v & 0xFF);
            out[2 * i + 1] = (uint8_t)(v >> 8);
        }
    }
}

// Bank-level build passes.  arenas[3] = merged, pe_forward, pe_reverse.
// keep_mask (optional): bit i set = input pair i kept (subsampler); pair_idx[a][id] maps a
// read to its input pair index (0-based bit position).  Pass NULL for no subsampling.
ORC_API int orc_build_pass1(const orc_arena* arenas, unsigned k, int key_bits, void* cms, int threads,
                    const uint64_t* keep_mask, const uint32_t* const* pair_idx) {
    Bank b;
    for (int i = 0; i < 3; ++i) b.a[i] = Arena{arenas[i].data, arenas[i].n_words, arenas[i].offsets, arenas[i].lengths, arenas[i].n_seqs};
    const uint32_t* pidx[3] = {pair_idx ? pair_idx[0] : nullptr, pair_idx ? pair_idx[1] : nullptr, pair_idx ? pair_idx[2] : nullptr};
    int th = resolve_threads(threads);
    CMS& c = *(CMS*)cms;
    if (key_bits == 64) pass1<K64>(b, k, c, th, keep_mask, pidx);
    else if (key_bits == 128) pass1<K128>(b, k, c, th, keep_mask, pidx);
    else if (key_bits == 256) pass1<K256>(b, k, c, th, keep_mask, pidx);
    else return -1;
    return 0;
}

ORC_API int orc_build_pass1_contigs(const uint8_t* ascii, const uint64_t* offs, uint64_t n, unsigned k, int key_bits, void* cms) {
    CMS& c = *(CMS*)cms;
    if (key_bits == 64) pass1_contigs<K64>(ascii, offs, n, k, c);
    else if (key_bits == 128) pass1_contigs<K128>(ascii, offs, n, k, c);
    else if (key_bits == 256) pass1_contigs<K256>(ascii, offs, n, k, c);
    else return -1;
    return 0;
}

struct OrcTable {
    int key_bits;
    void* t;
};

ORC_API void* orc_build_pass2(const orc_arena* arenas, unsigned k, int key_bits, const void* cms, unsigned t_solid, int threads,
                      const uint64_t* keep_mask, const uint32_t* const* pair_idx, const uint8_t* contig_ascii,
                      const uint64_t* contig_offs, uint64_t n_contigs) {
    Bank b;
    for (int i = 0; i < 3; ++i) b.a[i] = Arena{arenas[i].data, arenas[i].n_words, arenas[i].offsets, arenas[i].lengths, arenas[i].n_seqs};
    const uint32_t* pidx[3] = {pair_idx ? pair_idx[0] : nullptr, pair_idx ? pair_idx[1] : nullptr, pair_idx ? pair_idx[2] : nullptr};
    int th = resolve_threads(threads);
    const CMS& c = *(const CMS*)cms;
    OrcTable* ot = new OrcTable{key_bits, nullptr};
    if (key_bits == 64) { auto* t = new SolidTable<K64>(); pass2<K64>(b, k, c, t_solid, *t, th, keep_mask, pidx, contig_ascii, contig_offs, n_contigs); ot->t = t; }
    else if (key_bits == 128) { auto* t = new SolidTable<K128>(); pass2<K128>(b, k, c, t_solid, *t, th, keep_mask, pidx, contig_ascii, contig_offs, n_contigs); ot->t = t; }
    else if (key_bits == 256) { auto* t = new SolidTable<K256>(); pass2<K256>(b, k, c, t_solid, *t, th, keep_mask, pidx, contig_ascii, contig_offs, n_contigs); ot->t = t; }
    else { delete ot; return nullptr; }
    return ot;
}

ORC_API void orc_table_free(void* h) {
    OrcTable* ot = (OrcTable*)h;
    if (!ot) return;
    if (ot->key_bits == 64) delete (SolidTable<K64>*)ot->t;
    else if (ot->key_bits == 128) delete (SolidTable<K128>*)ot->t;
    else delete (SolidTable<K256>*)ot->t;
    delete ot;
}

template <class K>
static uint64_t table_size(void* t) {
    uint64_t n = 0;
    for (auto& s : ((SolidTable<K>*)t)->shards) n += s.n;
    return n;
}
ORC_API uint64_t orc_table_n_keys(void* h) {
    OrcTable* ot = (OrcTable*)h;
    if (ot->key_bits == 64) return table_size<K64>(ot->t);
    if (ot->key_bits == 128) return table_size<K128>(ot->t);
    return table_size<K256>(ot->t);
}

// Export every accumulated key (sorted): keys (nw words each), cov (u16), edges (8 x u16).
template <class K>
static uint64_t export_acc(void* t, uint64_t* keys, uint16_t* cov, uint16_t* edges, uint64_t cap) {
    auto rows = collect_sorted<K>(*(SolidTable<K>*)t);
    uint64_t n = std::min<uint64_t>(cap, rows.size());
    for (uint64_t i = 0; i < n; ++i) {
        rows[i].key.words(keys + i * K::NW);
        cov[i] = rows[i].acc.cov;
        for (int e = 0; e < 8; ++e) edges[i * 8 + e] = rows[i].acc.edge_counts[e];
    }
    return rows.size();
}
ORC_API uint64_t orc_table_export_acc(void* h, uint64_t* keys, uint16_t* cov, uint16_t* edges, uint64_t cap) {
    OrcTable* ot = (OrcTable*)h;
    if (ot->key_bits == 64) return export_acc<K64>(ot->t, keys, cov, edges, cap);
    if (ot->key_bits == 128) return export_acc<K128>(ot->t, keys, cov, edges, cap);
    return export_acc<K256>(ot->t, keys, cov, edges, cap);
}

// SolidKmerNode conversion (build.rs:302-328), sorted by key.
template <class K>
static uint64_t export_solid(void* t, unsigned min_trans_cov, uint64_t* keys, uint16_t* cov, uint8_t* mask, uint64_t cap) {
    auto rows = collect_sorted<K>(*(SolidTable<K>*)t);
    uint64_t n = 0;
    for (auto& r : rows) {
        uint8_t m = 0;
        for (int e = 0; e < 8; ++e)
            if (r.acc.edge_counts[e] >= min_trans_cov) m |= (uint8_t)(1u << e);
        if (m == 0) continue;
        if (n < cap) {
            r.key.words(keys + n * K::NW);
            uint16_t c = (uint16_t)(r.acc.cov / 2);
            cov[n] = c < 1 ? 1 : c;
            mask[n] = m;
        }
        n++;
    }
    return n;
}
ORC_API uint64_t orc_table_export_solid(void* h, unsigned min_trans_cov, uint64_t* keys, uint16_t* cov, uint8_t* mask, uint64_t cap) {
    OrcTable* ot = (OrcTable*)h;
    if (ot->key_bits == 64) return export_solid<K64>(ot->t, min_trans_cov, keys, cov, mask, cap);
    if (ot->key_bits == 128) return export_solid<K128>(ot->t, min_trans_cov, keys, cov, mask, cap);
    return export_solid<K256>(ot->t, min_trans_cov, keys, cov, mask, cap);
}

// Order-independent digest of the converted solid table: sum over entries of
// splitmix64(fold(key) ^ splitmix64(cov << 8 | mask)).  Used for full-size checks.
template <class K>
static uint64_t solid_digest(void* t, unsigned min_trans_cov, uint64_t* n_out) {
    uint64_t d = 0, n = 0;
    for (auto& sh : ((SolidTable<K>*)t)->shards)
        for (uint64_t i = 0; i < sh.cap; ++i) {
            if (!sh.used[i]) continue;
            const KmerAcc& a = sh.vals[i];
            uint8_t m = 0;
            for (int e = 0; e < 8; ++e)
                if (a.edge_counts[e] >= min_trans_cov) m |= (uint8_t)(1u << e);
            if (!m) continue;
            uint16_t c = (uint16_t)(a.cov / 2);
            if (c < 1) c = 1;
            uint64_t w[4] = {0, 0, 0, 0};
            sh.keys[i].words(w);
            uint64_t kd = 0;
            for (int j = 0; j < K::NW; ++j) kd = splitmix64(kd ^ w[j]);
            d += splitmix64(kd ^ splitmix64(((uint64_t)c << 8) | m));
            n++;
        }
    *n_out = n;
    return d;
}
ORC_API uint64_t orc_table_solid_digest(void* h, unsigned min_trans_cov, uint64_t* n_out) {
    OrcTable* ot = (OrcTable*)h;
    if (ot->key_bits == 64) return solid_digest<K64>(ot->t, min_trans_cov, n_out);
    if (ot->key_bits == 128) return solid_digest<K128>(ot->t, min_trans_cov, n_out);
    return solid_digest<K256>(ot->t, min_trans_cov, n_out);
}

// Order-independent digest of the whole accumulator (every key of the 64 shard maps with
// its KmerAcc, build.rs:145-196): sum over keys of
// splitmix64(kd ^ splitmix64(v0 ^ splitmix64(v1 ^ splitmix64(e7)))), kd = the key's
// big-endian words folded through splitmix64, v0 = cov | e0<<16 | e1<<32 | e2<<48,
// v1 = e3 | e4<<16 | e5<<32 | e6<<48.  Compares accumulators of tens of millions of
// keys at full size without exporting them.
template <class K>
static uint64_t acc_digest(void* t, uint64_t* n_out) {
    uint64_t d = 0, n = 0;
    for (auto& sh : ((SolidTable<K>*)t)->shards)
        for (uint64_t i = 0; i < sh.cap; ++i) {
            if (!sh.used[i]) continue;
            const KmerAcc& a = sh.vals[i];
            uint64_t w[4] = {0, 0, 0, 0};
            sh.keys[i].words(w);
            uint64_t kd = 0;
            for (int j = 0; j < K::NW; ++j) kd = splitmix64(kd ^ w[j]);
            const uint64_t v0 = (uint64_t)a.cov | ((uint64_t)a.edge_counts[0] << 16) | ((uint64_t)a.edge_counts[1] << 32) |
                                ((uint64_t)a.edge_counts[2] << 48);
            const uint64_t v1 = (uint64_t)a.edge_counts[3] | ((uint64_t)a.edge_counts[4] << 16) |
                                ((uint64_t)a.edge_counts[5] << 32) | ((uint64_t)a.edge_counts[6] << 48);
            d += splitmix64(kd ^ splitmix64(v0 ^ splitmix64(v1 ^ splitmix64((uint64_t)a.edge_counts[7]))));
            n++;
        }
    *n_out = n;
    return d;
}
ORC_API uint64_t orc_table_acc_digest(void* h, uint64_t* n_out) {
    OrcTable* ot = (OrcTable*)h;
    if (ot->key_bits == 64) return acc_digest<K64>(ot->t, n_out);
    if (ot->key_bits == 128) return acc_digest<K128>(ot->t, n_out);
    return acc_digest<K256>(ot->t, n_out);
}

// compute_dynamic_kmers — estimator.rs:104-161; target_max_k < 0 means None.
ORC_API int orc_compute_dynamic_kmers(uint64_t median_len, int64_t target_max_k, uint64_t* out, int cap) {
    std::vector<uint64_t> v;
    compute_dynamic_kmers(median_len, target_max_k, v);
    int n = (int)v.size();
    for (int i = 0; i < n && i < cap; ++i) out[i] = v[i];
    return n;
}

// Subsampler keep test — trim_merge.rs:324-348 (pair_idx is 1-based over all input pairs).
ORC_API int orc_subsample_keep(uint64_t pair_idx_1based, double factor, uint64_t seed) {
    if (!(factor < 0.999)) return 1;
    uint64_t keep_threshold = f64_to_u64_sat(factor * 18446744073709551616.0);
    return splitmix64(pair_idx_1based ^ seed) <= keep_threshold ? 1 : 0;
}

// Estimator sample loop + post-math (estimator.rs:296-439) over in-memory reads.
// reads: ASCII of R1,R2 interleaved per pair (read 2p = R1 of pair p, 2p+1 = R2),
// concatenated; read_offs has 2*n_pairs+1 entries.  stats is count_fastx_exact's result
// for the whole input (exact_read_pairs may exceed n_pairs: only the first
// min(max_pairs, 150000, exact_read_pairs) pairs are read).
// hll_p is 14 in the reference; regs_total/regs_solid (optional, 1<<hll_p bytes each)
// receive the final registers.
ORC_API int orc_estimate_from_reads(const uint8_t* reads, const uint64_t* read_offs, uint64_t n_pairs,
                            const orc_count_stats* stats, uint64_t max_pairs, double target_cov, unsigned k,
                            uint64_t cms_width, unsigned hll_p, orc_genome_estimate* out, uint8_t* regs_total,
                            uint8_t* regs_solid) {
    HLL hll_total(hll_p), hll_solid(hll_p);
    CMS cms(cms_width, 4);
    uint64_t sample_target = std::min<uint64_t>(std::min<uint64_t>(max_pairs, 150000), stats->exact_read_pairs);
    uint64_t m_sample = 0, pair_count = 0;
    while (pair_count < sample_target) {
        if (pair_count >= n_pairs) break;  // a reader ran dry: `_ => break` (estimator.rs:377)
        uint64_t p = pair_count;
        pair_count++;
        for (int mate = 0; mate < 2; ++mate) {
            const uint8_t* s = reads + read_offs[2 * p + mate];
            uint64_t len = read_offs[2 * p + mate + 1] - read_offs[2 * p + mate];
            if (len < k) continue;
            m_sample += len - k + 1;
            RollingNtHash rh(s, k);
            uint64_t raw = rh.canonical();
            uint32_t c = cms.add_and_estimate(raw);
            uint64_t mixed = splitmix64(raw);
            hll_total.add_hash(mixed);
            if (c >= 2) hll_solid.add_hash(mixed);
            for (uint64_t i = k; i < len; ++i) {
                raw = rh.roll(s[i - k], s[i]);
                c = cms.add_and_estimate(raw);
                mixed = splitmix64(raw);
                hll_total.add_hash(mixed);
                if (c >= 2) hll_solid.add_hash(mixed);
            }
        }
        if (pair_count >= 5000 && pair_count % 2000 == 0) {  // estimator.rs:366-375
            uint64_t u1 = f64_to_u64_sat(std::round(hll_total.estimate()));
            uint64_t u2 = f64_to_u64_sat(std::round(hll_solid.estimate()));
            uint64_t e1 = u1 > u2 ? u1 - u2 : 0;
            uint64_t m_tr = m_sample > e1 ? m_sample - e1 : 0;
            double lam = u2 > 0 ? (double)m_tr / (double)u2 : 0.0;
            if (lam >= 15.0) break;
        }
    }
    if (pair_count == 0) return -1;  // "Input FASTQ files contain 0 valid read pairs"
    uint64_t u_ge_1 = f64_to_u64_sat(std::round(hll_total.estimate()));
    uint64_t u_ge_2 = f64_to_u64_sat(std::round(hll_solid.estimate()));
    uint64_t e_1 = u_ge_1 > u_ge_2 ? u_ge_1 - u_ge_2 : 0;
    uint64_t m_true = m_sample > e_1 ? m_sample - e_1 : 0;
    double lambda_s = u_ge_2 > 0 ? (double)m_true / (double)u_ge_2 : 0.0;
    double p_ge_2 = 1.0 - (1.0 + lambda_s) * std::exp(-lambda_s);
    uint64_t est_g;
    if (p_ge_2 > 0.05) est_g = f64_to_u64_sat(std::round((double)u_ge_2 / p_ge_2));
    else est_g = u_ge_2 > 10000 ? u_ge_2 : 10000;
    if (est_g < 10000) est_g = 10000;
    double estimated_cov = (double)stats->total_bases / (double)est_g;
    double d_k = estimated_cov * ((stats->mean_read_len - (double)k + 1.0) / stats->mean_read_len);
    double solid_ratio = u_ge_1 > 0 ? (double)u_ge_2 / (double)u_ge_1 : 0.0;
    int conf;
    if (d_k < 5.0 || solid_ratio < 0.05 || u_ge_2 < 1000) conf = 2;
    else if (d_k < 20.0 || solid_ratio < 0.15) conf = 1;
    else conf = 0;
    double ssf = 1.0;
    if (target_cov > 0.0 && estimated_cov > 1.5 * target_cov) {
        ssf = target_cov / estimated_cov;
        if (ssf < 0.01) ssf = 0.01;
        if (ssf > 1.0) ssf = 1.0;
    }
    std::vector<uint64_t> ks;
    compute_dynamic_kmers(stats->median_read_len, -1, ks);
    memset(out, 0, sizeof(*out));
    out->genome_size = est_g;
    out->exact_read_pairs = stats->exact_read_pairs;
    out->total_bases = stats->total_bases;
    out->median_read_len = stats->median_read_len;
    out->max_read_len = stats->max_read_len;
    out->estimated_cov = estimated_cov;
    out->subsample_factor = ssf;
    out->n_kmers = ks.size();
    for (size_t i = 0; i < ks.size() && i < 8; ++i) out->kmers[i] = ks[i];
    out->confidence = conf;
    out->u_ge_1 = u_ge_1;
    out->u_ge_2 = u_ge_2;
    out->sample_kmer_depth = lambda_s;
    out->pairs_sampled = pair_count;
    out->m_sample = m_sample;
    if (regs_total) memcpy(regs_total, hll_total.reg.data(), hll_total.reg.size());
    if (regs_solid) memcpy(regs_solid, hll_solid.reg.data(), hll_solid.reg.size());
    return 0;
}

// The estimator sample loop split by pair range, for the sharded-estimator tests: a
// rank's part of the first-touch form of estimator.rs:338-363 (the estimate after the
// add at occurrence t is >= 2 iff every row's counter was touched before t).  Reads are
// as in orc_estimate_from_reads over the first n_use pairs; t counts the k-mers of all
// pairs before pair_begin.  orc_est_firstpos fills first[4*cms_width] with the smallest
// t of [pair_begin, pair_end) touching each counter (0xFFFFFFFF if none);
// orc_est_segments writes, from a merged first array, the HLL register maxima of the
// range per checkpoint segment (segment 0 = pairs 1..6000, segment j = pairs
// 6000+2000(j-1)+1 .. 6000+2000j), regs[2][n_segs][1 << hll_p]: total, then solid.
template <class F>
static void est_walk(const uint8_t* reads, const uint64_t* read_offs, uint64_t pair_begin, uint64_t pair_end, unsigned k,
                     F&& f) {
    uint64_t t = 0;
    for (uint64_t r = 0; r < 2 * pair_begin; ++r) {
        const uint64_t len = read_offs[r + 1] - read_offs[r];
        if (len >= k) t += len - k + 1;
    }
    for (uint64_t p = pair_begin; p < pair_end; ++p)
        for (int mate = 0; mate < 2; ++mate) {
            const uint8_t* s = reads + read_offs[2 * p + mate];
            const uint64_t len = read_offs[2 * p + mate + 1] - read_offs[2 * p + mate];
            if (len < k) continue;
            RollingNtHash rh(s, k);
            f(p, t++, rh.canonical());
            for (uint64_t i = k; i < len; ++i) f(p, t++, rh.roll(s[i - k], s[i]));
        }
}

ORC_API void orc_est_firstpos(const uint8_t* reads, const uint64_t* read_offs, uint64_t pair_begin, uint64_t pair_end,
                              unsigned k, uint64_t cms_width, uint32_t* first) {
    std::fill(first, first + 4 * cms_width, 0xFFFFFFFFu);
    est_walk(reads, read_offs, pair_begin, pair_end, k, [&](uint64_t, uint64_t t, uint64_t raw) {
        for (int r = 0; r < 4; ++r) {
            uint32_t& f = first[(uint64_t)r * cms_width + (splitmix64(raw ^ CMS_SEEDS[r]) & (cms_width - 1))];
            if (t < f) f = (uint32_t)t;
        }
    });
}

ORC_API void orc_est_segments(const uint8_t* reads, const uint64_t* read_offs, uint64_t n_use, uint64_t pair_begin,
                              uint64_t pair_end, unsigned k, uint64_t cms_width, unsigned hll_p, const uint32_t* first,
                              uint8_t* regs) {
    const uint32_t n_segs = n_use <= 6000 ? 1u : (uint32_t)(1 + (n_use - 6000 + 1999) / 2000);
    const uint64_t m = 1ULL << hll_p;
    std::fill(regs, regs + 2 * n_segs * m, 0);
    est_walk(reads, read_offs, pair_begin, pair_end, k, [&](uint64_t p, uint64_t t, uint64_t raw) {
        const uint64_t pc = p + 1;
        uint32_t seg = pc <= 6000 ? 0u : (uint32_t)(1 + (pc - 6001) / 2000);
        if (seg >= n_segs) seg = n_segs - 1;
        bool solid = true;
        for (int r = 0; r < 4; ++r)
            solid = solid && first[(uint64_t)r * cms_width + (splitmix64(raw ^ CMS_SEEDS[r]) & (cms_width - 1))] < t;
        const uint64_t h = splitmix64(raw);
        const uint64_t idx = h >> (64 - hll_p), w = h & ((1ULL << (64 - hll_p)) - 1);
        const uint8_t rho = w == 0 ? (uint8_t)(64 - hll_p + 1) : (uint8_t)(__builtin_clzll(w) - hll_p + 1);
        uint8_t* tot = regs + (uint64_t)seg * m;
        uint8_t* sol = regs + ((uint64_t)n_segs + seg) * m;
        if (rho > tot[idx]) tot[idx] = rho;
        if (solid && rho > sol[idx]) sol[idx] = rho;
    });
}

// count_fastx_exact — estimator.rs:167-283.  Returns 0, or -1 with the reference's
// error message text in err.
ORC_API int orc_count_fastx_exact(const char* r1, const char* r2, orc_count_stats* out, char* err, int errlen) {
    auto fail = [&](const std::string& m) { if (err && errlen > 0) snprintf(err, errlen, "%s", m.c_str()); return -1; };
    FastqReader a(r1), b(r2);
    if (!a.f) return fail(std::string("Failed to open file ") + r1);
    if (!b.f) return fail(std::string("Failed to open file ") + r2);
    uint64_t pairs = 0, tb1 = 0, tb2 = 0, mn = UINT64_MAX, mx = 0;
    std::vector<uint64_t> hist(4096, 0), overflow;
    std::string e1, e2;
    char msg[512];
    for (;;) {
        int x = a.next(e1), y = b.next(e2);
        if (x == 1 && y == 1) {
            pairs++;
            std::string p1 = read_id_prefix(a.hdr), p2 = read_id_prefix(b.hdr);
            if (p1 != p2) {
                snprintf(msg, sizeof msg, "FASTQ paired-end synchronization error at pair #%llu: R1 ID '\"%s\"' does not match R2 ID '\"%s\"'",
                         (unsigned long long)pairs, a.hdr.c_str(), b.hdr.c_str());
                return fail(msg);
            }
            uint64_t l1 = a.seq.size(), l2 = b.seq.size();
            tb1 += l1; tb2 += l2;
            mn = std::min(mn, std::min(l1, l2));
            mx = std::max(mx, std::max(l1, l2));
            if (l1 < 4096) hist[l1]++; else overflow.push_back(l1);
            if (l2 < 4096) hist[l2]++; else overflow.push_back(l2);
        } else if (x == 0 && y == 0) {
            break;
        } else if (x == 1 && y == 0) {
            snprintf(msg, sizeof msg, "FASTQ pairing mismatch: R1 has more reads than R2 (R2 ended prematurely after %llu pairs)", (unsigned long long)pairs);
            return fail(msg);
        } else if (x == 0 && y == 1) {
            snprintf(msg, sizeof msg, "FASTQ pairing mismatch: R2 has more reads than R1 (R1 ended prematurely after %llu pairs)", (unsigned long long)pairs);
            return fail(msg);
        } else if (x < 0) {
            snprintf(msg, sizeof msg, "Corrupted/truncated FASTQ record in R1 at pair #%llu: %s", (unsigned long long)(pairs + 1), e1.c_str());
            return fail(msg);
        } else {
            snprintf(msg, sizeof msg, "Corrupted/truncated FASTQ record in R2 at pair #%llu: %s", (unsigned long long)(pairs + 1), e2.c_str());
            return fail(msg);
        }
    }
    if (pairs == 0) return fail("Input FASTQ files contain 0 valid read pairs");
    uint64_t total = tb1 + tb2, reads = pairs * 2;
    uint64_t target = (reads + 1) / 2, cum = 0, med = 0;
    for (uint64_t l = 0; l < 4096; ++l) {
        cum += hist[l];
        if (cum >= target) { med = l; break; }
    }
    if (med == 0 && !overflow.empty()) {
        std::sort(overflow.begin(), overflow.end());
        med = overflow[std::min(overflow.size() / 2, overflow.size() - 1)];
    }
    out->exact_read_pairs = pairs;
    out->total_bases_r1 = tb1;
    out->total_bases_r2 = tb2;
    out->total_bases = total;
    out->min_read_len = mn;
    out->max_read_len = mx;
    out->mean_read_len = (double)total / (double)reads;
    out->median_read_len = med;
    return 0;
}

// estimate_genome — estimator.rs:286-440, reading the same two FASTQ files.
ORC_API int orc_estimate_genome(const char* r1, const char* r2, uint64_t max_pairs, double target_cov, orc_genome_estimate* out,
                        uint8_t* regs_total, uint8_t* regs_solid, char* err, int errlen) {
    orc_count_stats st;
    if (orc_count_fastx_exact(r1, r2, &st, err, errlen) != 0) return -1;
    uint64_t sample_target = std::min<uint64_t>(std::min<uint64_t>(max_pairs, 150000), st.exact_read_pairs);
    FastqReader a(r1), b(r2);
    std::vector<uint8_t> buf;
    std::vector<uint64_t> offs(1, 0);
    std::string e;
    uint64_t n = 0;
    while (n < sample_target) {
        if (a.next(e) != 1 || b.next(e) != 1) break;
        buf.insert(buf.end(), a.seq.begin(), a.seq.end());
        offs.push_back(buf.size());
        buf.insert(buf.end(), b.seq.begin(), b.seq.end());
        offs.push_back(buf.size());
        n++;
    }
    int rc = orc_estimate_from_reads(buf.data(), offs.data(), n, &st, max_pairs, target_cov, 21, 1ULL << 23, 14, out,
                                     regs_total, regs_solid);
    if (rc != 0 && err && errlen > 0) snprintf(err, errlen, "Input FASTQ files contain 0 valid read pairs");
    return rc;
}

// ===========================================================================
// Unitig compaction — build.rs:330-594 (boundary walks, circular components,
// overlap edges) over SolidKmerNode rows.  The reference keeps the nodes in 64
// hashbrown shards (shard = splitmix64(to_u64) & 63, build.rs:152-153) and walks
// them in map order; here std::unordered_map stands in, so the emission order (and,
// for circular components, the start of the rotation) may differ — results are
// compared as multisets.
// ===========================================================================
#include <unordered_map>

namespace {

template <class K>
struct KHash {
    size_t operator()(const K& x) const { return (size_t)splitmix64(x.to_u64()); }
};
template <class K>
struct KEq {
    bool operator()(const K& a, const K& b) const { return !(a < b) && !(b < a); }
};

struct SNode {
    uint16_t cov;
    uint8_t mask;
    uint8_t visited;
};

template <class K>
static std::string kmer_ascii(const K& x, unsigned k) {  // KmerInt::to_ascii (kmer.rs:83-90)
    constexpr int NW = sizeof(K) / 8 > 4 ? 4 : (int)(sizeof(K) / 8);
    uint64_t w[4] = {0, 0, 0, 0};
    x.words(w);
    const int nw = std::is_same<K, K64>::value ? 1 : std::is_same<K, K128>::value ? 2 : 4;
    (void)NW;
    std::string s(k, 'A');
    for (unsigned i = 0; i < k; ++i) {  // base i from the 3' end
        const unsigned bit = 2 * i;
        const uint64_t word = w[nw - 1 - bit / 64];
        const unsigned code = (unsigned)(word >> (bit % 64)) & 3u;
        s[k - 1 - i] = "ACGT"[code];
    }
    return s;
}

static std::string rc_ascii(const std::string& s) {  // reverse_complement_ascii (bitseq.rs:90-98)
    std::string r(s.size(), 'A');
    for (size_t i = 0; i < s.size(); ++i) r[s.size() - 1 - i] = "TGCA"[A2B.t[(uint8_t)s[i]]];
    return r;
}

struct OUnitig {
    std::string seq;
    float cov;
    bool circular;
    // (target id, target rc, overlap, support) per side
    std::vector<std::array<uint32_t, 4>> edges[2];
    void add_edge(bool rc_side, uint32_t tid, bool trc, uint32_t ov, uint32_t support) {  // cdbg.rs:113-122
        for (auto& e : edges[rc_side]) {
            if (e[0] == tid && e[1] == (uint32_t)trc && e[2] == ov) {
                e[3] = std::min<uint32_t>(65535, e[3] + support);
                return;
            }
        }
        edges[rc_side].push_back({tid, (uint32_t)trc, ov, support});
    }
};

template <class K>
static std::vector<OUnitig> compact_impl(unsigned k, const uint64_t* keys, const uint16_t* cov, const uint8_t* mask, uint64_t n) {
    constexpr int NWK = std::is_same<K, K64>::value ? 1 : std::is_same<K, K128>::value ? 2 : 4;
    using Map = std::unordered_map<K, SNode, KHash<K>, KEq<K>>;
    std::vector<Map> shards(64);
    auto shard_of = [](const K& x) { return (size_t)(splitmix64(x.to_u64()) & 63); };
    for (uint64_t i = 0; i < n; ++i) {
        K x = from_words<K>(keys + i * NWK);
        shards[shard_of(x)][x] = SNode{cov[i], mask[i], 0};
    }
    auto find = [&](const K& x) -> SNode* {
        auto& m = shards[shard_of(x)];
        auto it = m.find(x);
        return it == m.end() ? nullptr : &it->second;
    };
    std::vector<OUnitig> out;
    auto pc = [](uint8_t v) { return __builtin_popcount(v); };
    // 4. boundary directed k-mers (in_deg != 1 || out_deg != 1), build.rs:332-347
    std::vector<std::pair<K, bool>> boundary;
    for (auto& sh : shards)
        for (auto& kv : sh) {
            const uint8_t m = kv.second.mask;
            if (pc(m >> 4 & 0xF) != 1 || pc(m & 0xF) != 1) boundary.push_back({kv.first, false});
            if (pc(m & 0xF) != 1 || pc(m >> 4 & 0xF) != 1) boundary.push_back({kv.first, true});
        }
    auto next_dir = [&](const K& fwd, const K& rev, uint8_t b, K& can, bool& is_rc) {
        K nf = fwd, nr = rev;
        K::roll_next(nf, nr, b, k);
        is_rc = nr < nf;
        can = is_rc ? nr : nf;
    };
    auto oriented = [&](const K& kmer, bool is_rc, K& f, K& r) {
        if (!is_rc) {
            f = kmer;
            r = kmer.rev_comp(k);
        } else {
            f = kmer.rev_comp(k);
            r = kmer;
        }
    };
    // build.rs:349-445
    for (auto& u : boundary) {
        for (uint8_t b = 0; b < 4; ++b) {
            SNode* nu = find(u.first);
            if (!nu) break;
            const uint8_t u_out = !u.second ? (nu->mask & 0x0F) : ((nu->mask >> 4) & 0x0F);
            const uint8_t u_vis = !u.second ? (nu->visited & 0x0F) : ((nu->visited >> 4) & 0x0F);
            if (!((u_out >> b) & 1) || ((u_vis >> b) & 1)) continue;
            nu->visited |= (uint8_t)(1u << (!u.second ? b : b + 4));
            std::string path = kmer_ascii(u.first, k);
            if (u.second) path = rc_ascii(path);
            K fwd, rev;
            oriented(u.first, u.second, fwd, rev);
            const uint8_t rc_first = 3 - A2B.t[(uint8_t)kmer_ascii(fwd, k)[0]];
            K cur;
            bool cur_rc;
            next_dir(fwd, rev, b, cur, cur_rc);
            if (SNode* nc = find(cur)) nc->visited |= (uint8_t)(1u << (!cur_rc ? rc_first + 4 : rc_first));
            path.push_back("ACGT"[b]);
            uint64_t total_cov = nu->cov, points = 1;
            for (;;) {
                SNode* ncp = find(cur);
                if (!ncp) break;
                const SNode nc = *ncp;
                const uint8_t c_out = !cur_rc ? (nc.mask & 0x0F) : ((nc.mask >> 4) & 0x0F);
                const uint8_t c_in = !cur_rc ? ((nc.mask >> 4) & 0x0F) : (nc.mask & 0x0F);
                if (pc(c_in) != 1 || pc(c_out) != 1) break;
                const uint8_t nb = (uint8_t)__builtin_ctz(c_out);
                const uint8_t ebit = !cur_rc ? nb : nb + 4;
                if ((nc.visited >> ebit) & 1) break;
                ncp->visited |= (uint8_t)(1u << ebit);
                K cf, cr;
                oriented(cur, cur_rc, cf, cr);
                const uint8_t rc_p = 3 - A2B.t[(uint8_t)kmer_ascii(cf, k)[0]];
                K nxt;
                bool nxt_rc;
                next_dir(cf, cr, nb, nxt, nxt_rc);
                if (SNode* nn = find(nxt)) nn->visited |= (uint8_t)(1u << (!nxt_rc ? rc_p + 4 : rc_p));
                path.push_back("ACGT"[nb]);
                total_cov += nc.cov;
                points++;
                cur = nxt;
                cur_rc = nxt_rc;
            }
            const std::string rcs = rc_ascii(path);
            OUnitig t;
            t.seq = rcs < path ? rcs : path;
            t.cov = std::max(1.0f, (float)total_cov / (float)points);
            t.circular = false;
            out.push_back(std::move(t));
        }
    }
    // 5. isolated circular components, build.rs:450-555
    for (size_t s = 0; s < 64; ++s) {
        std::vector<K> ks;
        for (auto& kv : shards[s]) ks.push_back(kv.first);
        for (const K& kmer : ks) {
            SNode* np = find(kmer);
            if (!np) continue;
            const SNode n0 = *np;
            const uint8_t fo = n0.mask & 0x0F, fi = (n0.mask >> 4) & 0x0F;
            if (pc(fo) != 1 || pc(fi) != 1) continue;
            const uint8_t b = (uint8_t)__builtin_ctz(fo);
            if ((n0.visited >> b) & 1) continue;
            np->visited |= (uint8_t)(1u << b);
            std::string path = kmer_ascii(kmer, k);
            const K fwd = kmer, rev = kmer.rev_comp(k);
            K cur;
            bool cur_rc;
            next_dir(fwd, rev, b, cur, cur_rc);
            const uint8_t rc_first = 3 - A2B.t[(uint8_t)kmer_ascii(fwd, k)[0]];
            if (SNode* nc = find(cur)) nc->visited |= (uint8_t)(1u << (!cur_rc ? rc_first + 4 : rc_first));
            path.push_back("ACGT"[b]);
            uint64_t total_cov = n0.cov, points = 1;
            while (!KEq<K>()(cur, kmer)) {
                SNode* ncp = find(cur);
                if (!ncp) break;
                const SNode nc = *ncp;
                const uint8_t c_out = !cur_rc ? (nc.mask & 0x0F) : ((nc.mask >> 4) & 0x0F);
                const uint8_t c_in = !cur_rc ? ((nc.mask >> 4) & 0x0F) : (nc.mask & 0x0F);
                if (pc(c_in) != 1 || pc(c_out) != 1) break;
                const uint8_t nb = (uint8_t)__builtin_ctz(c_out);
                const uint8_t ebit = !cur_rc ? nb : nb + 4;
                if ((nc.visited >> ebit) & 1) break;
                ncp->visited |= (uint8_t)(1u << ebit);
                K cf, cr;
                oriented(cur, cur_rc, cf, cr);
                const uint8_t rc_p = 3 - A2B.t[(uint8_t)kmer_ascii(cf, k)[0]];
                K nxt;
                bool nxt_rc;
                next_dir(cf, cr, nb, nxt, nxt_rc);
                if (SNode* nn = find(nxt)) nn->visited |= (uint8_t)(1u << (!nxt_rc ? rc_p + 4 : rc_p));
                path.push_back("ACGT"[nb]);
                total_cov += nc.cov;
                points++;
                cur = nxt;
                cur_rc = nxt_rc;
            }
            if (KEq<K>()(cur, kmer) && path.size() > k) {
                if (path.size() > k && path.compare(path.size() - k, k, path, 0, k) == 0) path.resize(path.size() - k);
                else if (path.size() > k - 1 && path.compare(path.size() - (k - 1), k - 1, path, 0, k - 1) == 0)
                    path.resize(path.size() - (k - 1));
                OUnitig t;
                t.seq = path;
                t.cov = std::max(1.0f, (float)total_cov / (float)points);
                t.circular = true;
                const uint32_t id = (uint32_t)out.size();
                t.add_edge(false, id, false, k - 1, 10);
                out.push_back(std::move(t));
            }
        }
    }
    // 6. overlap edges of k and k-1 bases, build.rs:558-594
    for (unsigned ov : {k, k - 1}) {
        if (ov == 0) continue;
        std::unordered_map<std::string, std::vector<std::pair<uint32_t, bool>>> prefix;
        for (uint32_t id = 0; id < out.size(); ++id) {
            const std::string& f = out[id].seq;
            if (f.size() >= ov) {
                prefix[f.substr(0, ov)].push_back({id, false});
                prefix[rc_ascii(f).substr(0, ov)].push_back({id, true});
            }
        }
        for (uint32_t id = 0; id < out.size(); ++id) {
            const std::string f = out[id].seq, r = rc_ascii(f);
            if (f.size() < ov) continue;
            auto a = prefix.find(f.substr(f.size() - ov));
            if (a != prefix.end())
                for (auto& t : a->second)
                    if (t.first != id || out[id].circular) out[id].add_edge(false, t.first, t.second, ov, 10);
            auto c = prefix.find(r.substr(r.size() - ov));
            if (c != prefix.end())
                for (auto& t : c->second)
                    if (t.first != id || out[id].circular) out[id].add_edge(true, t.first, t.second, ov, 10);
        }
    }
    return out;
}

struct OCompacted {
    std::vector<OUnitig> u;
};

}  // namespace

// Compaction oracle: SolidKmerNode rows in, unitigs out (an opaque handle).
ORC_API void* orc_compact(int key_bits, unsigned k, const uint64_t* keys, const uint16_t* cov, const uint8_t* mask, uint64_t n) {
    auto* c = new OCompacted();
    if (key_bits == 64) c->u = compact_impl<K64>(k, keys, cov, mask, n);
    else if (key_bits == 128) c->u = compact_impl<K128>(k, keys, cov, mask, n);
    else if (key_bits == 256) c->u = compact_impl<K256>(k, keys, cov, mask, n);
    else {
        delete c;
        return nullptr;
    }
    return c;
}
ORC_API uint64_t orc_compact_count(const void* h) { return ((const OCompacted*)h)->u.size(); }
ORC_API uint64_t orc_compact_bases(const void* h) {
    uint64_t t = 0;
    for (auto& u : ((const OCompacted*)h)->u) t += u.seq.size();
    return t;
}
ORC_API uint64_t orc_compact_n_edges(const void* h) {
    uint64_t t = 0;
    for (auto& u : ((const OCompacted*)h)->u) t += u.edges[0].size() + u.edges[1].size();
    return t;
}
// seqs: concatenated ASCII; offs: n+1; cov; circular; edges: 6 u32 per edge
// (from id, from side, to id, to rc, overlap, support)
ORC_API void orc_compact_export(const void* h, uint8_t* seqs, uint64_t* offs, float* cov, uint8_t* circular, uint32_t* edges) {
    const auto& U = ((const OCompacted*)h)->u;
    uint64_t p = 0, e = 0;
    offs[0] = 0;
    for (size_t i = 0; i < U.size(); ++i) {
        memcpy(seqs + p, U[i].seq.data(), U[i].seq.size());
        p += U[i].seq.size();
        offs[i + 1] = p;
        cov[i] = U[i].cov;
        circular[i] = U[i].circular;
        for (int side = 0; side < 2; ++side)
            for (auto& ed : U[i].edges[side]) {
                uint32_t* o = edges + 6 * e++;
                o[0] = (uint32_t)i;
                o[1] = (uint32_t)side;
                o[2] = ed[0];
                o[3] = ed[1];
                o[4] = ed[2];
                o[5] = ed[3];
            }
    }
}
ORC_API void orc_compact_free(void* h) { delete (OCompacted*)h; }

// ===========================================================================
// filter_active_reads — local_multik.rs:259-333.  unitigs: ASCII + offsets, circular
// flags, edge counts per side; arenas: merged, pe_forward, pe_reverse.  keep: one byte
// per read in that order.
// ===========================================================================
#include <unordered_set>

static std::string arena_read(const orc_arena& a, uint64_t i) {  // BitSeqArena::extract_ascii_into
    std::string s(a.lengths[i], 'A');
    for (uint32_t j = 0; j < a.lengths[i]; ++j) {
        const uint64_t p = a.offsets[i] + j;
        s[j] = "ACGT"[(a.data[p >> 5] >> ((p & 31) * 2)) & 3];
    }
    return s;
}

ORC_API uint64_t orc_filter_active_reads(const orc_arena* arenas, const uint8_t* useq, const uint64_t* uoff, const uint8_t* circular,
                                         const uint32_t* efwd, const uint32_t* erev, uint64_t n_unitigs, unsigned graph_k,
                                         uint8_t* keep) {
    const unsigned k = std::min(graph_k, 31u);
    const uint64_t W = 350;
    std::unordered_set<uint64_t> boundary;
    auto h = [&](const char* s) { return orc_nthash_canonical((const uint8_t*)s, k); };
    for (uint64_t u = 0; u < n_unitigs; ++u) {
        const std::string seq((const char*)useq + uoff[u], uoff[u + 1] - uoff[u]);
        if (seq.size() < k) continue;
        if (seq.size() < 2000 || circular[u] || efwd[u] > 1 || erev[u] > 1) {
            for (size_t i = 0; i + k <= seq.size(); ++i) boundary.insert(h(seq.data() + i));
        } else {
            const size_t left = std::min<size_t>(W, seq.size() - k + 1);
            for (size_t i = 0; i < left; ++i) boundary.insert(h(seq.data() + i));
            const size_t right = std::min<size_t>(seq.size() > W ? seq.size() - W : 0, seq.size() - k);
            for (size_t i = right; i <= seq.size() - k; ++i) boundary.insert(h(seq.data() + i));
        }
    }
    auto active = [&](const std::string& s) {
        if (s.size() < k) return false;
        const size_t offs[3] = {0, (s.size() - k) / 2, s.size() - k};
        for (size_t o : offs)
            if (boundary.count(h(s.data() + o))) return true;
        return false;
    };
    uint64_t kept = 0, r = 0;
    const uint64_t M = arenas[0].n_seqs, F = arenas[1].n_seqs, R = arenas[2].n_seqs;
    for (uint64_t i = 0; i < M; ++i, ++r) kept += keep[r] = active(arena_read(arenas[0], i));
    for (uint64_t i = 0; i < F + R; ++i) keep[M + i] = 0;
    const uint64_t pe = std::min(F, R);
    for (uint64_t i = 0; i < pe; ++i) {
        const uint8_t kp = active(arena_read(arenas[1], i)) || active(arena_read(arenas[2], i));
        keep[M + i] = keep[M + F + i] = kp;
        kept += 2 * kp;
    }
    return kept;
}

// ===========================================================================
// index_terminal_kmers — src/resolve/mapper.rs:89-136 (sorted by key for comparison)
// ===========================================================================
template <class K>
static uint64_t term_index_impl(unsigned k, const uint8_t* useq, const uint64_t* uoff, uint64_t n, uint64_t* keys, uint32_t* unitig,
                                uint8_t* is_rc, uint32_t* pos, uint64_t cap) {
    std::unordered_map<uint64_t, uint32_t> counts;
    std::unordered_map<uint64_t, std::pair<uint32_t, uint32_t>> where;  // (id << 1 | is_rc, i)
    for (uint64_t id = 0; id < n; ++id) {
        const uint8_t* seq = useq + uoff[id];
        const uint64_t len = uoff[id + 1] - uoff[id];
        if (len < k) continue;
        const uint64_t total = len - k + 1;
        auto index_kmer = [&](uint64_t i) {
            const K f = K::from_ascii(seq + i, k), r = f.rev_comp(k);
            const bool rc = r < f;
            const uint64_t h = (rc ? r : f).to_u64();
            counts[h] += 1;
            where[h] = {(uint32_t)(id << 1 | (rc ? 1 : 0)), (uint32_t)i};
        };
        if (total <= 2000) {
            for (uint64_t i = 0; i < total; ++i) index_kmer(i);
        } else {
            for (uint64_t i = 0; i < 1000; ++i) index_kmer(i);
            for (uint64_t i = total - 1000; i < total; ++i) index_kmer(i);
        }
    }
    std::vector<std::pair<uint64_t, std::pair<uint32_t, uint32_t>>> out;
    for (auto& kv : where)
        if (counts[kv.first] == 1) out.push_back(kv);
    std::sort(out.begin(), out.end());
    for (uint64_t i = 0; i < out.size() && i < cap; ++i) {
        keys[i] = out[i].first;
        unitig[i] = out[i].second.first >> 1;
        is_rc[i] = out[i].second.first & 1;
        pos[i] = out[i].second.second;
    }
    return out.size();
}

ORC_API uint64_t orc_index_terminal_kmers(int key_bits, unsigned k, const uint8_t* useq, const uint64_t* uoff, uint64_t n,
                                          uint64_t* keys, uint32_t* unitig, uint8_t* is_rc, uint32_t* pos, uint64_t cap) {
    if (key_bits == 64) return term_index_impl<K64>(k, useq, uoff, n, keys, unitig, is_rc, pos, cap);
    if (key_bits == 128) return term_index_impl<K128>(k, useq, uoff, n, keys, unitig, is_rc, pos, cap);
    return term_index_impl<K256>(k, useq, uoff, n, keys, unitig, is_rc, pos, cap);
}

// ===========================================================================
// Read ingest — src/ingest/trim_merge.rs:17-238 (adapter clip, quality trim,
// FLASH-style overlap merge) and :307-417 (the ingest loop that fills a ReadBank).
// A literal restatement over ASCII records, kept apart from the library's own host
// and device ingest so that both can be checked against it.
// ===========================================================================
namespace orc_ingest {

static const char* ADAPTERS_AGAT[2] = {"AGATCGGAAGAGC", "AGATGTGTATAAGAGACAG"};  // trim_merge.rs:12-13
static const char* ADAPTER_CTGT = "CTGTCTCTTATACACATCT";                          // trim_merge.rs:14

static inline uint8_t upper(uint8_t c) { return (c >= 'a' && c <= 'z') ? (uint8_t)(c - 32) : c; }
static inline bool eq_nocase(uint8_t a, uint8_t b) { return upper(a) == upper(b); }

// At most one mismatch over the adapter's first min(10, len) bases at seq + i.
static bool adapter_at(const uint8_t* seq, uint64_t i, const char* adapter) {
    const uint64_t n = std::min<uint64_t>(10, strlen(adapter));
    unsigned mm = 0;
    for (uint64_t j = 0; j < n; ++j)
        if (!eq_nocase(seq[i + j], (uint8_t)adapter[j]) && ++mm > 1) return false;
    return true;
}

// trim_adapter — trim_merge.rs:17-76: the kept length.
static uint64_t trim_adapter(const uint8_t* seq, uint64_t len) {
    if (len < 10) return len;
    uint64_t cut = len;
    const uint64_t start = len > 100 ? len - 100 : 0;
    for (uint64_t i = start; i + 10 <= len; ++i) {
        const uint8_t b0 = upper(seq[i]), b1 = upper(seq[i + 1]);
        const bool agat = (b0 == 'A' && b1 == 'G') || b0 == 'A' || b1 == 'G';
        const bool ctgt = (b0 == 'C' && b1 == 'T') || b0 == 'C' || b1 == 'T';
        if (!agat && !ctgt) continue;
        if (agat)
            for (const char* a : ADAPTERS_AGAT)
                if (adapter_at(seq, i, a)) {
                    cut = std::min(cut, i);
                    break;
                }
        if (ctgt && cut > i && adapter_at(seq, i, ADAPTER_CTGT)) cut = std::min(cut, i);
    }
    return cut;
}

// trim_quality — trim_merge.rs:79-115: the kept length, or -1 for None.
static int64_t trim_quality(const uint8_t* qual, uint64_t len, uint64_t qual_len, unsigned min_qual, uint64_t min_len) {
    if (len < min_len || qual_len != len) return -1;
    uint64_t cut = len;
    const uint64_t W = 4;
    auto wsum = [&](uint64_t end) {
        uint64_t s = 0;
        for (uint64_t j = end - W; j < end; ++j) s += qual[j] > 33 ? qual[j] - 33 : 0;
        return s;
    };
    if (qual_len >= W) {
        if (wsum(cut) >= (uint64_t)min_qual * W) return (int64_t)len;
        while (cut >= W) {
            if (wsum(cut) / W >= min_qual) break;
            --cut;
        }
    }
    return cut < min_len ? -1 : (int64_t)cut;
}

// merge_read_pair — trim_merge.rs:135-238.  Returns the merged sequence's length
// (written to out) or -1 for Unmerged.
static int64_t merge_read_pair(const uint8_t* r1, const uint8_t* q1, uint64_t l1, uint64_t q1_len, const uint8_t* r2,
                               const uint8_t* q2, uint64_t l2, uint64_t q2_len, uint64_t min_overlap, double max_ratio,
                               std::vector<uint8_t>& out, uint64_t* overlap, uint64_t* mismatches) {
    if (l1 < min_overlap || l2 < min_overlap) return -1;
    // Reverse complement of R2.  A base other than ACGT (either case) becomes 'A' for
    // reads of up to 512 bases (the stack path, trim_merge.rs:152-162) but 'T' for longer
    // ones (reverse_complement_ascii, bitseq.rs:90-98, reads it as A and complements it).
    std::vector<uint8_t> rc2(l2);
    const uint8_t other = l2 <= 512 ? 'A' : TWO_BIT_TO_ASCII[COMPLEMENT_2BIT[A2B.t['N']]];
    for (uint64_t i = 0; i < l2; ++i) {
        switch (r2[l2 - 1 - i]) {
            case 'A': case 'a': rc2[i] = 'T'; break;
            case 'C': case 'c': rc2[i] = 'G'; break;
            case 'G': case 'g': rc2[i] = 'C'; break;
            case 'T': case 't': rc2[i] = 'A'; break;
            default: rc2[i] = other;
        }
    }
    const uint64_t max_d = std::min(l1, l2);
    uint64_t best_d = 0, best_mm = 0;
    double best_score = -INFINITY;
    for (uint64_t d = max_d; d >= min_overlap; --d) {
        const uint8_t* s1 = r1 + (l1 - d);
        const uint64_t allowed = (uint64_t)((double)d * max_ratio);
        uint64_t mm = 0;
        for (uint64_t i = 0; i < d; ++i)
            if (!eq_nocase(s1[i], rc2[i]) && ++mm > allowed) break;
        if (mm <= allowed) {
            const double score = (double)d - 2.5 * (double)mm;
            if (score > best_score) {
                best_score = score;
                best_d = d;
                best_mm = mm;
            }
        }
        if ((double)d <= best_score) break;
        if (d == 0) break;
    }
    if (best_d < min_overlap) return -1;
    out.clear();
    out.insert(out.end(), r1, r1 + (l1 - best_d));
    for (uint64_t i = 0; i < best_d; ++i) {
        const uint8_t b1 = r1[l1 - best_d + i], b2 = rc2[i];
        const uint8_t qa = (l1 - best_d + i) < q1_len ? q1[l1 - best_d + i] : 'I';
        const uint8_t qb = i < l2 ? ((l2 - 1 - i) < q2_len ? q2[l2 - 1 - i] : 'I') : 'I';
        if (eq_nocase(b1, b2) || qa >= qb) out.push_back(upper(b1));
        else out.push_back(upper(b2));
    }
    out.insert(out.end(), rc2.begin() + best_d, rc2.end());
    *overlap = best_d;
    *mismatches = best_mm;
    return (int64_t)out.size();
}

// BitSeqArena::push_seq — bitseq.rs:195-222, plus the input pair of the read.
struct OArena {
    std::vector<uint64_t> data, offsets;
    std::vector<uint32_t> lengths, pair_idx;
    uint64_t total = 0;
    void push(const uint8_t* s, uint64_t n, uint32_t pair) {
        offsets.push_back(total);
        lengths.push_back((uint32_t)n);
        pair_idx.push_back(pair);
        if (!n) return;
        const uint64_t end = total + n;
        if (data.size() < (end + 31) / 32) data.resize((end + 31) / 32, 0);
        for (uint64_t i = 0; i < n; ++i) {
            const uint64_t g = total + i;
            data[g >> 5] |= (uint64_t)A2B.t[s[i]] << ((g & 31) << 1);
        }
        total = end;
    }
};

struct OIngest {
    OArena a[3];  // merged_reads, pe_forward, pe_reverse (bitseq.rs:350-355)
    uint64_t stats[7] = {};  // IngestStats fields in declaration order, trim_merge.rs:262-271
};

}  // namespace orc_ingest

using namespace orc_ingest;

ORC_API uint64_t orc_trim_adapter(const uint8_t* seq, uint64_t len) { return orc_ingest::trim_adapter(seq, len); }
ORC_API int64_t orc_trim_quality(const uint8_t* qual, uint64_t len, unsigned min_qual, uint64_t min_len) {
    return orc_ingest::trim_quality(qual, len, len, min_qual, min_len);
}
ORC_API int64_t orc_merge_read_pair(const uint8_t* r1, const uint8_t* q1, uint64_t l1, const uint8_t* r2, const uint8_t* q2,
                                    uint64_t l2, uint64_t min_overlap, double max_ratio, uint8_t* out, uint64_t* overlap,
                                    uint64_t* mismatches) {
    std::vector<uint8_t> m;
    const int64_t n = orc_ingest::merge_read_pair(r1, q1, l1, l1, r2, q2, l2, l2, min_overlap, max_ratio, m, overlap, mismatches);
    if (n > 0) memcpy(out, m.data(), (size_t)n);
    return n;
}

// ingest_reads_ext_with_seed — trim_merge.rs:307-417.  Returns a handle, or null with
// the reference's error text in err.
ORC_API void* orc_ingest_fastq(const char* r1p, const char* r2p, double factor, uint64_t min_len, unsigned min_qual,
                               int enable_trim, int enable_merge, uint64_t seed, char* err, int errlen) {
    auto fail = [&](const std::string& m) -> void* {
        if (err && errlen > 0) snprintf(err, errlen, "%s", m.c_str());
        return nullptr;
    };
    FastqReader a(r1p), b(r2p);
    if (!a.f) return fail(std::string("Failed to open file ") + r1p);
    if (!b.f) return fail(std::string("Failed to open file ") + r2p);
    std::unique_ptr<OIngest> ing(new OIngest());
    uint64_t* st = ing->stats;  // input, retained, before, after, merged pairs, merged bases, unmerged
    const bool subsample = factor < 0.999;
    const uint64_t keep = f64_to_u64_sat(factor * 18446744073709551616.0);  // (f * u64::MAX as f64) as u64
    uint64_t pair = 0;
    std::string e1, e2;
    std::vector<uint8_t> merged;
    for (;;) {
        const int x = a.next(e1), y = b.next(e2);
        if (x == 0 && y == 0) break;
        if (x < 0) return fail("Corrupted record in R1 FASTQ: " + e1);
        if (y < 0) return fail("Corrupted record in R2 FASTQ: " + e2);
        if (x != y) return fail("Mismatched paired-end FASTQ mate counts between R1 and R2");
        ++pair;
        st[0]++;
        const uint8_t *s1 = (const uint8_t*)a.seq.data(), *q1 = (const uint8_t*)a.qual.data();
        const uint8_t *s2 = (const uint8_t*)b.seq.data(), *q2 = (const uint8_t*)b.qual.data();
        uint64_t l1 = a.seq.size(), l2 = b.seq.size();
        st[2] += l1 + l2;
        if (subsample && splitmix64(pair ^ seed) > keep) continue;
        if (enable_trim) {
            const uint64_t c1 = orc_ingest::trim_adapter(s1, l1), c2 = orc_ingest::trim_adapter(s2, l2);
            const int64_t t1 = orc_ingest::trim_quality(q1, c1, std::min<uint64_t>(c1, a.qual.size()), min_qual, min_len);
            const int64_t t2 = orc_ingest::trim_quality(q2, c2, std::min<uint64_t>(c2, b.qual.size()), min_qual, min_len);
            if (t1 < 0 || t2 < 0) continue;
            l1 = (uint64_t)t1;
            l2 = (uint64_t)t2;
        } else if (l1 < min_len || l2 < min_len) {
            continue;
        }
        st[1]++;
        st[3] += l1 + l2;
        uint64_t ov = 0, mm = 0;
        const int64_t n = enable_merge ? orc_ingest::merge_read_pair(s1, q1, l1, l1, s2, q2, l2, l2, 15, 0.10, merged, &ov, &mm) : -1;
        if (n >= 0) {
            st[4]++;
            st[5] += (uint64_t)n;
            ing->a[0].push(merged.data(), (uint64_t)n, (uint32_t)(pair - 1));
        } else {
            st[6]++;
            ing->a[1].push(s1, l1, (uint32_t)(pair - 1));
            ing->a[2].push(s2, l2, (uint32_t)(pair - 1));
        }
    }
    if (ing->a[0].lengths.empty() && ing->a[1].lengths.empty())
        return fail("No valid reads survived trimming and quality filtering (check input FASTQ files)");
    return ing.release();
}
ORC_API void orc_ingest_sizes(const void* h, int arena, uint64_t* n_words, uint64_t* n_seqs) {
    const OArena& a = ((const OIngest*)h)->a[arena];
    *n_words = a.data.size();
    *n_seqs = a.lengths.size();
}
ORC_API void orc_ingest_export(const void* h, int arena, uint64_t* data, uint64_t* offsets, uint32_t* lengths, uint32_t* pair_idx) {
    const OArena& a = ((const OIngest*)h)->a[arena];
    std::copy(a.data.begin(), a.data.end(), data);
    std::copy(a.offsets.begin(), a.offsets.end(), offsets);
    std::copy(a.lengths.begin(), a.lengths.end(), lengths);
    std::copy(a.pair_idx.begin(), a.pair_idx.end(), pair_idx);
}
ORC_API void orc_ingest_stats(const void* h, uint64_t* out7) { memcpy(out7, ((const OIngest*)h)->stats, 7 * sizeof(uint64_t)); }
ORC_API void orc_ingest_free(void* h) { delete (OIngest*)h; }
