// fbk_kernels.cuh — device views and kernel launchers shared by the CUDA
// translation units and the host API (fbk_api.cu).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace fbk {

// Read bank on the device: the three BitSeqArenas of a ReadBank concatenated
// (merged, pe_forward, pe_reverse — build.rs:90), offsets rebased onto one word
// array that carries 8 zero words of padding.
struct BankDev {
    const uint64_t* data;
    const uint64_t* off;       // base offset of each read
    const uint32_t* len;       // length of each read
    const uint32_t* pair_idx;  // input pair of each read (may be null)
    const uint64_t* keep_bits; // subsampler bitmap over input pairs (null = keep all)
    uint64_t r_begin, r_end;   // read range processed by a launch
};

__host__ __device__ inline bool bank_keep(const BankDev& b, uint64_t r) {
#ifdef __CUDA_ARCH__
    if (!b.keep_bits) return true;
    const uint32_t pi = b.pair_idx[r];
    return (b.keep_bits[pi >> 6] >> (pi & 63)) & 1ull;
#else
    (void)b; (void)r;
    return true;
#endif
}

// Open-addressing solid table.  NW == 1: keys[] holds the key itself (EMPTY = ~0;
// a k <= 31 key uses 62 bits).  NW == 2: keys[] holds the two words, claimed with one
// 16-byte CAS (EMPTY = all ones).  NW == 4: a tag claims the slot (0 empty,
// fingerprint, fingerprint|READY once the key words are published) and keys[] holds
// the four words.  The tag of slot s is tags[s * tag_stride]: for k <= 96 the key's
// most significant word is always zero, so the tag lives there (tags == keys, stride
// 4) and one 32-byte sector holds tag and key; for k > 96 tags[] is its own array
// (stride 1).  cnt[] holds 8 edge counters (u32) per slot, 32-byte aligned.
struct TableDev {
    uint64_t* keys;
    uint64_t* tags;
    uint32_t tag_stride;
    uint32_t* cnt;
    uint32_t* cov;       // separate cov counters, only when prior contigs are used
    uint64_t cap;        // slots (any size: home slot = high 64 bits of hash * cap)
    uint32_t max_probe;
    uint32_t spin_limit;
};

// Pass-2 records, grouped by the slot range of their key's home slot: the bucket of a
// key is the high 64 bits of its row-0 hash times the bucket count P, and its home slot
// the high bits of the same hash times the table capacity, so bucket b covers the
// home slots [b cap / P, (b + 1) cap / P) for any capacity (the table can be sized
// after the records are written).  Bucket b
// holds S stripes of stripe_cap records; warps append to stripe (warp % S) with one
// atomic per (warp iteration, bucket).  A record is the canonical key and the pushes
// it makes (the info byte: bits 0-2 edge as u, bit 3 present; bits 4-6 edge as v,
// bit 7 present), packed into rw = ceil((2k + 8) / 64) words (record_format).
struct BucketDev {
    uint64_t* recs;              // rw words per record
    unsigned long long* fill;    // P * S append counters
    uint64_t stripe_cap;
    uint32_t shift;              // host sizing: a bucket's table range is at most 2^shift slots
    uint32_t n_buckets, stripes; // bucket of a key = high 64 bits of (row-0 hash) x n_buckets
    uint32_t* overflow;          // set when a stripe runs out of room
    uint32_t rw, ws, packed;     // record layout (record_format)
};

// Record layout of a pass at k with NW-word keys.  The key's leading ws = (64 NW - 2k)
// / 64 words are zero and not stored; its significant words follow in big-endian
// order.  When the first significant word leaves its top 8 bits free (2k - 64 (NK - 1)
// <= 56 for NK = NW - ws significant words) the info byte goes there and a record is
// NK words (packed); otherwise the info byte takes a word of its own before the key
// (NK + 1 words).  k = 21: 1 word; k = 31: 2; k = 33 and 55: 2; k = 63: 3; k = 77: 3;
// k = 127: 5.
struct RecFmt {
    uint32_t rw, ws, packed;
};
__host__ __device__ inline RecFmt record_format(uint32_t k, int nw) {
    const uint32_t ws = (64u * (uint32_t)nw - 2u * k) >> 6;
    const uint32_t nk = (uint32_t)nw - ws;
    const uint32_t top_bits = 2u * k - 64u * (nk - 1);
    RecFmt f;
    f.ws = ws;
    f.packed = top_bits <= 56 ? 1u : 0u;
    f.rw = nk + (f.packed ? 0u : 1u);
    return f;
}

// Record filter of pass 2 (see k_count_records): 2^log2m counters, the threshold, and
// where the pushes of skipped records are counted.
struct RecordFilter {
    uint32_t* cnt;                 // nullptr: no filter
    uint32_t log2m;
    uint32_t min_records;
    unsigned long long* skipped;  // pushes of the records the upsert skipped
};

// Output of the SolidKmerNode conversion.
struct ConvOut {
    uint64_t* keys;             // n_solid * NW words
    uint16_t* cov;
    uint8_t* mask;
    uint64_t* acc_keys;         // optional: every accumulated key
    uint16_t* acc_cov;
    uint16_t* acc_edges;        // 8 per key
    unsigned long long* counts; // [0] n_keys, [1] n_solid, [2] digest, [3] raw edge total, [4] acc rows,
                                // [5] accumulator digest (when acc_digest)
    uint64_t cap_solid, cap_acc;
    int acc_digest;             // also sum the order-free digest of every accumulated key
};

// One isolate of a multi-isolate wave (fbk_k_batch.cu).
constexpr uint32_t BATCH_MAX_ISO = 256;
constexpr uint32_t BATCH_HLL_SAMPLE = 16;  // 1 in 16 keys (by hash) feeds the table-sizing HyperLogLog
constexpr uint32_t PASS1_HLL_SAMPLE = 16;  // the same sampling in the single-isolate pass 1
struct IsoDev {
    BankDev b;                      // r_begin = 0, r_end = the isolate's reads
    uint32_t* cnt;                  // exact u32 sketch, 4 rows of 2^log2w (or null with a ladder)
    uint32_t* lad;                  // t_solid-level gate ladder (or null with a sketch)
    uint32_t* hll12;                // p=12 registers of the keys (table sizing)
    uint32_t* bm;                   // solidity bitmap
    unsigned long long* n_records;  // [0] pass-2 records, [1] pass-1 and [2] pass-2 k-mer occurrences
    uint32_t log2w, t_solid, cap, _pad;
    TableDev t;
    BucketDev bk;
    uint32_t* status;               // ST_* bits of this isolate
};

struct Launch {
    int grid;     // <= 0: occupancy-derived persistent grid (resident blocks x SMs)
    int block;
    cudaStream_t stream;
    int sms;
};

// ---- build passes (fbk_k_pass.cu) -------------------------------------------
// Pass 1 sweep: for every k-mer of every kept read with len >= k and every row in
// [r0, r1), a column in [c0, c1) gets `mult` added to its u32 count.  hll12
// (optional, 4096 u32) collects a p=12 HyperLogLog of the keys (table sizing only).
cudaError_t launch_pass1_sweep(int nw, const Launch& L, const BankDev& b, uint32_t k, uint32_t* cnt, uint32_t log2w,
                               uint32_t r0, uint32_t r1, uint64_t c0, uint64_t c1, uint32_t mult, uint32_t* hll12);
// Solidity sweep: clears bitmap bit (first base of window) when, in any row of
// [r0, r1) whose column lies in [c0, c1), the window's capped count is below t_solid.
cudaError_t launch_solid_sweep(int nw, const Launch& L, const BankDev& b, uint32_t k, const uint32_t* cnt, uint32_t log2w,
                               uint32_t r0, uint32_t r1, uint64_t c0, uint64_t c1, uint32_t t_solid, uint32_t cap,
                               uint32_t* bm);
// Pass 2 sweep over the keys whose home slot lies in [s0, s1): each push adds
// w_edge to an edge counter (and w_cov to the cov counter when the table keeps one).
cudaError_t launch_pass2_sweep(int nw, const Launch& L, const BankDev& b, uint32_t k, const uint32_t* bm, int gate,
                               uint64_t s0, uint64_t s1, uint32_t w_edge, uint32_t w_cov, const TableDev& t,
                               uint32_t* status);
// Pass 2 in two phases: one scan emits the records of solid windows into slot-range
// buckets; then one launch per bucket upserts its records (the bucket's table range
// stays L2-resident while every lane works on its own record).
cudaError_t launch_emit(int nw, const Launch& L, const BankDev& b, uint32_t k, const uint32_t* bm, int gate, const TableDev& t,
                        const BucketDev& bk);
cudaError_t launch_upsert(int nw, const Launch& L, const BucketDev& bk, uint32_t bucket, uint32_t w_edge, uint32_t w_cov,
                          const TableDev& t, uint32_t* status, const RecordFilter& flt = RecordFilter{}, int queue = 0);
// Counters of cnt[0, n) at or above min, added to *out.
cudaError_t launch_count_at_least(const Launch& L, const uint32_t* cnt, uint64_t n, uint32_t min, unsigned long long* out);
cudaError_t launch_count_records(int nw, const Launch& L, const BucketDev& bk, uint32_t bucket, const RecordFilter& flt);
// every bucket in one persistent launch; *work (zeroed by the caller) hands out items
cudaError_t launch_upsert_all(int nw, const Launch& L, const BucketDev& bk, uint32_t w_edge, uint32_t w_cov, const TableDev& t,
                              uint32_t* status, unsigned long long* work,
                              int form = 1);
cudaError_t launch_convert(int nw, const Launch& L, const TableDev& t, uint32_t min_trans_cov, const ConvOut& o);
cudaError_t launch_clamp_counters(const Launch& L, uint32_t* cnt, uint64_t n);
cudaError_t launch_table_init(int nw, const Launch& L, const TableDev& t);

// ---- one isolate across ranks (fbk_shard.cu) -------------------------------------
// Rows are NW key words and two words of packed u16 edge counts; the owner of a key
// is splitmix64(fold(key)) mod world.
cudaError_t launch_owner_hist(int nw, const Launch& L, const uint64_t* keys, uint64_t n, uint32_t world,
                              unsigned long long* counts);
cudaError_t launch_owner_scatter(int nw, const Launch& L, const uint64_t* keys, const uint16_t* edges, uint64_t n, uint32_t world,
                                 unsigned long long* cursor, uint64_t* rows);
cudaError_t launch_rows_upsert(int nw, const Launch& L, const uint64_t* rows, uint64_t n, const TableDev& t, uint32_t* status);

// ---- threshold ladders (fbk_k_ladder.cu) -----------------------------------------
// The CMS gate of pass 2 without counts: t levels x 4 rows x 2^log2w bits, level j of
// (row, col) set once the count reached j + 1.  1 <= t <= LADDER_MAX_LEVELS.
constexpr uint32_t LADDER_MAX_LEVELS = 8;
// ilp: windows per lane per step (1 or 2).
cudaError_t launch_ladder_pass1(int nw, const Launch& L, const BankDev& b, uint32_t k, uint32_t* lad, uint32_t log2w, uint32_t t,
                                uint32_t* hll12, int ilp);
cudaError_t launch_ladder_solid(int nw, const Launch& L, const BankDev& b, uint32_t k, const uint32_t* lad, uint32_t log2w,
                                uint32_t t, uint32_t* bm);
// Record emit of pass 2 with the ladder gate evaluated inline (no solidity bitmap).
// lookahead 1: the gate of the next chunk is resolved before each chunk is emitted;
// 2: the loads of the chunk after it are in flight while a chunk is emitted.
cudaError_t launch_emit_ladder(int nw, const Launch& L, const BankDev& b, uint32_t k, const uint32_t* lad, uint32_t log2w,
                               uint32_t t_solid, const TableDev& t, const BucketDev& bk, int lookahead);

// One lane per read, k-mers rolled base by base, each warp's run of 32 reads staged in
// shared memory (fbk_k_roll.cu); the same results as launch_ladder_pass1 and
// launch_emit_ladder.  Blocks of 256 threads.
cudaError_t launch_ladder_pass1_roll(int nw, const Launch& L, const BankDev& b, uint32_t k, uint32_t* lad, uint32_t log2w,
                                     uint32_t t, uint32_t* hll12, int windows_per_step);
cudaError_t launch_emit_roll(int nw, const Launch& L, const BankDev& b, uint32_t k, const uint32_t* lad, uint32_t log2w,
                             uint32_t t_solid, const TableDev& t, const BucketDev& bk,
                             bool two_blocks = false);

// ---- multi-isolate waves (fbk_k_batch.cu) ----------------------------------------
// read_base: n_iso + 1 global read indices (isolate i owns [read_base[i], read_base[i+1])).
cudaError_t launch_batch_pass1(int nw, const Launch& L, const IsoDev* iso, const unsigned long long* read_base, uint32_t n_iso,
                               uint32_t k, uint32_t r0, uint32_t r1, int do_hll);
cudaError_t launch_batch_solid(int nw, const Launch& L, const IsoDev* iso, const unsigned long long* read_base, uint32_t n_iso,
                               uint32_t k, uint32_t r0, uint32_t r1);
cudaError_t launch_batch_count(const Launch& L, const IsoDev* iso, const unsigned long long* read_base, uint32_t n_iso, uint32_t k);
// Ladder form of pass 1 (every isolate's gate is a t_solid-level ladder): one sweep.
cudaError_t launch_batch_lpass1(int nw, const Launch& L, const IsoDev* iso, const unsigned long long* read_base, uint32_t n_iso,
                                uint32_t k);

cudaError_t launch_batch_emit(int nw, const Launch& L, const IsoDev* iso, const unsigned long long* read_base, uint32_t n_iso,
                              uint32_t k, uint32_t stripes);


// ---- estimator and utilities (fbk_k_est.cu) -----------------------------------
cudaError_t launch_est_firstpos(const Launch& L, const BankDev& b, const uint64_t* kbase, uint32_t k, uint32_t* first,
                                uint32_t log2w);
cudaError_t launch_est_hll(const Launch& L, const BankDev& b, const uint64_t* kbase, uint32_t k, const uint32_t* first,
                           uint32_t log2w, uint32_t p, uint32_t n_segs, uint32_t* regs_total, uint32_t* regs_solid);
cudaError_t launch_est_prefix(const Launch& L, uint32_t* regs, uint32_t p, uint32_t n_segs);
cudaError_t launch_est_sums(const Launch& L, const uint32_t* regs_total, const uint32_t* regs_solid, uint32_t p,
                            uint32_t n_segs, double* sums, unsigned long long* zeros);
cudaError_t launch_hll_add(const Launch& L, uint32_t* regs, uint32_t p, const uint64_t* hashes, uint64_t n, int mix);
cudaError_t launch_hll_merge(const Launch& L, uint32_t* dst, const uint32_t* src, uint64_t n);
cudaError_t launch_subsample_mask(const Launch& L, uint64_t n_pairs, double factor, uint64_t seed, uint64_t* bits);
// Count-Min Sketch of exact u32 counts (4 rows of 2^log2w); readers cap at `cap`.
cudaError_t launch_cms_keys(const Launch& L, uint32_t* cnt, uint32_t log2w, uint32_t cap, const uint64_t* keys, uint64_t n,
                            uint32_t* est_out, int add);
cudaError_t launch_cms_merge(const Launch& L, uint32_t* dst, const uint32_t* src, uint64_t n);
// Reference byte layout: counter_bits 4 = nibbles (byte c>>1, high nibble for odd c),
// 16 = little-endian u16; values min(cap, count).
cudaError_t launch_cms_export(int cb, const Launch& L, const uint32_t* cnt, uint64_t n, uint8_t* out);
cudaError_t launch_cms_import(int cb, const Launch& L, uint32_t* cnt, uint64_t n, const uint8_t* in);
cudaError_t launch_nthash_arena(const Launch& L, const BankDev& b, const uint64_t* kbase, uint32_t k, uint64_t* out);
cudaError_t launch_canon_arena(int nw, const Launch& L, const BankDev& b, const uint64_t* kbase, uint32_t k,
                               uint64_t* out_words, uint8_t* out_rc);
cudaError_t launch_add_u64(const Launch& L, uint64_t* p, uint64_t n, uint64_t add);

}  // namespace fbk
