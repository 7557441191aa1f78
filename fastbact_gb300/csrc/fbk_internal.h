// fbk_internal.h — host-side internals shared by the C-ABI translation units.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/fbk.h"
#include "fbk_kernels.cuh"

namespace fbk {

// First-fit device memory pool carved from one cudaMalloc (256-byte granules).
class DevicePool {
  public:
    bool init(uint64_t bytes, std::string& err);
    void release();
    void* alloc(uint64_t bytes);
    void free(void* p);
    uint64_t used() const { return used_bytes_; }
    uint64_t size() const { return size_; }
    uint64_t largest_free() const;
    uint64_t free_bytes() const { return size_ - used_bytes_; }
    bool active() const { return base_ != nullptr; }
    ~DevicePool() { release(); }

  private:
    char* base_ = nullptr;
    uint64_t size_ = 0, used_bytes_ = 0;
    std::map<uint64_t, uint64_t> free_;  // offset -> size
    std::map<uint64_t, uint64_t> live_;  // offset -> size
    mutable std::mutex mu_;
};

struct TimedLaunch {
    std::string name;
    cudaEvent_t a, b;
};

}  // namespace fbk

struct fbk_ctx {
    int device = 0;
    int num_sms = 0;
    cudaStream_t stream = nullptr;
    cudaStream_t copy_stream = nullptr;      // asynchronous uploads and exports (created on first use)
    std::shared_ptr<fbk::DevicePool> pool;  // shared by contexts forked from this one
    uint32_t* d_status = nullptr;            // device status bits (4 words)
    unsigned long long* d_counts = nullptr;  // conversion counters (4)
    void* h_pinned = nullptr;                // 64 KiB pinned host scratch
    void* h_stage[2] = {};                   // pinned staging slots for pageable copies (lazy)
    cudaEvent_t stage_ev[2] = {};            // last DMA that used each slot
    std::string err;
    bool timing = false;
    std::vector<fbk::TimedLaunch> pending;
    std::vector<cudaEvent_t> free_events;
    std::map<std::string, std::pair<double, uint64_t>> timed;
    uint64_t launches = 0;
    cudaEvent_t markers[16] = {};
    // launch shapes (block size; grid 0 = 4 blocks per SM)
    int block_pass1 = 256, grid_pass1 = 0;
    int block_pass2 = 256, grid_pass2 = 0;
    int block_emit = 128;  // flat and read-by-read record emits (128 measured 2-5% faster than 256); the rolled emit runs 256
    int block_misc = 256;
    // sweep sizing: bytes of sketch per pass-1 / solidity sweep, and bytes of table
    // per pass-2 slot range (the hot part of a range must stay L2-resident)
    uint64_t sweep_bytes = 64ull << 20;
    uint64_t bucket_bytes = 256ull << 20;  // table bytes per pass-2 record bucket
    uint32_t stripes = 64;                // append stripes per bucket
    double load_factor = 0.62;            // solid table keys / slots when sized from the estimate
    int pass2_mode = 1;                   // 1 = record buckets, 0 = direct sweep
    double record_factor = 1.25;          // bucket capacity / expected records per stripe
    int sketch_mode = 1;                  // 1: a build that does not return its sketch keeps only the gate ladder
    // Ladder pass 1: 1 or 2 windows per lane per step, 3 pipelined over chunks, 4 one lane
    // per read with rolled k-mers, 5 the same with two windows per lane per step; 0
    // (default) picks by key width: 5 for 128- and 256-bit keys, 1 for 64-bit keys.
    // Measured per 100x pass (forms 1 / 4 / 5): k = 21 6.62 / 7.47 / 7.13 ms, k = 33
    // 7.30 / 7.37 / 6.68, k = 55 5.71 / 6.26 / 5.59, k = 77 5.98 / 5.37 / 4.74.
    int ladder_ilp = 0;
    // Record emit: gate loads 1 or 2 chunks ahead read by read; 3 = 2 ahead over a flattened
    // window stream; 4 = one lane per read with rolled k-mers (5: the same at two blocks
    // per SM for every key width).  0 (default) = 4 (per 100x pass, flat -> rolled: k = 21
    // 8.57 -> 7.02 ms, k = 33 9.04 -> 8.16, k = 55 7.38 -> 6.77, k = 77 7.34 -> 5.74 with
    // two blocks per SM for 256-bit keys).
    int emit_lookahead = 0;
    // Filtered upserts: 1 (default) queues the filter's survivors per warp so that the
    // probes run on full warps, 2 the same at six blocks per SM, 0 tests the filter
    // inline.  Measured per 100x pass (0 / 1 / 2): k = 55 7.44 / 6.67 / 7.93 ms, k = 77
    // 10.88 / 7.70 / 9.10.
    int upsert_queue = 1;
    // Filtered passes: 1 (default) sizes the table from the keys that pass the filter in
    // the first bucket, at filter_load keys per slot (plus 30% headroom), 0 from the
    // distinct k-mers of pass 1 at load_factor.  Measured per 100x step (ms): distinct
    // 97.0; filter_load 0.12 94.1, 0.2 93.3, 0.3 92.8, 0.62 99.0 (probe runs grow long
    // where a bucket holds more survivors than bucket 0 predicted).
    int filter_sizing = 1;
    double filter_load = 0.3;
    int batch_pass1 = 0;                  // batches with a ladder gate: 0 autotuned, 1 one multi-isolate launch, 2 a launch per isolate
    // Unfiltered passes: 1 upserts every bucket in one persistent launch, 2 (default) the
    // same with every lane's probe advanced a slot per step (64/128-bit keys; per 100x
    // pass k = 21 5.60 -> 5.59 ms, k = 33 6.70 -> 6.58), 0 one launch per bucket
    int upsert_all = 2;
    // keys with fewer records than min_trans_cov stay out of the table: 0 never, 2 always,
    // 1 where it pays (256-bit keys, and passes whose distinct k-mers exceed a fifth of
    // their windows; acc_filter_on)
    int acc_filter = 1;
    bool capturing = false;               // launches are being captured into a CUDA graph
};

struct fbk_bank {
    fbk_ctx* ctx = nullptr;
    uint64_t* data = nullptr;
    uint64_t* off = nullptr;
    uint32_t* len = nullptr;
    uint32_t* pair_idx = nullptr;
    uint64_t n_reads = 0, n_words = 0, n_bases = 0, n_pairs = 0;
    uint32_t max_len = 0;
    std::vector<uint64_t> chunk_starts;  // read-range boundaries (see bank_upload_impl)
    std::vector<uint64_t> arena_reads;   // reads of each uploaded arena, in bank order
    uint64_t max_chunk = 0;              // most bases in one range
    uint64_t max_chunk_bases() const { return max_chunk; }
    std::vector<uint64_t> len_hist;      // read-length histogram (last bin: all longer reads)
    uint64_t long_bases = 0;             // bases of reads in the last bin
    cudaEvent_t ready = nullptr;         // an asynchronous upload's copies (null: uploaded synchronously)
    // upper bound of the windows of length k in reads with len >= min_len
    uint64_t windows(uint32_t k, uint32_t min_len) const {
        uint64_t w = 0;
        const uint64_t last = len_hist.empty() ? 0 : len_hist.size() - 1;
        for (uint64_t L = std::max<uint64_t>(min_len, k); L < last; ++L) w += len_hist[L] * (L - k + 1);
        return w + long_bases;
    }
};

struct fbk_cms {
    fbk_ctx* ctx = nullptr;
    uint32_t* cnt = nullptr;    // exact u32 count per (row, column), 4 rows of 2^log2w; <= 65535 between calls
    uint32_t* hll12 = nullptr;  // p=12 registers of the keys added by bank passes (table sizing)
    uint32_t log2w = 0;
    uint32_t cbits = 4;         // reference layout and cap: 4 -> nibbles / 15, 16 -> u16 / 65535
    uint64_t n = 0;             // 4 << log2w counters
    uint32_t cap() const { return cbits == 4 ? 15u : 0xFFFFu; }
};

struct fbk_hll {
    fbk_ctx* ctx = nullptr;
    uint32_t* regs = nullptr;
    uint32_t p = 14;
};

struct fbk_table {
    fbk_ctx* ctx = nullptr;
    uint32_t nw = 1, k = 0, min_trans_cov = 3;
    uint64_t cap = 0;
    uint64_t* keys = nullptr;
    uint64_t* tags = nullptr;  // == keys when the tags live in word 0 of the keys
    uint32_t* cnt = nullptr;
    uint32_t* cov = nullptr;
    // converted SolidKmerNode rows
    uint64_t* out_keys = nullptr;
    uint16_t* out_cov = nullptr;
    uint8_t* out_mask = nullptr;
    uint64_t out_cap = 0;
    uint64_t n_keys = 0, n_solid = 0, digest = 0, pushes = 0;
    uint64_t skipped_pushes = 0;  // pushes of records the record filter kept out of the table
    bool filtered = false;        // the accumulator holds only keys that may become solid
    cudaEvent_t converted = nullptr, exported = nullptr;  // an asynchronous export's order and completion
};

namespace fbk {

// The pass-1 and emit forms a context's tuning selects for keys of nw words.
inline int ladder_form(const fbk_ctx* ctx, int nw) { return ctx->ladder_ilp ? ctx->ladder_ilp : (nw == 1 ? 1 : 5); }
inline int emit_form(const fbk_ctx* ctx, int nw) { return ctx->emit_lookahead ? ctx->emit_lookahead : 4; }

fbk_status set_err(fbk_ctx* ctx, fbk_status st, const std::string& msg);
// Orders the context's stream after an asynchronous upload of b (no-op otherwise).
cudaError_t bank_wait(fbk_ctx* ctx, const fbk_bank* b);
fbk_status cuda_err(fbk_ctx* ctx, cudaError_t e, const char* what);
void* dev_alloc(fbk_ctx* ctx, uint64_t bytes);
void dev_free(fbk_ctx* ctx, void* p);
Launch launch_cfg(fbk_ctx* ctx, int block, int grid);
// grid <= 0 is left to the launcher: resident blocks per SM x SMs
Launch launch_cfg_persistent(fbk_ctx* ctx, int block, int grid);
// Brackets a launch with timing events when timing is on.
void time_begin(fbk_ctx* ctx, const char* name, TimedLaunch& t);
void time_end(fbk_ctx* ctx, TimedLaunch& t);
fbk_status ctx_check_status(fbk_ctx* ctx, uint32_t* bits);

// One host pass over the sequences of a set of arenas: bounds check, totals, the
// read-length histogram and the sums of fixed read blocks (for the chunk walk).
// Blocks of BLOCK reads are scanned by up to 16 threads; the results do not depend on
// the thread count.
struct ArenaScan {
    static constexpr uint64_t BLOCK = 1 << 16;
    static constexpr uint64_t BINS = 1 << 16;
    uint64_t n_reads = 0, n_bases = 0, max_pair = 0;
    uint32_t max_len = 0;
    bool bad = false;
    std::vector<uint64_t> hist, block_bases;  // hist over lengths < BINS - 1 (capped index)
    uint64_t long_bases = 0;                  // bases of reads of length >= BINS - 1
};

void scan_arenas(const fbk_arena_view* arenas, int n_arenas, ArenaScan& sc);

// Host<->device copies on the context's stream.  Page-locked host memory and small
// copies go straight to the DMA engines; larger pageable buffers move through two
// pinned staging slots, the host side copied by the worker pool while the other
// slot's DMA runs (a GPU reading pageable memory that it has not mapped recently
// runs far below the copy engines' rate).  copy_h2d returns with the last DMA in
// flight (src may be reused at once); copy_d2h returns when dst holds the data.
cudaError_t copy_h2d(fbk_ctx* ctx, void* dst, const void* src, size_t bytes);
cudaError_t copy_d2h(fbk_ctx* ctx, void* dst, const void* src, size_t bytes);

// Upload of a packed arena set into a device bank (used by the estimator for its
// sample and by prior-contig handling).
// chunk_bases: read ranges are cut so that each holds fewer bases than this.
fbk_status bank_upload_impl(fbk_ctx* ctx, const fbk_arena_view* arenas, int n_arenas, fbk_bank** out,
                            uint64_t chunk_bases = 1ull << 30, bool async = false);
BankDev bank_view(const fbk_bank* b, uint64_t r_begin, uint64_t r_end, const uint64_t* keep_bits);

// 256-bit keys of k <= 96 have a zero most significant word, which then holds the
// slot's tag (no separate tag array).
inline bool tag_in_key(uint32_t nw, uint32_t k) { return nw == 4 && k <= 96; }

// Whether the record filter applies under tuning acc_filter (0 never, 2 always, 1
// auto).  Counting costs about one L2 atomic per record; it pays when many keys are
// seen once or twice: for 256-bit keys, and when the distinct k-mers of pass 1 exceed
// a fifth of the records (measured at 100x: k = 55, 24% distinct, 12.7 -> 10.1 ms; k = 33,
// 14%, 10.6 -> 11.8 ms; k = 21, 8%, 8.5 -> 12.2 ms).
inline bool acc_filter_on(int mode, int nw, uint64_t distinct, uint64_t records) {
    return mode == 2 || (mode == 1 && (nw == 4 || distinct * 5 > records));
}

// Single-isolate pieces reused by the multi-isolate host code (fbk_api.cu).
int key_words(uint32_t key_bits);     // 64 -> 1, 128 -> 2, 256 -> 4, else 0
uint32_t key_k_max(uint32_t key_bits);
fbk_status keep_bits_for(fbk_ctx* ctx, const fbk_bank* b, const fbk_subsample* ss, uint64_t** bits_out);
TableDev tbl_dev(const fbk_table* t);
fbk_status tbl_alloc(fbk_table* t, uint64_t cap, bool with_cov);
void tbl_free_storage(fbk_table* t);
void tbl_free_out(fbk_table* t);
fbk_status tbl_convert(fbk_table* t);  // conversion, growing the output when it was too small
fbk_status solid_build(fbk_ctx* ctx, const fbk_bank* b, const fbk_cms* cms, const fbk_build_params* p, const uint64_t* keep_bits,
                       uint64_t distinct_hint, fbk_table** out);
// The same with the pass-1 gate as a t_solid-level ladder (fbk_k_ladder.cu).
fbk_status solid_build_ladder(fbk_ctx* ctx, const fbk_bank* b, uint32_t* ladder, uint32_t log2w, const fbk_build_params* p,
                              const uint64_t* keep_bits, uint64_t distinct_hint, fbk_table** out);

// host f64 HyperLogLog::estimate from the register sum and zero count (sketch.rs:83-114)
double hll_estimate_from_sum(double sum, uint64_t zeros, uint32_t p);
uint64_t f64_to_u64_sat(double x);

}  // namespace fbk

#define CK(ctx, call)                                               \
    do {                                                            \
        cudaError_t e_ = (call);                                    \
        if (e_ != cudaSuccess) return fbk::cuda_err(ctx, e_, #call); \
    } while (0)

#define TIMED(ctx, name, call)                                      \
    do {                                                            \
        fbk::TimedLaunch tl_;                                       \
        fbk::time_begin(ctx, name, tl_);                            \
        cudaError_t e_ = (call);                                    \
        fbk::time_end(ctx, tl_);                                    \
        if (e_ != cudaSuccess) return fbk::cuda_err(ctx, e_, name); \
    } while (0)
