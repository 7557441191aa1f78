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
// a k <= 31 key uses 62 bits).  NW > 1: tags[] claims slots (0 empty, fingerprint,
// fingerprint|READY once the key words are published) and keys[] holds NW words per
// slot.  cnt[] holds 8 edge counters (u32) per slot, 32-byte aligned.
struct TableDev {
    uint64_t* keys;
    uint64_t* tags;
    uint32_t* cnt;
    uint32_t* cov;       // separate cov counters, only when prior contigs are used
    uint64_t mask;       // capacity - 1
    uint32_t max_probe;
    uint32_t spin_limit;
};

// Output of the SolidKmerNode conversion.
struct ConvOut {
    uint64_t* keys;             // n_solid * NW words
    uint16_t* cov;
    uint8_t* mask;
    uint64_t* acc_keys;         // optional: every accumulated key
    uint16_t* acc_cov;
    uint16_t* acc_edges;        // 8 per key
    unsigned long long* counts; // [0] n_keys, [1] n_solid, [2] digest, [3] raw edge total, [4] acc rows
    uint64_t cap_solid, cap_acc;
};

struct Launch {
    int grid;
    int block;
    cudaStream_t stream;
};

// ---- build passes (fbk_k_pass.cu) -------------------------------------------
// Pass 1: every k-mer of every kept read with len >= k adds `mult` (saturating) to
// its four CMS counters.  hll12 (optional, 4096 u32) collects a p=12 HyperLogLog
// of the keys, used only to size the solid table.
cudaError_t launch_pass1(int nw, int cb, const Launch& L, const BankDev& b, uint32_t k, uint32_t* cms, uint32_t log2w,
                         uint32_t mult, uint32_t* hll12);
// Pass 2: transitions between adjacent k-mers; with gate != 0 both ends must have
// CMS estimate >= t_solid.  Each push adds w_edge to an edge counter (and w_cov to
// the cov counter when the table keeps one).
cudaError_t launch_pass2(int nw, int cb, const Launch& L, const BankDev& b, uint32_t k, const uint32_t* cms, uint32_t log2w,
                         uint32_t t_solid, int gate, uint32_t w_edge, uint32_t w_cov, const TableDev& t, uint32_t* status);
cudaError_t launch_convert(int nw, const Launch& L, const TableDev& t, uint32_t min_trans_cov, const ConvOut& o);
cudaError_t launch_clamp_counters(const Launch& L, uint32_t* cnt, uint64_t n);
cudaError_t launch_table_init(int nw, const Launch& L, const TableDev& t);

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
cudaError_t launch_cms_keys(int cb, const Launch& L, uint32_t* cms, uint32_t log2w, const uint64_t* keys, uint64_t n,
                            uint32_t* est_out, int add);
cudaError_t launch_cms_merge(int cb, const Launch& L, uint32_t* dst, const uint32_t* src, uint64_t n_words);
cudaError_t launch_nthash_arena(const Launch& L, const BankDev& b, const uint64_t* kbase, uint32_t k, uint64_t* out);
cudaError_t launch_canon_arena(int nw, const Launch& L, const BankDev& b, const uint64_t* kbase, uint32_t k,
                               uint64_t* out_words, uint8_t* out_rc);
cudaError_t launch_add_u64(const Launch& L, uint64_t* p, uint64_t n, uint64_t add);

}  // namespace fbk
