// fbk_estimator.cu — estimate_genome (src/ingest/estimator.rs:286-440): the
// sample loop runs on the device (fbk_k_est.cu), the checkpoint decisions and the
// f64 post-math run here on the host with the same operation order as the Rust code
// (compiled with -ffp-contract=off; log/exp come from the platform libm, as Rust's do).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "fbk_device.cuh"
#include "fbk_internal.h"
#include "host/fbk_host.h"

using namespace fbk;

namespace {

// compute_dynamic_kmers — estimator.rs:104-161 (target_max_k < 0 = None)
std::vector<uint64_t> dynamic_kmers(uint64_t median_len, int64_t target_max_k) {
    std::vector<uint64_t> out;
    const uint64_t min_k = median_len < 75 ? 21 : 31;
    const uint64_t effective_len = (median_len * 16) / 10;
    const uint64_t auto_max = f64_to_u64_sat((double)effective_len * 0.85);
    uint64_t max_k = target_max_k >= 0 ? (uint64_t)target_max_k : auto_max;
    max_k = std::min<uint64_t>(std::max(max_k, min_k), 127);
    if (max_k % 2 == 0) max_k -= 1;
    if (max_k <= min_k) return {min_k};
    if (median_len >= 100) {
        const uint64_t mid_k = 63;
        if (max_k > mid_k + 10) return {min_k, mid_k, max_k};
        if (max_k > min_k) return {min_k, max_k};
        return {min_k};
    }
    uint64_t step = (max_k - min_k) / 2;
    if (step % 2 == 1) step += 1;
    if (step < 6) step = 6;
    for (uint64_t k = min_k; k <= max_k; k += step) out.push_back(k);
    const uint64_t last = out.back();
    if (last != max_k && max_k > last) {
        if (max_k - last >= 10) out.push_back(max_k);
        else out.back() = max_k;
    }
    out.erase(std::unique(out.begin(), out.end()), out.end());
    return out;
}

struct Buffers {
    fbk_ctx* ctx;
    std::vector<void*> ptrs;
    explicit Buffers(fbk_ctx* c) : ctx(c) {}
    void* get(uint64_t bytes) {
        void* p = dev_alloc(ctx, bytes);
        if (p) ptrs.push_back(p);
        return p;
    }
    ~Buffers() {
        cudaStreamSynchronize(ctx->stream);
        for (void* p : ptrs) dev_free(ctx, p);
    }
};

}  // namespace

#define CKE(call)                                               \
    do {                                                        \
        cudaError_t e_ = (call);                                \
        if (e_ != cudaSuccess) return cuda_err(ctx, e_, #call); \
    } while (0)

#define TIMEDE(name, call)                                     \
    do {                                                       \
        TimedLaunch tl_;                                       \
        time_begin(ctx, name, tl_);                            \
        cudaError_t e_ = (call);                               \
        time_end(ctx, tl_);                                    \
        if (e_ != cudaSuccess) return cuda_err(ctx, e_, name); \
    } while (0)

extern "C" {

FBK_API void fbk_estimator_defaults(fbk_estimator_params* p) {
    if (!p) return;
    memset(p, 0, sizeof(*p));
    p->k = 21;
    p->cms_log2_width = 23;
    p->hll_p = 14;
    p->sample_cap = 150000;
    p->max_pairs = 250000;  // src/main.rs:65
    p->target_cov = 0.0;
}

FBK_API int fbk_compute_dynamic_kmers(uint64_t median_len, int64_t target_max_k, uint64_t* out, int cap) {
    std::vector<uint64_t> v = dynamic_kmers(median_len, target_max_k);
    for (int i = 0; out && i < (int)v.size() && i < cap; ++i) out[i] = v[i];
    return (int)v.size();
}

}  // extern "C"

namespace {

fbk_status check_est_params(fbk_ctx* ctx, const fbk_estimator_params* prm) {
    const uint32_t k = prm->k, p = prm->hll_p, log2w = prm->cms_log2_width;
    if (k == 0 || p < 4 || p > 18 || log2w < 3 || log2w > 30) return set_err(ctx, FBK_ERR_INVALID, "estimator parameters out of range");
    return FBK_OK;
}

// Occurrence bookkeeping of a sample of n_use pairs (reads R1,R2 interleaved):
// kbase[r] = index of read r's first k-mer, m_pair[P] = k-mers of the first P pairs.
struct EstPlan {
    std::vector<uint64_t> kbase, m_pair;
    uint32_t n_segs = 1;
};

fbk_status est_plan(fbk_ctx* ctx, const uint32_t* lengths, uint64_t n_use, uint32_t k, EstPlan& pl) {
    const uint64_t n_reads = 2 * n_use;
    pl.kbase.assign(n_reads + 1, 0);
    pl.m_pair.assign(n_use + 1, 0);
    for (uint64_t r = 0; r < n_reads; ++r) {
        const uint32_t L = lengths[r];
        pl.kbase[r + 1] = pl.kbase[r] + (L >= k ? L - k + 1 : 0);
        if (r & 1) pl.m_pair[(r >> 1) + 1] = pl.kbase[r + 1];
    }
    // Checkpoints after pair counts 6000, 8000, ... (estimator.rs:366-375); segment j
    // ends at 6000 + 2000 j.
    pl.n_segs = n_use <= 6000 ? 1u : (uint32_t)(1 + (n_use - 6000 + 1999) / 2000);
    if (pl.kbase.back() >= 0xFFFFFFFFULL) return set_err(ctx, FBK_ERR_INVALID, "estimator sample holds 2^32 or more k-mers");
    return FBK_OK;
}

uint64_t est_n_use(const fbk_count_stats* stats, const fbk_estimator_params* prm, uint64_t n_pairs) {
    const uint64_t sample_target = std::min(std::min(prm->max_pairs, prm->sample_cap), stats->exact_read_pairs);
    return std::min(sample_target, n_pairs);  // a reader that runs dry ends the loop (estimator.rs:377)
}

// The early stop and the post-math (estimator.rs:366-439) from the HLL sums of every
// checkpoint segment: sums[which * n_segs + j], which 0 = total, 1 = solid.  Returns the
// segment whose registers are final.
uint32_t est_decide(const double* sums, const unsigned long long* zeros, const EstPlan& pl, uint64_t n_use,
                    const fbk_count_stats* stats, const fbk_estimator_params* prm, fbk_genome_estimate* out) {
    const uint32_t k = prm->k, p = prm->hll_p, n_segs = pl.n_segs;
    auto est = [&](int which, uint32_t seg) {
        const uint32_t i = which * n_segs + seg;
        return hll_estimate_from_sum(sums[i], zeros[i], p);
    };
    uint32_t final_seg = n_segs - 1;
    uint64_t pairs_done = n_use;
    for (uint32_t j = 0; j < n_segs; ++j) {
        const uint64_t P = 6000 + 2000ULL * j;
        if (P > n_use) break;
        const uint64_t u1 = f64_to_u64_sat(std::round(est(0, j)));
        const uint64_t u2 = f64_to_u64_sat(std::round(est(1, j)));
        const uint64_t e1 = u1 > u2 ? u1 - u2 : 0;
        const uint64_t m_tr = pl.m_pair[P] > e1 ? pl.m_pair[P] - e1 : 0;
        const double lam = u2 > 0 ? (double)m_tr / (double)u2 : 0.0;
        if (lam >= 15.0) {
            final_seg = j;
            pairs_done = P;
            break;
        }
    }
    const uint64_t m_sample = pl.m_pair[pairs_done];

    // post-math — estimator.rs:386-439
    const uint64_t u_ge_1 = f64_to_u64_sat(std::round(est(0, final_seg)));
    const uint64_t u_ge_2 = f64_to_u64_sat(std::round(est(1, final_seg)));
    const uint64_t e_1 = u_ge_1 > u_ge_2 ? u_ge_1 - u_ge_2 : 0;
    const uint64_t m_true = m_sample > e_1 ? m_sample - e_1 : 0;
    const double lambda_s = u_ge_2 > 0 ? (double)m_true / (double)u_ge_2 : 0.0;
    const double p_ge_2 = 1.0 - (1.0 + lambda_s) * std::exp(-lambda_s);
    uint64_t est_g = p_ge_2 > 0.05 ? f64_to_u64_sat(std::round((double)u_ge_2 / p_ge_2)) : std::max<uint64_t>(u_ge_2, 10000);
    if (est_g < 10000) est_g = 10000;
    const double estimated_cov = (double)stats->total_bases / (double)est_g;
    const double d_k = estimated_cov * ((stats->mean_read_len - (double)k + 1.0) / stats->mean_read_len);
    const double solid_ratio = u_ge_1 > 0 ? (double)u_ge_2 / (double)u_ge_1 : 0.0;
    int conf;
    if (d_k < 5.0 || solid_ratio < 0.05 || u_ge_2 < 1000) conf = 2;
    else if (d_k < 20.0 || solid_ratio < 0.15) conf = 1;
    else conf = 0;
    double ssf = 1.0;
    if (prm->target_cov > 0.0 && estimated_cov > 1.5 * prm->target_cov)
        ssf = std::min(std::max(prm->target_cov / estimated_cov, 0.01), 1.0);
    std::vector<uint64_t> ks = dynamic_kmers(stats->median_read_len, -1);

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
    out->pairs_sampled = pairs_done;
    out->m_sample = m_sample;
    return final_seg;
}

// Sample loop on a device-resident sample bank whose first 2*n_use reads are the
// pairs, R1 then R2; lengths is the host copy of those reads' lengths.
fbk_status estimate_impl(fbk_ctx* ctx, const fbk_bank* bank, const uint32_t* lengths, uint64_t n_use,
                                const fbk_count_stats* stats, const fbk_estimator_params* prm, fbk_genome_estimate* out,
                                uint8_t* regs_total, uint8_t* regs_solid) {
    const uint32_t k = prm->k, p = prm->hll_p, log2w = prm->cms_log2_width;
    const uint64_t n_reads = 2 * n_use;
    EstPlan pl;
    fbk_status st = est_plan(ctx, lengths, n_use, k, pl);
    if (st) return st;
    const uint64_t m = 1ULL << p;
    const uint32_t n_segs = pl.n_segs;
    Buffers buf(ctx);
    uint64_t* d_kbase = (uint64_t*)buf.get((n_reads + 1) * 8);
    uint32_t* first = (uint32_t*)buf.get((4ULL << log2w) * 4);
    uint32_t* regs_t = (uint32_t*)buf.get((uint64_t)n_segs * m * 4);
    uint32_t* regs_s = (uint32_t*)buf.get((uint64_t)n_segs * m * 4);
    double* sums = (double*)buf.get(2 * n_segs * sizeof(double));
    unsigned long long* zeros = (unsigned long long*)buf.get(2 * n_segs * sizeof(unsigned long long));
    if (!d_kbase || !first || !regs_t || !regs_s || !sums || !zeros) return set_err(ctx, FBK_ERR_OOM, "estimator buffers");
    CKE(cudaMemcpyAsync(d_kbase, pl.kbase.data(), (n_reads + 1) * 8, cudaMemcpyHostToDevice, ctx->stream));
    CKE(cudaMemsetAsync(first, 0xFF, (4ULL << log2w) * 4, ctx->stream));
    CKE(cudaMemsetAsync(regs_t, 0, (uint64_t)n_segs * m * 4, ctx->stream));
    CKE(cudaMemsetAsync(regs_s, 0, (uint64_t)n_segs * m * 4, ctx->stream));

    const BankDev bv = bank_view(bank, 0, n_reads, nullptr);
    Launch L = launch_cfg(ctx, 256, 0);
    TIMEDE("est_firstpos", launch_est_firstpos(L, bv, d_kbase, k, first, log2w));
    TIMEDE("est_hll", launch_est_hll(L, bv, d_kbase, k, first, log2w, p, n_segs, regs_t, regs_s));
    TIMEDE("est_prefix", launch_est_prefix(L, regs_t, p, n_segs));
    TIMEDE("est_prefix", launch_est_prefix(L, regs_s, p, n_segs));
    TIMEDE("est_sums", launch_est_sums(L, regs_t, regs_s, p, n_segs, sums, zeros));
    std::vector<double> h_sums(2 * n_segs);
    std::vector<unsigned long long> h_zeros(2 * n_segs);
    CKE(cudaMemcpyAsync(h_sums.data(), sums, 2 * n_segs * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    CKE(cudaMemcpyAsync(h_zeros.data(), zeros, 2 * n_segs * sizeof(unsigned long long), cudaMemcpyDeviceToHost, ctx->stream));
    CKE(cudaStreamSynchronize(ctx->stream));
    const uint32_t final_seg = est_decide(h_sums.data(), h_zeros.data(), pl, n_use, stats, prm, out);

    if (regs_total || regs_solid) {
        std::vector<uint32_t> r(m);
        for (int which = 0; which < 2; ++which) {
            uint8_t* dst = which == 0 ? regs_total : regs_solid;
            if (!dst) continue;
            const uint32_t* src = (which == 0 ? regs_t : regs_s) + (uint64_t)final_seg * m;
            CKE(cudaMemcpyAsync(r.data(), src, m * 4, cudaMemcpyDeviceToHost, ctx->stream));
            CKE(cudaStreamSynchronize(ctx->stream));
            for (uint64_t i = 0; i < m; ++i) dst[i] = (uint8_t)r[i];
        }
    }
    return FBK_OK;
}

// One rank's part of the sharded sample loop: pairs [pair_begin, pair_end) of a
// resident sample of n_use pairs, with global occurrence indices.  Stage 1 (first ==
// nullptr) writes the rank's first-touch array to first_out; stage 2 reads the merged
// array and writes the rank's per-segment register maxima (u8, total then solid).
fbk_status est_shard_stage(fbk_ctx* ctx, const fbk_bank* bank, const uint32_t* lengths, uint64_t n_use,
                                  uint64_t pair_begin, uint64_t pair_end, const fbk_estimator_params* prm,
                                  const uint32_t* first_in, uint32_t* first_out, uint8_t* regs_out) {
    if (!ctx || !bank || !lengths || !prm) return FBK_ERR_INVALID;
    fbk_status st = check_est_params(ctx, prm);
    if (st) return st;
    if (pair_begin > pair_end || pair_end > n_use) return set_err(ctx, FBK_ERR_INVALID, "pair range outside the sample");
    if (bank->n_reads < 2 * n_use) return set_err(ctx, FBK_ERR_INVALID, "sample holds fewer than 2*n_use reads");
    CKE(cudaSetDevice(ctx->device));
    CKE(bank_wait(ctx, bank));
    const uint32_t k = prm->k, p = prm->hll_p, log2w = prm->cms_log2_width;
    EstPlan pl;
    st = est_plan(ctx, lengths, n_use, k, pl);
    if (st) return st;
    const uint64_t m = 1ULL << p, n_reads = 2 * n_use, cols = 4ULL << log2w;
    const uint32_t n_segs = pl.n_segs;
    Buffers buf(ctx);
    uint64_t* d_kbase = (uint64_t*)buf.get((n_reads + 1) * 8);
    uint32_t* first = (uint32_t*)buf.get(cols * 4);
    if (!d_kbase || !first) return set_err(ctx, FBK_ERR_OOM, "estimator buffers");
    CKE(cudaMemcpyAsync(d_kbase, pl.kbase.data(), (n_reads + 1) * 8, cudaMemcpyHostToDevice, ctx->stream));
    const BankDev bv = bank_view(bank, 2 * pair_begin, 2 * pair_end, nullptr);
    Launch L = launch_cfg(ctx, 256, 0);
    if (!first_in) {
        CKE(cudaMemsetAsync(first, 0xFF, cols * 4, ctx->stream));
        if (pair_end > pair_begin) TIMEDE("est_firstpos", launch_est_firstpos(L, bv, d_kbase, k, first, log2w));
        CKE(cudaMemcpyAsync(first_out, first, cols * 4, cudaMemcpyDeviceToHost, ctx->stream));
        CKE(cudaStreamSynchronize(ctx->stream));
        return FBK_OK;
    }
    uint32_t* regs = (uint32_t*)buf.get(2 * (uint64_t)n_segs * m * 4);
    if (!regs) return set_err(ctx, FBK_ERR_OOM, "estimator buffers");
    CKE(cudaMemcpyAsync(first, first_in, cols * 4, cudaMemcpyHostToDevice, ctx->stream));
    CKE(cudaMemsetAsync(regs, 0, 2 * (uint64_t)n_segs * m * 4, ctx->stream));
    if (pair_end > pair_begin)
        TIMEDE("est_hll", launch_est_hll(L, bv, d_kbase, k, first, log2w, p, n_segs, regs, regs + (uint64_t)n_segs * m));
    std::vector<uint32_t> h(2 * (uint64_t)n_segs * m);
    CKE(cudaMemcpyAsync(h.data(), regs, h.size() * 4, cudaMemcpyDeviceToHost, ctx->stream));
    CKE(cudaStreamSynchronize(ctx->stream));
    for (size_t i = 0; i < h.size(); ++i) regs_out[i] = (uint8_t)h[i];
    return FBK_OK;
}

}  // namespace

extern "C" {

FBK_API fbk_status fbk_estimate_sample(fbk_ctx* ctx, const fbk_arena_view* sample, uint64_t n_pairs, const fbk_count_stats* stats,
                                       const fbk_estimator_params* prm, fbk_genome_estimate* out, uint8_t* regs_total,
                                       uint8_t* regs_solid) {
    if (!ctx || !sample || !stats || !prm || !out) return FBK_ERR_INVALID;
    fbk_status st = check_est_params(ctx, prm);
    if (st) return st;
    if (sample->n_seqs < 2 * n_pairs) return set_err(ctx, FBK_ERR_INVALID, "sample holds fewer than 2*n_pairs reads");
    CKE(cudaSetDevice(ctx->device));
    const uint64_t n_use = est_n_use(stats, prm, n_pairs);
    if (n_use == 0) return set_err(ctx, FBK_ERR_EMPTY, "Input FASTQ files contain 0 valid read pairs");
    fbk_arena_view v = *sample;
    v.n_seqs = 2 * n_use;
    v.pair_idx = nullptr;
    fbk_bank* bank = nullptr;
    st = bank_upload_impl(ctx, &v, 1, &bank);
    if (st) return st;
    st = estimate_impl(ctx, bank, sample->lengths, n_use, stats, prm, out, regs_total, regs_solid);
    fbk_bank_release(bank);
    return st;
}

FBK_API fbk_status fbk_estimate_bank(fbk_ctx* ctx, const fbk_bank* sample, const uint32_t* read_lengths, uint64_t n_pairs,
                                     const fbk_count_stats* stats, const fbk_estimator_params* prm, fbk_genome_estimate* out,
                                     uint8_t* regs_total, uint8_t* regs_solid) {
    if (!ctx || !sample || !read_lengths || !stats || !prm || !out) return FBK_ERR_INVALID;
    fbk_status st = check_est_params(ctx, prm);
    if (st) return st;
    if (sample->n_reads < 2 * n_pairs) return set_err(ctx, FBK_ERR_INVALID, "sample holds fewer than 2*n_pairs reads");
    CKE(cudaSetDevice(ctx->device));
    CKE(bank_wait(ctx, sample));
    const uint64_t n_use = est_n_use(stats, prm, n_pairs);
    if (n_use == 0) return set_err(ctx, FBK_ERR_EMPTY, "Input FASTQ files contain 0 valid read pairs");
    return estimate_impl(ctx, sample, read_lengths, n_use, stats, prm, out, regs_total, regs_solid);
}

FBK_API fbk_status fbk_est_shard_plan(const uint32_t* read_lengths, uint64_t n_pairs, const fbk_count_stats* stats,
                                      const fbk_estimator_params* prm, uint64_t* n_use, uint32_t* n_segs) {
    if (!read_lengths || !stats || !prm || !n_use || !n_segs) return FBK_ERR_INVALID;
    fbk_status st = check_est_params(nullptr, prm);
    if (st) return st;
    *n_use = est_n_use(stats, prm, n_pairs);
    if (*n_use == 0) return FBK_ERR_EMPTY;
    EstPlan pl;
    st = est_plan(nullptr, read_lengths, *n_use, prm->k, pl);
    *n_segs = pl.n_segs;
    return st;
}

FBK_API fbk_status fbk_est_shard_firstpos(fbk_ctx* ctx, const fbk_bank* sample, const uint32_t* read_lengths, uint64_t n_use,
                                          uint64_t pair_begin, uint64_t pair_end, const fbk_estimator_params* prm,
                                          uint32_t* first) {
    if (!first) return FBK_ERR_INVALID;
    return est_shard_stage(ctx, sample, read_lengths, n_use, pair_begin, pair_end, prm, nullptr, first, nullptr);
}

FBK_API fbk_status fbk_est_shard_segments(fbk_ctx* ctx, const fbk_bank* sample, const uint32_t* read_lengths, uint64_t n_use,
                                          uint64_t pair_begin, uint64_t pair_end, const fbk_estimator_params* prm,
                                          const uint32_t* first, uint8_t* regs) {
    if (!first || !regs) return FBK_ERR_INVALID;
    return est_shard_stage(ctx, sample, read_lengths, n_use, pair_begin, pair_end, prm, first, nullptr, regs);
}

FBK_API fbk_status fbk_est_shard_finish(const uint32_t* read_lengths, uint64_t n_use, const fbk_count_stats* stats,
                                        const fbk_estimator_params* prm, const uint8_t* regs, fbk_genome_estimate* out,
                                        uint8_t* regs_total, uint8_t* regs_solid) {
    if (!read_lengths || !stats || !prm || !regs || !out) return FBK_ERR_INVALID;
    fbk_status st = check_est_params(nullptr, prm);
    if (st) return st;
    if (n_use == 0) return FBK_ERR_EMPTY;
    EstPlan pl;
    st = est_plan(nullptr, read_lengths, n_use, prm->k, pl);
    if (st) return st;
    const uint64_t m = 1ULL << prm->hll_p;
    const uint32_t n_segs = pl.n_segs;
    // registers at each checkpoint = running max over segments; sums of 2^-reg in
    // register order, as HyperLogLog::estimate adds them (sketch.rs:88-96)
    std::vector<uint8_t> run(2 * m, 0);
    std::vector<double> sums(2 * n_segs);
    std::vector<unsigned long long> zeros(2 * n_segs);
    std::vector<uint8_t> at_final(2 * m);
    for (int which = 0; which < 2; ++which) {
        uint8_t* cur = run.data() + which * m;
        for (uint32_t j = 0; j < n_segs; ++j) {
            const uint8_t* seg = regs + ((uint64_t)which * n_segs + j) * m;
            double sum = 0.0;
            unsigned long long z = 0;
            for (uint64_t i = 0; i < m; ++i) {
                if (seg[i] > cur[i]) cur[i] = seg[i];
                sum += std::ldexp(1.0, -(int)cur[i]);
                z += cur[i] == 0;
            }
            sums[which * n_segs + j] = sum;
            zeros[which * n_segs + j] = z;
        }
    }
    const uint32_t final_seg = est_decide(sums.data(), zeros.data(), pl, n_use, stats, prm, out);
    for (int which = 0; which < 2; ++which) {
        uint8_t* dst = which == 0 ? regs_total : regs_solid;
        if (!dst) continue;
        std::memset(dst, 0, m);
        for (uint32_t j = 0; j <= final_seg; ++j) {
            const uint8_t* seg = regs + ((uint64_t)which * n_segs + j) * m;
            for (uint64_t i = 0; i < m; ++i) dst[i] = std::max(dst[i], seg[i]);
        }
    }
    return FBK_OK;
}

FBK_API fbk_status fbk_estimate_genome(fbk_ctx* ctx, const char* r1, const char* r2, uint64_t max_pairs, double target_cov,
                                       fbk_genome_estimate* out) {
    if (!ctx || !r1 || !r2 || !out) return FBK_ERR_INVALID;
    fbk_count_stats stats;
    std::string err;
    fbk_status st = count_fastx_exact_impl(r1, r2, &stats, err);
    if (st) return set_err(ctx, st, err);
    fbk_estimator_params prm;
    fbk_estimator_defaults(&prm);
    prm.max_pairs = max_pairs;
    prm.target_cov = target_cov;
    const uint64_t want = std::min(std::min(max_pairs, prm.sample_cap), stats.exact_read_pairs);
    FastqReader a(r1), b(r2);
    if (!a.ok() || !b.ok()) return set_err(ctx, FBK_ERR_IO, "Failed to reopen FASTQ input");
    HostArena ar;
    std::string e;
    uint64_t n = 0;
    while (n < want) {
        if (a.next(e) != 1 || b.next(e) != 1) break;
        ar.push_ascii((const uint8_t*)a.seq.data(), a.seq.size(), (uint32_t)n);
        ar.push_ascii((const uint8_t*)b.seq.data(), b.seq.size(), (uint32_t)n);
        n++;
    }
    fbk_arena_view v = ar.view();
    return fbk_estimate_sample(ctx, &v, n, &stats, &prm, out, nullptr, nullptr);
}

}  // extern "C"
