// fbk_batch.cu — many isolates per launch: the counting stages of the reference
// pipeline (src/main.rs stage 1 estimate + subsampling policy, then the build front
// end src/graph/build.rs:84-328 at one k) for every isolate of a batch.
//
// Flow of fbk_batch_run:
//   1. estimator per isolate (fbk_estimate_bank on its raw sample pairs), the
//      subsampling policy (main.rs:76-180) and the subsampler bitmap;
//   2. phase A for a wave of isolates: sketch clear, pass 1, solidity bitmap and
//      the record / k-mer counts — one multi-isolate launch per step;
//   3. the host reads each isolate's distinct-key estimate and record count and
//      carves tables and record buckets for as many isolates as the pool holds;
//   4. phase B per sub-wave: table init, record emit, record prefix, upsert — one
//      multi-isolate launch each — and the SolidKmerNode conversion per isolate;
//   5. isolates whose buckets or table overflowed are redone by the
//      single-isolate path, which grows what overflowed.
// Each phase can run as one CUDA graph (captured on the context's stream).
#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

#include "fbk_device.cuh"
#include "fbk_internal.h"

using namespace fbk;

namespace {

struct BatchIso {
    uint64_t id = 0;
    fbk_bank* bank = nullptr;
    fbk_bank* sample = nullptr;
    std::vector<uint32_t> sample_len;
    uint64_t sample_pairs = 0;
    fbk_count_stats stats{};
    fbk_batch_result res{};
    uint64_t* keep = nullptr;
    uint32_t* cnt = nullptr;   // exact sketch (keep_sketch), or
    uint32_t* lad = nullptr;   // the gate ladder
    uint32_t* hll12 = nullptr;
    uint32_t* bm = nullptr;
    uint64_t distinct = 0, records = 0;
    fbk_table* table = nullptr;
    // phase-B storage
    uint64_t* recs = nullptr;
    unsigned long long* fill = nullptr;
    BucketDev bk{};
};

struct Shape {
    int block, grid, rows;
};

double now_ms() {
    return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

}  // namespace

struct fbk_batch {
    fbk_ctx* ctx = nullptr;
    fbk_batch_params p{};
    int nw = 1;
    bool ladder = false;  // the gate is a t_solid-level ladder (no sketch kept)
    std::vector<std::unique_ptr<BatchIso>> isos;
    fbk_batch_stats stats{};
    Shape pass1{256, 0, 4}, solid{256, 0, 4}, emit{256, 0, 0}, upsert{256, 0, 0};
    int emit_form = 0;     // 0: the context's choice (emit_form); else the phase-B autotuner's
    bool pass1_single = false;  // ladder pass 1 as one single-isolate launch per isolate (autotuned)
    bool pass1_single_used = false;  // the form the last wave ran
    bool tuned = false;    // pass-1 shape tuned
    bool tuned_b = false;  // emit form and shape, persistent-upsert shape tuned
    cudaEvent_t ev[2] = {nullptr, nullptr};
    void* h_stage = nullptr;  // pinned staging for descriptors and read-backs
    uint64_t h_stage_bytes = 0;
};

namespace {

constexpr uint32_t BATCH_STRIPES = 64;

uint32_t cms_cap_of(uint32_t cbits) { return cbits == 4 ? 15u : 0xFFFFu; }

void free_counting(fbk_batch* B, BatchIso* it, bool keep_sketch) {
    fbk_ctx* ctx = B->ctx;
    if (!keep_sketch) {
        dev_free(ctx, it->cnt);
        it->cnt = nullptr;
    }
    dev_free(ctx, it->lad);
    dev_free(ctx, it->hll12);
    dev_free(ctx, it->bm);
    it->lad = nullptr;
    it->hll12 = nullptr;
    it->bm = nullptr;
}

void free_buckets(fbk_batch* B, BatchIso* it) {
    dev_free(B->ctx, it->recs);
    dev_free(B->ctx, it->fill);
    it->recs = nullptr;
    it->fill = nullptr;
}

void free_iso(fbk_batch* B, BatchIso* it) {
    fbk_ctx* ctx = B->ctx;
    cudaStreamSynchronize(ctx->stream);
    free_buckets(B, it);
    free_counting(B, it, false);
    dev_free(ctx, it->keep);
    it->keep = nullptr;
    if (it->table) fbk_table_release(it->table);
    it->table = nullptr;
    if (it->bank) fbk_bank_release(it->bank);
    if (it->sample) fbk_bank_release(it->sample);
    it->bank = it->sample = nullptr;
}

fbk_status stage(fbk_batch* B, uint64_t bytes) {
    if (bytes <= B->h_stage_bytes) return FBK_OK;
    if (B->h_stage) cudaFreeHost(B->h_stage);
    B->h_stage = nullptr;
    B->h_stage_bytes = 0;
    const uint64_t nb = std::max<uint64_t>(bytes, 1 << 20);
    CK(B->ctx, cudaMallocHost(&B->h_stage, nb));
    B->h_stage_bytes = nb;
    return FBK_OK;
}

// Runs body() on the context's stream — captured as one CUDA graph when the batch
// uses graphs — and adds the phase's device time to *ms.
template <class F>
fbk_status run_phase(fbk_batch* B, double* ms, F&& body) {
    fbk_ctx* ctx = B->ctx;
    if (!B->p.use_graphs) {
        CK(ctx, cudaEventRecord(B->ev[0], ctx->stream));
        fbk_status st = body();
        if (st) return st;
        CK(ctx, cudaEventRecord(B->ev[1], ctx->stream));
    } else {
        CK(ctx, cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
        ctx->capturing = true;
        fbk_status st = body();
        ctx->capturing = false;
        cudaGraph_t g = nullptr;
        cudaError_t e = cudaStreamEndCapture(ctx->stream, &g);
        if (st) {
            if (g) cudaGraphDestroy(g);
            return st;
        }
        if (e != cudaSuccess) return cuda_err(ctx, e, "batch phase capture");
        cudaGraphExec_t x = nullptr;
        e = cudaGraphInstantiate(&x, g, 0);
        if (e == cudaSuccess) e = cudaEventRecord(B->ev[0], ctx->stream);
        if (e == cudaSuccess) e = cudaGraphLaunch(x, ctx->stream);
        if (e == cudaSuccess) e = cudaEventRecord(B->ev[1], ctx->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
        if (x) cudaGraphExecDestroy(x);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) return cuda_err(ctx, e, "batch phase graph");
        B->stats.graph_launches++;
    }
    CK(ctx, cudaEventSynchronize(B->ev[1]));
    float t = 0.f;
    CK(ctx, cudaEventElapsedTime(&t, B->ev[0], B->ev[1]));
    *ms += t;
    return FBK_OK;
}

Launch shape_launch(fbk_ctx* ctx, const Shape& s) { return launch_cfg_persistent(ctx, s.block, s.grid); }

// Stage 1: estimate, subsampling decision and subsampler bitmap of one isolate.
fbk_status estimate_one(fbk_batch* B, BatchIso* it) {
    fbk_ctx* ctx = B->ctx;
    fbk_estimator_params ep;
    fbk_estimator_defaults(&ep);
    ep.max_pairs = B->p.est_max_pairs;
    ep.target_cov = B->p.policy.depth;
    fbk_status st = fbk_estimate_bank(ctx, it->sample, it->sample_len.data(), it->sample_pairs, &it->stats, &ep,
                                      &it->res.estimate, nullptr, nullptr);
    if (st) return st;
    st = fbk_subsample_decide(&B->p.policy, &it->res.estimate, &it->res.subsample_factor, &it->res.subsample_reason);
    if (st) return set_err(ctx, st, "invalid subsampling policy");
    fbk_subsample ss{it->res.subsample_factor, B->p.subsample_seed};
    st = keep_bits_for(ctx, it->bank, &ss, &it->keep);
    if (st) return st;
    // the estimator's sample is no longer needed
    fbk_bank_release(it->sample);
    it->sample = nullptr;
    it->res.state = 1;
    return FBK_OK;
}

IsoDev iso_dev(const fbk_batch* B, const BatchIso* it, unsigned long long* nrec, uint32_t* status) {
    IsoDev d{};
    d.b = bank_view(it->bank, 0, it->bank->n_reads, it->keep);
    d.cnt = it->cnt;
    d.lad = it->lad;
    d.hll12 = it->hll12;
    d.bm = it->bm;
    d.n_records = nrec;
    d.log2w = B->p.cms_log2_width;
    d.t_solid = B->p.t_solid;
    d.cap = cms_cap_of(B->p.counter_bits);
    d.status = status;
    if (it->table) d.t = tbl_dev(it->table);
    d.bk = it->bk;
    return d;
}

// Per-wave device scratch: descriptors, read bases, counters.
struct WaveBufs {
    fbk_ctx* ctx = nullptr;
    IsoDev* iso = nullptr;
    unsigned long long* rb = nullptr;
    unsigned long long* cnt = nullptr;   // 8 per isolate: [0..2] record/k-mer counts, [3..7] conversion counts
    uint32_t* status = nullptr;          // 2 per isolate: status bits, bucket overflow
    ~WaveBufs() {
        if (!ctx) return;
        cudaStreamSynchronize(ctx->stream);
        dev_free(ctx, iso);
        dev_free(ctx, rb);
        dev_free(ctx, cnt);
        dev_free(ctx, status);
    }
};

fbk_status wave_bufs(fbk_batch* B, uint32_t n, bool phase_b, WaveBufs& w) {
    fbk_ctx* ctx = B->ctx;
    w.ctx = ctx;
    w.iso = (IsoDev*)dev_alloc(ctx, n * sizeof(IsoDev));
    w.rb = (unsigned long long*)dev_alloc(ctx, (n + 1) * 8);
    w.cnt = (unsigned long long*)dev_alloc(ctx, (uint64_t)n * 8 * 8);
    w.status = (uint32_t*)dev_alloc(ctx, (uint64_t)n * 2 * 4);
    (void)phase_b;
    if (!w.iso || !w.rb || !w.cnt || !w.status)
        return set_err(ctx, FBK_ERR_OOM, "batch wave descriptors");
    return FBK_OK;
}

// Copies descriptors and read bases of a wave to the device (before any capture).
fbk_status upload_wave(fbk_batch* B, const std::vector<BatchIso*>& W, WaveBufs& w) {
    fbk_ctx* ctx = B->ctx;
    const uint32_t n = (uint32_t)W.size();
    fbk_status st = stage(B, n * sizeof(IsoDev) + (n + 1) * 8);
    if (st) return st;
    IsoDev* hd = (IsoDev*)B->h_stage;
    unsigned long long* hb = (unsigned long long*)((char*)B->h_stage + n * sizeof(IsoDev));
    hb[0] = 0;
    for (uint32_t i = 0; i < n; ++i) {
        hd[i] = iso_dev(B, W[i], w.cnt + 8 * i, w.status + 2 * i);
        hd[i].bk.overflow = w.status + 2 * i + 1;
        hb[i + 1] = hb[i] + W[i]->bank->n_reads;
    }
    CK(ctx, cudaMemcpyAsync(w.iso, hd, n * sizeof(IsoDev), cudaMemcpyHostToDevice, ctx->stream));
    CK(ctx, cudaMemcpyAsync(w.rb, hb, (n + 1) * 8, cudaMemcpyHostToDevice, ctx->stream));
    CK(ctx, cudaStreamSynchronize(ctx->stream));  // the staging buffer is reused next
    return FBK_OK;
}

uint64_t gate_bytes(const fbk_batch* B) {
    return B->ladder ? (uint64_t)B->p.t_solid * (4ULL << B->p.cms_log2_width) / 8 + 256 : (4ULL << B->p.cms_log2_width) * 4;
}

uint64_t phase_a_bytes(const fbk_batch* B, const BatchIso* it) {
    return gate_bytes(B) + 4096 * 4 + (B->ladder ? 0 : (it->bank->n_words + 9) * 4) + 4096;
}

// Autotuner: times candidate launch shapes of the pass-1 and solidity kernels on one
// isolate (its own sketch and bitmap as scratch) and keeps the fastest.
fbk_status autotune(fbk_batch* B, BatchIso* it) {
    fbk_ctx* ctx = B->ctx;
    const double t0 = now_ms();
    WaveBufs w;
    fbk_status st = wave_bufs(B, 1, false, w);
    if (st) return st;
    std::vector<BatchIso*> one{it};
    st = upload_wave(B, one, w);
    if (st) return st;
    const uint64_t cms_bytes = gate_bytes(B);
    const int blocks[] = {128, 256};
    const int per_sm[] = {0, 2, 4};
    const int rows_all[] = {4, 2, 1};
    const int rows_one[] = {4};
    // a ladder serves all rows in one sweep: only block and grid are tuned
    const std::vector<int> rows = B->ladder ? std::vector<int>(rows_one, rows_one + 1) : std::vector<int>(rows_all, rows_all + 3);
    uint32_t* gate = B->ladder ? it->lad : it->cnt;
    auto timed = [&](auto&& launch, float* ms) -> fbk_status {
        CK(ctx, cudaEventRecord(B->ev[0], ctx->stream));
        fbk_status s2 = launch();
        if (s2) return s2;
        CK(ctx, cudaEventRecord(B->ev[1], ctx->stream));
        CK(ctx, cudaEventSynchronize(B->ev[1]));
        CK(ctx, cudaEventElapsedTime(ms, B->ev[0], B->ev[1]));
        return FBK_OK;
    };
    float best = 1e30f;
    Shape best1 = B->pass1;
    for (int rp : rows)
        for (int bl : blocks)
            for (int ps : per_sm) {
                Shape s{bl, ps ? ps * ctx->num_sms : 0, rp};
                CK(ctx, cudaMemsetAsync(gate, 0, cms_bytes, ctx->stream));
                float ms = 0;
                st = timed([&]() -> fbk_status {
                    if (B->ladder) {
                        TIMED(ctx, "tune_pass1", launch_batch_lpass1(B->nw, shape_launch(ctx, s), w.iso, w.rb, 1, B->p.k));
                        return FBK_OK;
                    }
                    for (uint32_t r = 0; r < 4; r += (uint32_t)rp)
                        TIMED(ctx, "tune_pass1", launch_batch_pass1(B->nw, shape_launch(ctx, s), w.iso, w.rb, 1, B->p.k, r, r + rp, 0));
                    return FBK_OK;
                }, &ms);
                if (st) return st;
                if (ms < best) {
                    best = ms;
                    best1 = s;
                }
            }
    // With a ladder gate the single-isolate pass 1 (its form chosen per key width by the
    // context) is a candidate too: one launch per isolate of the wave.
    bool single = false;
    if (B->ladder) {
        CK(ctx, cudaMemsetAsync(gate, 0, cms_bytes, ctx->stream));
        CK(ctx, cudaMemsetAsync(it->hll12, 0, 4096 * 4, ctx->stream));
        float ms = 0;
        st = timed([&]() -> fbk_status {
            TIMED(ctx, "tune_pass1", launch_ladder_pass1(B->nw, launch_cfg_persistent(ctx, 256, 0),
                                                         bank_view(it->bank, 0, it->bank->n_reads, it->keep), B->p.k, it->lad,
                                                         B->p.cms_log2_width, B->p.t_solid, it->hll12,
                                                         ladder_form(ctx, B->nw)));
            return FBK_OK;
        }, &ms);
        if (st) return st;
        single = ms < best;
    }
    // the sketch now holds the isolate's full counts: tune the solidity sweep on it
    // (a ladder gate has no solidity sweep: the emit evaluates it)
    const uint64_t bm_bytes = (it->bank->n_words + 9) * 4;
    best = 1e30f;
    Shape best2 = B->solid;
    for (int rp : (B->ladder ? std::vector<int>() : rows))
        for (int bl : blocks)
            for (int ps : per_sm) {
                Shape s{bl, ps ? ps * ctx->num_sms : 0, rp};
                CK(ctx, cudaMemsetAsync(it->bm, 0xFF, bm_bytes, ctx->stream));
                float ms = 0;
                st = timed([&]() -> fbk_status {
                    for (uint32_t r = 0; r < 4; r += (uint32_t)rp)
                        TIMED(ctx, "tune_solid", launch_batch_solid(B->nw, shape_launch(ctx, s), w.iso, w.rb, 1, B->p.k, r, r + rp));
                    return FBK_OK;
                }, &ms);
                if (st) return st;
                if (ms < best) {
                    best = ms;
                    best2 = s;
                }
            }
    B->pass1 = best1;
    B->pass1_single = single;
    B->solid = best2;
    B->tuned = true;
    B->stats.tuned = 1;
    B->stats.tune_ms += now_ms() - t0;
    return FBK_OK;
}

// Phase-B autotuner (ladder gate): on the first phase-B isolate, with its table and
// record buckets allocated, time the record emit in each form and block shape — flat
// window stream with blocks of 128 or 256, one lane per read (rolled) — and, when the
// isolate's pass upserts every bucket in one persistent launch, that launch with blocks
// of 128 or 256 at the occupancy grid or 2 or 4 blocks per SM.  Each trial starts from
// cleared bucket counters (and, for the upsert, a cleared table); phase B itself clears
// both again before it runs, so the trials leave nothing behind.
fbk_status autotune_b(fbk_batch* B, BatchIso* it, bool persistent_upsert) {
    fbk_ctx* ctx = B->ctx;
    const double t0 = now_ms();
    auto timed = [&](auto&& launch, float* ms) -> fbk_status {
        CK(ctx, cudaEventRecord(B->ev[0], ctx->stream));
        fbk_status s2 = launch();
        if (s2) return s2;
        CK(ctx, cudaEventRecord(B->ev[1], ctx->stream));
        CK(ctx, cudaEventSynchronize(B->ev[1]));
        CK(ctx, cudaEventElapsedTime(ms, B->ev[0], B->ev[1]));
        return FBK_OK;
    };
    uint32_t* flags = (uint32_t*)dev_alloc(ctx, 256);  // overflow flag, status word, work counter
    if (!flags) return set_err(ctx, FBK_ERR_OOM, "batch autotuner");
    BucketDev bk = it->bk;
    bk.overflow = flags;
    unsigned long long* work = (unsigned long long*)(flags + 2);
    const BankDev bv = bank_view(it->bank, 0, it->bank->n_reads, it->keep);
    struct Cand {
        int form, block;
    };
    const Cand emits[] = {{3, 128}, {3, 256}, {4, 256}};
    float best = 1e30f;
    Cand best_e = emits[0];
    fbk_status st = FBK_OK;
    for (const Cand& c : emits) {
        cudaError_t e = cudaMemsetAsync(it->fill, 0, (uint64_t)bk.n_buckets * bk.stripes * 8, ctx->stream);
        if (e == cudaSuccess) e = cudaMemsetAsync(flags, 0, 16, ctx->stream);
        if (e != cudaSuccess) {
            st = cuda_err(ctx, e, "batch autotuner");
            break;
        }
        float ms = 0;
        st = timed([&]() -> fbk_status {
            TIMED(ctx, "tune_emit", launch_emit_ladder(B->nw, launch_cfg_persistent(ctx, c.block, 0), bv, B->p.k, it->lad,
                                                       B->p.cms_log2_width, B->p.t_solid, tbl_dev(it->table), bk, c.form));
            return FBK_OK;
        }, &ms);
        if (st) break;
        if (ms < best) {
            best = ms;
            best_e = c;
        }
    }
    if (st == FBK_OK && persistent_upsert) {
        // the buckets hold the last trial's records (every form writes the same records)
        const int blocks[] = {128, 256};
        const int per_sm[] = {0, 2, 4};
        best = 1e30f;
        Shape best_u = B->upsert;
        for (int bl : blocks)
            for (int ps : per_sm) {
                const Shape sh{bl, ps ? ps * ctx->num_sms : 0, 0};
                cudaError_t e = cudaSuccess;
                st = FBK_OK;
                TIMED(ctx, "table_init", launch_table_init(B->nw, launch_cfg(ctx, 256, 0), tbl_dev(it->table)));
                e = cudaMemsetAsync(it->table->cnt, 0, it->table->cap * 32, ctx->stream);
                if (e == cudaSuccess) e = cudaMemsetAsync(flags, 0, 24, ctx->stream);
                if (e != cudaSuccess) {
                    st = cuda_err(ctx, e, "batch autotuner");
                    break;
                }
                float ms = 0;
                st = timed([&]() -> fbk_status {
                    TIMED(ctx, "tune_upsert", launch_upsert_all(B->nw, shape_launch(ctx, sh), bk, 1, 1, tbl_dev(it->table),
                                                                flags + 1, work, ctx->upsert_all));
                    return FBK_OK;
                }, &ms);
                if (st) break;
                if (ms < best) {
                    best = ms;
                    best_u = sh;
                }
            }
        if (st == FBK_OK) B->upsert = best_u;
    }
    cudaStreamSynchronize(ctx->stream);
    dev_free(ctx, flags);
    if (st) return st;
    B->emit = Shape{best_e.block, 0, 0};
    B->emit_form = best_e.form;
    B->tuned_b = true;
    B->stats.tune_ms += now_ms() - t0;
    return FBK_OK;
}

// Phase A of a wave: pass 1, solidity bitmap, counts; then the host reads each
// isolate's distinct-key estimate and record count.
fbk_status phase_a(fbk_batch* B, const std::vector<BatchIso*>& W) {
    fbk_ctx* ctx = B->ctx;
    const uint32_t n = (uint32_t)W.size();
    const uint64_t cms_bytes = gate_bytes(B);
    for (BatchIso* it : W) {
        if (B->ladder) it->lad = (uint32_t*)dev_alloc(ctx, cms_bytes);
        else it->cnt = (uint32_t*)dev_alloc(ctx, cms_bytes);
        it->hll12 = (uint32_t*)dev_alloc(ctx, 4096 * 4);
        if (!B->ladder) it->bm = (uint32_t*)dev_alloc(ctx, (it->bank->n_words + 9) * 4);
        if (!(it->cnt || it->lad) || !it->hll12 || (!B->ladder && !it->bm)) return set_err(ctx, FBK_ERR_OOM, "batch sketches");
    }
    if (B->p.autotune && !B->tuned) {
        BatchIso* big = *std::max_element(W.begin(), W.end(), [](const BatchIso* a, const BatchIso* b) {
            return a->bank->n_bases < b->bank->n_bases;
        });
        fbk_status st = autotune(B, big);
        if (st) return st;
    }
    WaveBufs w;
    fbk_status st = wave_bufs(B, n, false, w);
    if (st) return st;
    st = upload_wave(B, W, w);
    if (st) return st;
    const uint32_t k = B->p.k;
    st = run_phase(B, &B->stats.ms_phase_a, [&]() -> fbk_status {
        for (BatchIso* it : W) {
            CK(ctx, cudaMemsetAsync(B->ladder ? it->lad : it->cnt, 0, cms_bytes, ctx->stream));
            CK(ctx, cudaMemsetAsync(it->hll12, 0, 4096 * 4, ctx->stream));
            if (it->bm) CK(ctx, cudaMemsetAsync(it->bm, 0xFF, (it->bank->n_words + 9) * 4, ctx->stream));
        }
        CK(ctx, cudaMemsetAsync(w.cnt, 0, (uint64_t)n * 64, ctx->stream));
        CK(ctx, cudaMemsetAsync(w.status, 0, (uint64_t)n * 8, ctx->stream));
        if (B->ladder) {
            // the gate is evaluated inside the record emit: no bitmap, and the
            // records are bounded by the windows the count kernel tallies
            // The autotuner compares the two forms on one isolate; a wave whose gates
            // together outgrow half the L2 runs its isolates one launch each, since the
            // multi-isolate launch then climbs every gate of the wave at once (64
            // isolates of 4 MB gates: 396 vs 364 ms of pass 1 per cohort).
            const bool single = ctx->batch_pass1 ? ctx->batch_pass1 == 2
                                                 : B->pass1_single || (uint64_t)n * gate_bytes(B) > (64ull << 20);
            B->pass1_single_used = single;
            if (single) {
                for (BatchIso* it : W)
                    TIMED(ctx, "batch_pass1", launch_ladder_pass1(B->nw, launch_cfg_persistent(ctx, 256, 0),
                                                                  bank_view(it->bank, 0, it->bank->n_reads, it->keep), k, it->lad,
                                                                  B->p.cms_log2_width, B->p.t_solid, it->hll12,
                                                                  ladder_form(ctx, B->nw)));
            } else {
                TIMED(ctx, "batch_pass1", launch_batch_lpass1(B->nw, shape_launch(ctx, B->pass1), w.iso, w.rb, n, k));
            }
            TIMED(ctx, "batch_count", launch_batch_count(shape_launch(ctx, B->solid), w.iso, w.rb, n, k));
            return FBK_OK;
        }
        for (uint32_t r = 0; r < 4; r += (uint32_t)B->pass1.rows)
            TIMED(ctx, "batch_pass1", launch_batch_pass1(B->nw, shape_launch(ctx, B->pass1), w.iso, w.rb, n, k, r,
                                                         r + (uint32_t)B->pass1.rows, r == 0));
        for (uint32_t r = 0; r < 4; r += (uint32_t)B->solid.rows)
            TIMED(ctx, "batch_solid", launch_batch_solid(B->nw, shape_launch(ctx, B->solid), w.iso, w.rb, n, k, r,
                                                         r + (uint32_t)B->solid.rows));
        TIMED(ctx, "batch_count", launch_batch_count(shape_launch(ctx, B->solid), w.iso, w.rb, n, k));
        return FBK_OK;
    });
    if (st) return st;
    // read back the HyperLogLog registers and counts
    const double h0 = now_ms();
    st = stage(B, (uint64_t)n * (4096 * 4 + 64));
    if (st) return st;
    uint32_t* hr = (uint32_t*)B->h_stage;
    unsigned long long* hc = (unsigned long long*)(hr + (uint64_t)n * 4096);
    for (uint32_t i = 0; i < n; ++i)
        CK(ctx, cudaMemcpyAsync(hr + (uint64_t)i * 4096, W[i]->hll12, 4096 * 4, cudaMemcpyDeviceToHost, ctx->stream));
    CK(ctx, cudaMemcpyAsync(hc, w.cnt, (uint64_t)n * 64, cudaMemcpyDeviceToHost, ctx->stream));
    CK(ctx, cudaStreamSynchronize(ctx->stream));
    for (uint32_t i = 0; i < n; ++i) {
        BatchIso* it = W[i];
        double sum = 0.0;
        uint64_t zeros = 0;
        for (int j = 0; j < 4096; ++j) {
            const uint32_t v = hr[(uint64_t)i * 4096 + j];
            sum += std::ldexp(1.0, -(int)v);
            zeros += v == 0;
        }
        // the registers saw 1 in BATCH_HLL_SAMPLE keys (by hash)
        it->distinct = (uint64_t)(hll_estimate_from_sum(sum, zeros, 12) * BATCH_HLL_SAMPLE * 1.08) + 4096;
        it->records = B->ladder ? hc[8 * i + 2] : hc[8 * i];
        it->res.kmers = hc[8 * i + 1] + hc[8 * i + 2];
        it->res.state = 2;
    }
    B->stats.ms_host += now_ms() - h0;
    return FBK_OK;
}

uint64_t slot_bytes_of(int nw) { return 8ULL * nw + (nw > 2 ? 8 : 0) + 32; }

// Table capacity, bucket geometry and device bytes of phase B for one isolate.
struct PlanB {
    uint64_t cap, out_cap, per_stripe, bytes;
    uint32_t shift, n_buckets;
};

PlanB plan_b(const fbk_batch* B, const BatchIso* it) {
    const fbk_ctx* ctx = B->ctx;
    PlanB q;
    q.cap = std::max<uint64_t>(1024, (uint64_t)((double)it->distinct / ctx->load_factor) + 1024);
    q.out_cap = std::min<uint64_t>(q.cap, (uint64_t)(1.1 * (double)it->distinct) + 4096);
    const uint64_t sb = slot_bytes_of(B->nw);
    uint32_t shift = 0;
    while (shift < 40 && (2ULL << shift) * sb <= ctx->bucket_bytes) ++shift;
    while (((q.cap + (1ULL << shift) - 1) >> shift) > 64) ++shift;
    q.shift = shift;
    q.n_buckets = (uint32_t)((q.cap + (1ULL << shift) - 1) >> shift);
    q.per_stripe = (uint64_t)(1.15 * (double)it->records / ((double)q.n_buckets * BATCH_STRIPES)) + 2048;
    q.bytes = q.cap * sb + q.out_cap * (8ULL * B->nw + 3) +
              (uint64_t)q.n_buckets * BATCH_STRIPES * (q.per_stripe * 8 * record_format(B->p.k, B->nw).rw + 8) + 8192;
    return q;
}

// Allocates an isolate's table, output rows and record buckets.
fbk_status alloc_b(fbk_batch* B, BatchIso* it, const PlanB& q) {
    fbk_ctx* ctx = B->ctx;
    fbk_table* t = new fbk_table();
    t->ctx = ctx;
    t->nw = (uint32_t)B->nw;
    t->k = B->p.k;
    t->min_trans_cov = B->p.min_trans_cov;
    it->table = t;
    t->cap = q.cap;
    t->keys = (uint64_t*)dev_alloc(ctx, q.cap * 8 * t->nw);
    if (t->nw > 2) t->tags = tag_in_key(t->nw, t->k) ? t->keys : (uint64_t*)dev_alloc(ctx, q.cap * 8);
    t->cnt = (uint32_t*)dev_alloc(ctx, q.cap * 32);
    t->out_keys = (uint64_t*)dev_alloc(ctx, q.out_cap * 8 * t->nw);
    t->out_cov = (uint16_t*)dev_alloc(ctx, q.out_cap * 2);
    t->out_mask = (uint8_t*)dev_alloc(ctx, q.out_cap);
    t->out_cap = q.out_cap;
    const RecFmt fmt = record_format(B->p.k, B->nw);
    it->recs = (uint64_t*)dev_alloc(ctx, (uint64_t)q.n_buckets * BATCH_STRIPES * q.per_stripe * 8 * fmt.rw);
    it->fill = (unsigned long long*)dev_alloc(ctx, (uint64_t)q.n_buckets * BATCH_STRIPES * 8);
    if (!t->keys || (t->nw > 2 && !t->tags) || !t->cnt || !t->out_keys || !t->out_cov || !t->out_mask || !it->recs || !it->fill)
        return set_err(ctx, FBK_ERR_OOM, "batch table");
    it->bk = BucketDev{};
    it->bk.recs = it->recs;
    it->bk.fill = it->fill;
    it->bk.stripe_cap = q.per_stripe;
    it->bk.shift = q.shift;
    it->bk.n_buckets = q.n_buckets;
    it->bk.stripes = BATCH_STRIPES;
    it->bk.rw = fmt.rw;
    it->bk.ws = fmt.ws;
    it->bk.packed = fmt.packed;
    return FBK_OK;
}

void release_b(fbk_batch* B, BatchIso* it) {
    free_buckets(B, it);
    if (it->table) fbk_table_release(it->table);
    it->table = nullptr;
}

void finish_iso(fbk_batch* B, BatchIso* it);

// The single-isolate path for an isolate whose wave buckets or table overflowed.
fbk_status fallback(fbk_batch* B, BatchIso* it) {
    fbk_ctx* ctx = B->ctx;
    release_b(B, it);
    fbk_cms view;
    view.ctx = ctx;
    view.cnt = it->cnt;
    view.log2w = B->p.cms_log2_width;
    view.cbits = B->p.counter_bits;
    view.n = 4ULL << view.log2w;
    fbk_build_params bp{};
    bp.k = B->p.k;
    bp.key_bits = B->p.key_bits;
    bp.cms_log2_width = B->p.cms_log2_width;
    bp.counter_bits = B->p.counter_bits;
    bp.t_solid = B->p.t_solid;
    bp.min_trans_cov = B->p.min_trans_cov;
    fbk_status st = B->ladder ? solid_build_ladder(ctx, it->bank, it->lad, B->p.cms_log2_width, &bp, it->keep, it->distinct * 2, &it->table)
                              : solid_build(ctx, it->bank, &view, &bp, it->keep, it->distinct * 2, &it->table);
    view.cnt = nullptr;
    if (st) return st;
    it->res.fallback = 1;
    B->stats.fallbacks++;
    return FBK_OK;
}

// Phase B of a sub-wave: tables, emit, prefix, upsert, conversion; then per-isolate
// checks and clean-up.
fbk_status phase_b(fbk_batch* B, const std::vector<BatchIso*>& V) {
    fbk_ctx* ctx = B->ctx;
    const uint32_t n = (uint32_t)V.size();
    WaveBufs w;
    fbk_status st = wave_bufs(B, n, true, w);
    if (st) return st;
    st = upload_wave(B, V, w);
    if (st) return st;
    const uint32_t k = B->p.k;
    // record filter (see k_count_records): one pair of counter rows serves the wave's
    // bucket upserts in turn; isolates whose reads span several chunks go unfiltered
    std::vector<RecordFilter> flt(n);
    uint32_t log2m_max = 0;
    for (uint32_t i = 0; i < n; ++i) {
        const BatchIso* it = V[i];
        if (!acc_filter_on(ctx->acc_filter, B->nw, it->distinct, it->records) || B->p.min_trans_cov < 2 ||
            it->bank->chunk_starts.size() != 2)
            continue;
        uint32_t log2m = 11;
        while (log2m < 23 && (1ULL << log2m) < it->records / std::max<uint32_t>(1, it->bk.n_buckets)) ++log2m;
        flt[i].log2m = log2m;
        flt[i].min_records = B->p.min_trans_cov;
        flt[i].skipped = w.cnt + 8 * i;  // word 0 of the isolate's counters is free in phase B
        log2m_max = std::max(log2m_max, log2m);
    }
    struct FilterBuf {
        fbk_ctx* c;
        uint32_t* p = nullptr;
        ~FilterBuf() {
            if (p) {
                cudaStreamSynchronize(c->stream);
                dev_free(c, p);
            }
        }
    } fbuf{ctx};
    if (log2m_max) {
        fbuf.p = (uint32_t*)dev_alloc(ctx, (1ULL << log2m_max) * 4);
        if (!fbuf.p) return set_err(ctx, FBK_ERR_OOM, "batch record filter");
        for (uint32_t i = 0; i < n; ++i)
            if (flt[i].log2m) flt[i].cnt = fbuf.p;
    }
    // work-item counters of the persistent upserts (unfiltered isolates)
    struct WorkBuf {
        fbk_ctx* c;
        unsigned long long* p = nullptr;
        ~WorkBuf() {
            if (p) {
                cudaStreamSynchronize(c->stream);
                dev_free(c, p);
            }
        }
    } work{ctx};
    if (ctx->upsert_all) {
        work.p = (unsigned long long*)dev_alloc(ctx, (uint64_t)n * 8);
        if (!work.p) return set_err(ctx, FBK_ERR_OOM, "batch upsert counters");
    }
    if (B->p.autotune && B->ladder && !B->tuned_b) {
        st = autotune_b(B, V[0], work.p != nullptr && !flt[0].cnt);
        if (st) return st;
    }
    const int eform = B->emit_form ? B->emit_form : emit_form(ctx, B->nw);
    st = run_phase(B, &B->stats.ms_phase_b, [&]() -> fbk_status {
        CK(ctx, cudaMemsetAsync(w.cnt, 0, (uint64_t)n * 64, ctx->stream));
        CK(ctx, cudaMemsetAsync(w.status, 0, (uint64_t)n * 8, ctx->stream));
        for (BatchIso* it : V) {
            TIMED(ctx, "table_init", launch_table_init(B->nw, launch_cfg(ctx, 256, 0), tbl_dev(it->table)));
            CK(ctx, cudaMemsetAsync(it->table->cnt, 0, it->table->cap * 32, ctx->stream));
            CK(ctx, cudaMemsetAsync(it->fill, 0, (uint64_t)it->bk.n_buckets * BATCH_STRIPES * 8, ctx->stream));
        }
        if (B->ladder) {
            for (uint32_t i = 0; i < n; ++i) {
                BatchIso* it = V[i];
                BucketDev bk = it->bk;
                bk.overflow = w.status + 2 * i + 1;
                TIMED(ctx, "batch_emit", launch_emit_ladder(B->nw, shape_launch(ctx, B->emit),
                                                            bank_view(it->bank, 0, it->bank->n_reads, it->keep), k, it->lad,
                                                            B->p.cms_log2_width, B->p.t_solid, tbl_dev(it->table), bk,
                                                            eform));
            }
        } else {
            TIMED(ctx, "batch_emit", launch_batch_emit(B->nw, shape_launch(ctx, B->emit), w.iso, w.rb, n, k, BATCH_STRIPES));
        }
        // upserts bucket by bucket, so each launch's table range stays in L2
        if (work.p) CK(ctx, cudaMemsetAsync(work.p, 0, (uint64_t)n * 8, ctx->stream));
        for (uint32_t i = 0; i < n; ++i) {
            BatchIso* it = V[i];
            BucketDev bk = it->bk;
            bk.overflow = w.status + 2 * i + 1;
            if (work.p && !flt[i].cnt) {
                TIMED(ctx, "batch_upsert", launch_upsert_all(B->nw, shape_launch(ctx, B->upsert), bk, 1, 1, tbl_dev(it->table),
                                                             w.status + 2 * i, work.p + i, ctx->upsert_all));
                continue;
            }
            for (uint32_t bu = 0; bu < bk.n_buckets; ++bu) {
                if (flt[i].cnt) {
                    CK(ctx, cudaMemsetAsync(flt[i].cnt, 0, (1ULL << flt[i].log2m) * 4, ctx->stream));
                    TIMED(ctx, "batch_filter", launch_count_records(B->nw, shape_launch(ctx, B->upsert), bk, bu, flt[i]));
                }
                TIMED(ctx, "batch_upsert", launch_upsert(B->nw, shape_launch(ctx, B->upsert), bk, bu, 1, 1, tbl_dev(it->table),
                                                         w.status + 2 * i, flt[i], ctx->upsert_queue));
            }
        }
        for (uint32_t i = 0; i < n; ++i) {
            fbk_table* t = V[i]->table;
            ConvOut o{};
            o.keys = t->out_keys;
            o.cov = t->out_cov;
            o.mask = t->out_mask;
            o.cap_solid = t->out_cap;
            o.counts = w.cnt + 8 * i + 3;
            TIMED(ctx, "convert", launch_convert(B->nw, launch_cfg(ctx, 256, 0), tbl_dev(t), t->min_trans_cov, o));
        }
        return FBK_OK;
    });
    if (st) return st;
    st = stage(B, (uint64_t)n * 72);
    if (st) return st;
    unsigned long long* hc = (unsigned long long*)B->h_stage;
    uint32_t* hs = (uint32_t*)(hc + 8ULL * n);
    CK(ctx, cudaMemcpyAsync(hc, w.cnt, (uint64_t)n * 64, cudaMemcpyDeviceToHost, ctx->stream));
    CK(ctx, cudaMemcpyAsync(hs, w.status, (uint64_t)n * 8, cudaMemcpyDeviceToHost, ctx->stream));
    CK(ctx, cudaStreamSynchronize(ctx->stream));
    std::vector<unsigned long long> counts(hc, hc + 8ULL * n);
    std::vector<uint32_t> stat(hs, hs + 2ULL * n);
    for (uint32_t i = 0; i < n; ++i) {
        BatchIso* it = V[i];
        const uint32_t bits = stat[2 * i], ovf = stat[2 * i + 1];
        if (bits & ST_SPIN_TIMEOUT) {
            release_b(B, it);
            return set_err(ctx, FBK_ERR_TIMEOUT, "batch: a bounded wait for a key publication gave up");
        }
        if ((bits & ST_TABLE_FULL) || ovf) {
            st = fallback(B, it);
            if (st) return st;
        } else {
            fbk_table* t = it->table;
            t->n_keys = counts[8 * i + 3];
            t->n_solid = counts[8 * i + 4];
            t->digest = counts[8 * i + 5];
            t->skipped_pushes = counts[8 * i + 0];
            t->pushes = counts[8 * i + 6] + t->skipped_pushes;
            t->filtered = flt[i].cnt != nullptr;
            free_buckets(B, it);
            if (t->n_solid > t->out_cap) {
                st = tbl_convert(t);
                if (st) return st;
            }
        }
        finish_iso(B, it);
    }
    return FBK_OK;
}

// Records the finished table of an isolate in its result and frees what the table
// no longer needs.
void finish_iso(fbk_batch* B, BatchIso* it) {
    fbk_table* t = it->table;
    tbl_free_storage(t);  // the accumulator slots are not needed once the rows are converted
    it->res.n_keys = t->n_keys;
    it->res.n_solid = t->n_solid;
    it->res.digest = t->digest;
    it->res.pushes = t->pushes;
    it->res.table_capacity = t->cap;
    free_counting(B, it, B->p.keep_sketch != 0);
    dev_free(B->ctx, it->keep);
    it->keep = nullptr;
    it->res.state = 3;
    B->stats.isolates_done++;
}

// Phase B for isolates whose phase A is done, in sub-waves that fit the free pool
// memory; an isolate that does not fit even alone takes the single-isolate path.
fbk_status drain_b(fbk_batch* B, const std::vector<BatchIso*>& W) {
    fbk_ctx* ctx = B->ctx;
    const uint32_t max_wave = std::max<uint32_t>(1, std::min<uint32_t>(BATCH_MAX_ISO, B->p.max_wave ? B->p.max_wave : 64));
    size_t j = 0;
    fbk_status st = FBK_OK;
    while (j < W.size()) {
        const double h0 = now_ms();
        uint64_t free_b = 0, largest = 0;
        fbk_ctx_pool_free(ctx, &free_b, &largest);
        if (B->p.max_wave_bytes) free_b = std::min(free_b, B->p.max_wave_bytes);
        std::vector<BatchIso*> V;
        uint64_t bytes = 0;
        while (j < W.size() && V.size() < max_wave) {
            const PlanB q = plan_b(B, W[j]);
            if (!V.empty() && bytes + q.bytes + (64ULL << 20) > free_b) break;
            st = alloc_b(B, W[j], q);
            if (st) {
                // the pool is full or fragmented: run what fits, retry this isolate next
                release_b(B, W[j]);
                ctx->err.clear();
                if (!V.empty()) {
                    st = FBK_OK;
                    break;
                }
                st = fallback(B, W[j]);
                if (st) break;
                finish_iso(B, W[j]);
                ++j;
                continue;
            }
            bytes += q.bytes;
            V.push_back(W[j++]);
        }
        B->stats.ms_host += now_ms() - h0;
        if (st == FBK_OK && !V.empty()) st = phase_b(B, V);
        if (st) {
            for (BatchIso* it : W) {
                if (it->res.state == 3) continue;
                release_b(B, it);
                free_counting(B, it, false);
                it->res.state = -1;
                it->res.status = st;
            }
            return st;
        }
    }
    return FBK_OK;
}

fbk_status run_impl(fbk_batch* B) {
    fbk_ctx* ctx = B->ctx;
    CK(ctx, cudaSetDevice(ctx->device));
    // stage 1: estimates
    for (auto& up : B->isos) {
        BatchIso* it = up.get();
        if (it->res.state != 0) continue;
        CK(ctx, cudaEventRecord(B->ev[0], ctx->stream));
        fbk_status st = estimate_one(B, it);
        if (st) {
            it->res.state = -1;
            it->res.status = st;
            continue;
        }
        CK(ctx, cudaEventRecord(B->ev[1], ctx->stream));
        CK(ctx, cudaEventSynchronize(B->ev[1]));
        float t = 0.f;
        cudaEventElapsedTime(&t, B->ev[0], B->ev[1]);
        B->stats.ms_estimate += t;
    }
    std::vector<BatchIso*> todo;
    for (auto& up : B->isos)
        if (up->res.state == 1) todo.push_back(up.get());
    const uint32_t max_wave = std::max<uint32_t>(1, std::min<uint32_t>(BATCH_MAX_ISO, B->p.max_wave ? B->p.max_wave : 64));
    size_t next = 0;
    while (next < todo.size()) {
        // phase-A wave: isolates whose sketches and bitmaps fill at most half of the
        // free pool memory; the rest is left for phase-B tables and record buckets
        uint64_t free_b = 0, largest = 0;
        fbk_ctx_pool_free(ctx, &free_b, &largest);
        if (B->p.max_wave_bytes) free_b = std::min(free_b, B->p.max_wave_bytes);
        std::vector<BatchIso*> W;
        uint64_t used = 0;
        while (next < todo.size() && W.size() < max_wave) {
            const uint64_t need = phase_a_bytes(B, todo[next]);
            if (!W.empty() && (used + need) * 2 > free_b) break;
            W.push_back(todo[next++]);
            used += need;
        }
        const uint32_t wave_no = (uint32_t)B->stats.waves;
        for (BatchIso* it : W) it->res.wave = (int32_t)wave_no;
        fbk_status st = phase_a(B, W);
        if (st) {
            for (BatchIso* it : W) {
                free_counting(B, it, false);
                it->res.state = -1;
                it->res.status = st;
            }
            return st;
        }
        B->stats.waves++;
        st = drain_b(B, W);
        if (st) return st;
    }
    return FBK_OK;
}

}  // namespace

extern "C" {

FBK_API void fbk_subsample_policy_defaults(fbk_subsample_policy* p) {
    if (!p) return;
    std::memset(p, 0, sizeof(*p));
    p->depth = 120.0;
    p->threshold_ratio = 1.5;
}

// src/main.rs:76-180, branch for branch.
FBK_API fbk_status fbk_subsample_decide(const fbk_subsample_policy* p, const fbk_genome_estimate* e, double* factor,
                                        int32_t* reason) {
    if (!p || !e || !factor) return FBK_ERR_INVALID;
    if (!std::isfinite(p->threshold_ratio) || p->threshold_ratio < 1.0) return FBK_ERR_INVALID;
    const double trigger_mult = p->threshold_ratio;
    double f = 1.0;
    int32_t why;
    if (p->no_subsample) {
        why = 0;
    } else if (p->enable_auto_subsample) {
        if (p->has_genome_size) {
            if (p->genome_size == 0) {
                why = 1;
            } else {
                const double explicit_cov = (double)e->total_bases / (double)p->genome_size;
                const double trigger_cov = trigger_mult * p->depth;
                if (p->depth > 0.0 && explicit_cov > trigger_cov) {
                    f = std::min(1.0, std::max(0.01, p->depth / explicit_cov));
                    why = 2;
                } else {
                    why = 3;
                }
            }
        } else if (e->confidence == 0) {
            const double est_cov = e->estimated_cov;
            const double trigger_cov = trigger_mult * p->depth;
            if (p->depth > 0.0 && est_cov > trigger_cov) {
                f = std::min(1.0, std::max(0.01, p->depth / est_cov));
                why = 4;
            } else {
                why = 5;
            }
        } else if (e->confidence == 1) {
            why = 6;
        } else {
            why = 7;
        }
    } else if (p->has_genome_size) {
        why = 8;
    } else {
        why = 9;
    }
    *factor = f;
    if (reason) *reason = why;
    return FBK_OK;
}

FBK_API void fbk_batch_defaults(fbk_batch_params* p) {
    if (!p) return;
    std::memset(p, 0, sizeof(*p));
    p->k = 31;
    p->key_bits = 64;
    p->cms_log2_width = 22;
    p->counter_bits = 16;
    p->t_solid = 2;
    p->min_trans_cov = 3;
    p->use_graphs = 1;
    p->autotune = 1;
    p->max_wave = 64;
    p->est_max_pairs = 250000;
    fbk_subsample_policy_defaults(&p->policy);
}

FBK_API fbk_status fbk_batch_create(fbk_ctx* ctx, const fbk_batch_params* p, fbk_batch** out) {
    if (!ctx || !p || !out) return FBK_ERR_INVALID;
    *out = nullptr;
    const int nw = key_words(p->key_bits);
    if (!nw || p->k < 1 || p->k > key_k_max(p->key_bits)) return set_err(ctx, FBK_ERR_INVALID, "batch: k out of range for key_bits");
    if (p->cms_log2_width < 10 || p->cms_log2_width > 28) return set_err(ctx, FBK_ERR_INVALID, "batch: cms_log2_width out of range");
    if (p->counter_bits != 4 && p->counter_bits != 16) return set_err(ctx, FBK_ERR_INVALID, "batch: counter_bits must be 4 or 16");
    if (p->t_solid > 0xFFFF || p->min_trans_cov > 0xFFFF) return set_err(ctx, FBK_ERR_INVALID, "batch: thresholds must fit u16");
    if (p->max_wave > BATCH_MAX_ISO) return set_err(ctx, FBK_ERR_INVALID, "batch: max_wave above 256");
    if (!std::isfinite(p->policy.threshold_ratio) || p->policy.threshold_ratio < 1.0)
        return set_err(ctx, FBK_ERR_INVALID, "Invalid --subsample-threshold-ratio: must be a finite float >= 1.0");
    fbk_batch* B = new fbk_batch();
    B->ctx = ctx;
    B->p = *p;
    B->nw = nw;
    B->ladder = !p->keep_sketch && ctx->sketch_mode == 1 && p->t_solid >= 1 && p->t_solid <= LADDER_MAX_LEVELS &&
                p->t_solid <= cms_cap_of(p->counter_bits);
    B->pass1 = {ctx->block_pass1, ctx->grid_pass1, 4};
    B->solid = {ctx->block_pass2, ctx->grid_pass2, 4};
    B->emit = {ctx->block_pass2, ctx->grid_pass2, 0};
    B->upsert = {ctx->block_pass2, ctx->grid_pass2, 0};
    // whole rows per sweep while they fit the context's sweep size
    const uint64_t row_bytes = (1ULL << p->cms_log2_width) * 4;
    const int rows = ctx->sweep_bytes >= 4 * row_bytes ? 4 : ctx->sweep_bytes >= 2 * row_bytes ? 2 : 1;
    B->pass1.rows = B->solid.rows = rows;
    cudaSetDevice(ctx->device);
    if (cudaEventCreate(&B->ev[0]) != cudaSuccess || cudaEventCreate(&B->ev[1]) != cudaSuccess) {
        fbk_batch_release(B);
        return set_err(ctx, FBK_ERR_CUDA, "batch events");
    }
    *out = B;
    return FBK_OK;
}

FBK_API fbk_status fbk_batch_submit(fbk_batch* B, const fbk_arena_view bank[3], const fbk_arena_view* sample, uint64_t sample_pairs,
                                    const fbk_count_stats* stats, uint64_t* id) {
    if (!B || !bank || !sample || !stats) return FBK_ERR_INVALID;
    fbk_ctx* ctx = B->ctx;
    CK(ctx, cudaSetDevice(ctx->device));
    if (sample->n_seqs < 2 * sample_pairs) return set_err(ctx, FBK_ERR_INVALID, "sample holds fewer than 2*sample_pairs reads");
    auto it = std::make_unique<BatchIso>();
    it->id = B->isos.size();
    it->stats = *stats;
    it->sample_pairs = sample_pairs;
    it->sample_len.assign(sample->lengths, sample->lengths + 2 * sample_pairs);
    fbk_status st = bank_upload_impl(ctx, bank, 3, &it->bank);
    if (st) return st;
    if (it->bank->n_bases >= (1ULL << 31)) {
        fbk_bank_release(it->bank);
        return set_err(ctx, FBK_ERR_INVALID, "batch: an isolate of 2^31 bases or more takes the single-isolate path");
    }
    fbk_arena_view v = *sample;
    v.n_seqs = 2 * sample_pairs;
    v.pair_idx = nullptr;
    st = bank_upload_impl(ctx, &v, 1, &it->sample);
    if (st) {
        fbk_bank_release(it->bank);
        return st;
    }
    if (id) *id = it->id;
    B->isos.push_back(std::move(it));
    return FBK_OK;
}

FBK_API fbk_status fbk_batch_run(fbk_batch* B) {
    if (!B) return FBK_ERR_INVALID;
    return run_impl(B);
}

FBK_API fbk_status fbk_batch_get_result(const fbk_batch* B, uint64_t id, fbk_batch_result* out) {
    if (!B || !out || id >= B->isos.size()) return FBK_ERR_INVALID;
    *out = B->isos[id]->res;
    return FBK_OK;
}

FBK_API fbk_status fbk_batch_take_table(fbk_batch* B, uint64_t id, fbk_table** out) {
    if (!B || !out || id >= B->isos.size()) return FBK_ERR_INVALID;
    BatchIso* it = B->isos[id].get();
    if (it->res.state != 3 || !it->table) return set_err(B->ctx, FBK_ERR_INVALID, "batch: isolate has no table to take");
    *out = it->table;
    it->table = nullptr;
    return FBK_OK;
}

FBK_API fbk_status fbk_batch_drop(fbk_batch* B, uint64_t id) {
    if (!B || id >= B->isos.size()) return FBK_ERR_INVALID;
    free_iso(B, B->isos[id].get());
    return FBK_OK;
}

FBK_API fbk_status fbk_batch_get_stats(const fbk_batch* B, fbk_batch_stats* out) {
    if (!B || !out) return FBK_ERR_INVALID;
    *out = B->stats;
    out->pass1_block = B->pass1.block;
    out->pass1_grid = B->pass1.grid;
    out->pass1_rows = (B->ladder && B->pass1_single_used) ? 0 : B->pass1.rows;
    out->solid_block = B->solid.block;
    out->solid_grid = B->solid.grid;
    out->solid_rows = B->solid.rows;
    out->emit_block = B->emit.block;
    out->emit_grid = B->emit.grid;
    out->upsert_block = B->upsert.block;
    out->upsert_grid = B->upsert.grid;
    out->emit_form = B->emit_form ? B->emit_form : emit_form(B->ctx, B->nw);
    out->kernel_launches = B->ctx->launches;
    return FBK_OK;
}

FBK_API fbk_status fbk_batch_release(fbk_batch* B) {
    if (!B) return FBK_OK;
    for (auto& up : B->isos) free_iso(B, up.get());
    for (cudaEvent_t e : B->ev)
        if (e) cudaEventDestroy(e);
    if (B->h_stage) cudaFreeHost(B->h_stage);
    delete B;
    return FBK_OK;
}

}  // extern "C"

// ===========================================================================
// Serving: a request loop with continuous batching (see include/fbk.h)
// ===========================================================================
namespace {

struct Req {
    std::unique_ptr<BatchIso> iso;
    fbk_arena_view bank[3]{};
    fbk_arena_view sample{};
    uint64_t n_bases = 0, n_reads = 0, sample_bases = 0;
    int32_t state = 0;
    fbk_status status = FBK_OK;
    double t_submit = 0, t_admit = 0, t_done = 0;
    double t_uploaded = 0, t_estimated = 0, t_counted = 0;
    uint64_t reserved = 0;
};

// Device bytes a request may need before its pass 1 tells the exact table and
// bucket sizes: reads, sketch, bitmap, and records/table/rows from the k-mer
// occurrences (records <= windows; table keys taken as a quarter of the windows).
uint64_t request_estimate(const fbk_batch_params& p, int nw, uint64_t n_bases, uint64_t n_reads, uint64_t sample_bases) {
    const uint64_t reads = n_bases / 4 + n_reads * 16 + 8192;
    const uint64_t sample = sample_bases / 4 + 65536;
    const uint64_t a = (4ULL << p.cms_log2_width) * 4 + 4096 * 4 + n_bases / 8 + n_reads / 8 + 8192;
    const double w = (double)n_bases;
    const double b = w * (0.9 * 1.15 * 8.0 * record_format(p.k, nw).rw + 0.25 / 0.62 * (double)slot_bytes_of(nw) +
                          0.275 * (8.0 * nw + 3));
    return reads + sample + a + (uint64_t)b + (16ULL << 20);
}

uint64_t bank_bytes(const fbk_bank* b) { return b ? b->n_words * 8 + b->n_reads * 16 + 4096 : 0; }

void bank_free_done(fbk_ctx* ctx, fbk_bank*& b) {
    if (!b) return;
    dev_free(ctx, b->data);
    dev_free(ctx, b->off);
    dev_free(ctx, b->len);
    dev_free(ctx, b->pair_idx);
    delete b;
    b = nullptr;
}

// Frees a finished request's device state without waiting on any stream (its work
// has completed; the memory goes back to the shared pool).
void free_iso_done(fbk_ctx* ctx, BatchIso* it) {
    for (void** q : {(void**)&it->recs, (void**)&it->fill, (void**)&it->cnt, (void**)&it->lad, (void**)&it->hll12,
                     (void**)&it->bm, (void**)&it->keep}) {
        dev_free(ctx, *q);
        *q = nullptr;
    }
    if (it->table) {
        tbl_free_storage(it->table);
        tbl_free_out(it->table);
        delete it->table;
        it->table = nullptr;
    }
    bank_free_done(ctx, it->bank);
    bank_free_done(ctx, it->sample);
}

}  // namespace

struct fbk_server {
    fbk_ctx* ctx = nullptr;
    fbk_server_params p{};
    int nw = 1;
    std::vector<fbk_ctx*> wctx;
    std::vector<fbk_batch*> wb;
    std::vector<std::thread> th;
    std::mutex mu;
    std::condition_variable cv;
    std::deque<uint64_t> queued;
    std::deque<uint64_t> counted;
    std::map<uint64_t, std::unique_ptr<Req>> reqs;
    uint64_t next_id = 0, budget = 0, reserved = 0, in_flight = 0;
    bool stop = false;
    double t0 = 0;
    fbk_server_stats stats{};
    Shape pass1{256, 0, 4}, solid{256, 0, 4};
    bool tuned = false, tuning = false;
};

namespace {

double srv_ms(const fbk_server* S) { return now_ms() - S->t0; }

void reserve_set(fbk_server* S, Req* r, uint64_t bytes) {  // caller holds the lock
    S->reserved = S->reserved - r->reserved + bytes;
    r->reserved = bytes;
    S->stats.peak_reserved_bytes = std::max(S->stats.peak_reserved_bytes, S->reserved);
}

void fail_req(fbk_server* S, Req* r, fbk_status st) {  // caller holds the lock
    r->state = -1;
    r->status = st;
    r->t_done = srv_ms(S);
    S->stats.failed++;
    if (S->in_flight) S->in_flight--;
    reserve_set(S, r, 0);
}

// Uploads, estimates and phase A of a wave of newly admitted requests.
void job_admit(fbk_server* S, int w, const std::vector<Req*>& job) {
    fbk_batch* B = S->wb[w];
    fbk_ctx* ctx = B->ctx;
    std::vector<Req*> ok;
    for (Req* r : job) {
        BatchIso* it = r->iso.get();
        fbk_status st = bank_upload_impl(ctx, r->bank, 3, &it->bank);
        if (st == FBK_OK) {
            fbk_arena_view v = r->sample;
            v.n_seqs = 2 * it->sample_pairs;
            v.pair_idx = nullptr;
            st = bank_upload_impl(ctx, &v, 1, &it->sample);
        }
        if (st == FBK_OK) {
            std::lock_guard<std::mutex> lk(S->mu);
            r->state = 2;  // the host buffers are no longer read
            r->t_uploaded = srv_ms(S);
            S->cv.notify_all();
        }
        if (st == FBK_OK) {
            cudaEventRecord(B->ev[0], ctx->stream);
            st = estimate_one(B, it);
            if (st == FBK_OK) {
                float t_est = 0.f;
                cudaEventRecord(B->ev[1], ctx->stream);
                cudaEventSynchronize(B->ev[1]);
                cudaEventElapsedTime(&t_est, B->ev[0], B->ev[1]);
                B->stats.ms_estimate += t_est;
                r->t_estimated = srv_ms(S);
            }
        }
        if (st) {
            free_iso(B, it);
            std::lock_guard<std::mutex> lk(S->mu);
            fail_req(S, r, st);
            continue;
        }
        ok.push_back(r);
    }
    if (ok.empty()) return;
    std::vector<BatchIso*> W;
    for (Req* r : ok) W.push_back(r->iso.get());
    bool tune_here = false;
    {
        std::lock_guard<std::mutex> lk(S->mu);
        if (B->p.autotune && !S->tuned && !S->tuning) {
            S->tuning = true;
            tune_here = true;
            B->tuned = false;
        } else {
            B->pass1 = S->pass1;
            B->solid = S->solid;
            B->tuned = true;  // tuned already, or another worker is tuning
        }
    }
    const double a0 = now_ms();
    fbk_status st = phase_a(B, W);
    const double a1 = now_ms();
    std::lock_guard<std::mutex> lk(S->mu);
    if (tune_here) {
        S->tuning = false;
        if (B->tuned) {
            S->pass1 = B->pass1;
            S->solid = B->solid;
            S->tuned = true;
        }
    }
    S->stats.busy_ms += a1 - a0;
    if (st) {
        for (Req* r : ok) {
            free_iso(B, r->iso.get());
            fail_req(S, r, st);
        }
        S->cv.notify_all();
        return;
    }
    S->stats.waves_a++;
    S->stats.isolates_a += ok.size();
    for (Req* r : ok) {
        BatchIso* it = r->iso.get();
        r->state = 3;
        r->t_counted = srv_ms(S);
        reserve_set(S, r, bank_bytes(it->bank) + phase_a_bytes(B, it) + plan_b(B, it).bytes);
        S->counted.push_back(r->iso->id);
    }
    S->cv.notify_all();
}

// Phase B of a wave of counted requests; their tables stay on the device.
void job_tables(fbk_server* S, int w, const std::vector<Req*>& job) {
    fbk_batch* B = S->wb[w];
    std::vector<BatchIso*> W;
    for (Req* r : job) W.push_back(r->iso.get());
    const double b0 = now_ms();
    fbk_status st = drain_b(B, W);
    const double b1 = now_ms();
    std::lock_guard<std::mutex> lk(S->mu);
    S->stats.busy_ms += b1 - b0;
    S->stats.waves_b++;
    S->stats.isolates_b += job.size();
    for (Req* r : job) {
        BatchIso* it = r->iso.get();
        if (it->res.state != 3) {
            free_iso(B, it);
            fail_req(S, r, st ? st : it->res.status);
            continue;
        }
        bank_free_done(B->ctx, it->bank);  // the reads are consumed (the wave has completed)
        uint64_t keep = it->table ? it->table->out_cap * (8ULL * S->nw + 3) : 0;
        if (it->cnt) keep += (4ULL << B->p.cms_log2_width) * 4;
        reserve_set(S, r, keep);
        r->state = 4;
        r->t_done = srv_ms(S);
        S->stats.done++;
        if (S->in_flight) S->in_flight--;
    }
    S->cv.notify_all();
}

void worker_main(fbk_server* S, int w) {
    cudaSetDevice(S->ctx->device);
    const uint32_t max_wave = std::max<uint32_t>(1, std::min<uint32_t>(BATCH_MAX_ISO, S->p.batch.max_wave ? S->p.batch.max_wave : 64));
    std::unique_lock<std::mutex> lk(S->mu);
    for (;;) {
        std::vector<Req*> job;
        int kind = 0;
        if (!S->counted.empty()) {
            kind = 2;
            while (!S->counted.empty() && job.size() < max_wave) {
                job.push_back(S->reqs[S->counted.front()].get());
                S->counted.pop_front();
            }
        } else if (!S->queued.empty() && !S->stop) {
            kind = 1;
            while (!S->queued.empty() && job.size() < max_wave) {
                Req* r = S->reqs[S->queued.front()].get();
                const uint64_t est = r->reserved;  // the estimate, reserved on admission
                const bool fits = S->reserved + est <= S->budget;
                // first come, first served; a request alone always runs
                if (!fits && !(S->in_flight == 0 && job.empty())) break;
                S->queued.pop_front();
                r->state = 1;
                r->t_admit = srv_ms(S);
                S->reserved += est;
                S->stats.peak_reserved_bytes = std::max(S->stats.peak_reserved_bytes, S->reserved);
                S->in_flight++;
                S->stats.peak_in_flight = std::max<uint64_t>(S->stats.peak_in_flight, S->in_flight);
                job.push_back(r);
            }
        }
        if (job.empty()) {
            if (S->stop && S->counted.empty()) break;
            S->cv.wait_for(lk, std::chrono::milliseconds(20));
            continue;
        }
        lk.unlock();
        if (kind == 1) job_admit(S, w, job);
        else job_tables(S, w, job);
        lk.lock();
    }
}

}  // namespace

extern "C" {

FBK_API void fbk_server_defaults(fbk_server_params* p) {
    if (!p) return;
    std::memset(p, 0, sizeof(*p));
    fbk_batch_defaults(&p->batch);
    p->batch.policy.enable_auto_subsample = 1;
    p->batch.policy.depth = 110.0;
    p->batch.policy.threshold_ratio = 150.0 / 110.0;
    p->workers = 2;
}

FBK_API fbk_status fbk_server_create(fbk_ctx* ctx, const fbk_server_params* p, fbk_server** out) {
    if (!ctx || !p || !out) return FBK_ERR_INVALID;
    *out = nullptr;
    if (p->workers < 1 || p->workers > 8) return set_err(ctx, FBK_ERR_INVALID, "server: 1 to 8 workers");
    fbk_server* S = new fbk_server();
    S->ctx = ctx;
    S->p = *p;
    S->nw = key_words(p->batch.key_bits);
    S->t0 = now_ms();
    fbk_status st = FBK_OK;
    for (uint32_t w = 0; w < p->workers && st == FBK_OK; ++w) {
        fbk_ctx* c = nullptr;
        st = fbk_ctx_fork(ctx, &c);
        if (st) break;
        S->wctx.push_back(c);
        fbk_batch* B = nullptr;
        st = fbk_batch_create(c, &p->batch, &B);
        if (st) {
            ctx->err = c->err;
            break;
        }
        S->wb.push_back(B);
    }
    if (st) {
        fbk_server_destroy(S);
        return st;
    }
    S->pass1 = S->wb[0]->pass1;
    S->solid = S->wb[0]->solid;
    uint64_t budget = p->budget_bytes;
    if (!budget) {
        uint64_t used = 0, size = 0, free_b = 0, largest = 0;
        fbk_ctx_mem_info(ctx, &used, &size);
        fbk_ctx_pool_free(ctx, &free_b, &largest);
        budget = (uint64_t)(0.9 * (double)(size ? size : free_b));
    }
    // each worker keeps room for the estimator's scratch and its wave descriptors
    const uint64_t scratch = (uint64_t)p->workers * (512ULL << 20);
    S->budget = budget > scratch ? budget - scratch : budget / 2;
    S->stats.budget_bytes = S->budget;
    for (uint32_t w = 0; w < p->workers; ++w) S->th.emplace_back(worker_main, S, (int)w);
    *out = S;
    return FBK_OK;
}

FBK_API fbk_status fbk_server_submit(fbk_server* S, const fbk_arena_view bank[3], const fbk_arena_view* sample,
                                     uint64_t sample_pairs, const fbk_count_stats* stats, uint64_t* id) {
    if (!S || !bank || !sample || !stats) return FBK_ERR_INVALID;
    if (sample->n_seqs < 2 * sample_pairs) return FBK_ERR_INVALID;
    auto r = std::make_unique<Req>();
    r->iso = std::make_unique<BatchIso>();
    r->iso->stats = *stats;
    r->iso->sample_pairs = sample_pairs;
    r->iso->sample_len.assign(sample->lengths, sample->lengths + 2 * sample_pairs);
    for (int a = 0; a < 3; ++a) r->bank[a] = bank[a];
    {
        ArenaScan sc;
        scan_arenas(bank, 3, sc);
        r->n_bases = sc.n_bases;
        r->n_reads = sc.n_reads;
    }
    if (r->n_bases >= (1ULL << 31)) return FBK_ERR_INVALID;
    r->sample = *sample;
    for (uint64_t i = 0; i < 2 * sample_pairs; ++i) r->sample_bases += sample->lengths[i];
    std::lock_guard<std::mutex> lk(S->mu);
    if (S->stop) return FBK_ERR_BUSY;
    const uint64_t i = S->next_id++;
    r->iso->id = i;
    r->t_submit = srv_ms(S);
    r->reserved = request_estimate(S->p.batch, S->nw, r->n_bases, r->n_reads, r->sample_bases);
    S->reqs[i] = std::move(r);
    S->queued.push_back(i);
    S->stats.submitted++;
    if (id) *id = i;
    S->cv.notify_all();
    return FBK_OK;
}

static void request_info(const fbk_server* S, const Req* r, fbk_request_info* out) {
    out->state = r->state;
    out->status = r->status;
    out->t_submit_ms = r->t_submit;
    out->t_admit_ms = r->t_admit;
    out->t_done_ms = r->t_done;
    out->t_uploaded_ms = r->t_uploaded;
    out->t_estimated_ms = r->t_estimated;
    out->t_counted_ms = r->t_counted;
    out->reserved_bytes = r->state == 0 ? 0 : r->reserved;
    out->result = r->iso->res;
    (void)S;
}

FBK_API fbk_status fbk_server_poll(fbk_server* S, uint64_t id, fbk_request_info* out) {
    if (!S || !out) return FBK_ERR_INVALID;
    std::lock_guard<std::mutex> lk(S->mu);
    auto f = S->reqs.find(id);
    if (f == S->reqs.end()) return FBK_ERR_INVALID;
    request_info(S, f->second.get(), out);
    return FBK_OK;
}

FBK_API fbk_status fbk_server_wait(fbk_server* S, uint64_t id, double timeout_ms, fbk_request_info* out) {
    if (!S) return FBK_ERR_INVALID;
    std::unique_lock<std::mutex> lk(S->mu);
    auto f = S->reqs.find(id);
    if (f == S->reqs.end()) return FBK_ERR_INVALID;
    Req* r = f->second.get();
    // NaN or negative: no wait; infinite or huge: 1e12 ms (the microsecond count stays in int64)
    const double tmo = timeout_ms > 0.0 ? std::min(timeout_ms, 1e12) : 0.0;
    const auto until = std::chrono::steady_clock::now() + std::chrono::microseconds((int64_t)(tmo * 1000.0));
    while (r->state >= 0 && r->state < 4) {
        if (S->cv.wait_until(lk, until) == std::cv_status::timeout && r->state >= 0 && r->state < 4) {
            if (out) request_info(S, r, out);
            return FBK_ERR_NOT_READY;
        }
    }
    if (out) request_info(S, r, out);
    return r->state < 0 ? (fbk_status)r->status : FBK_OK;
}

FBK_API fbk_status fbk_server_take_table(fbk_server* S, uint64_t id, fbk_table** out) {
    if (!S || !out) return FBK_ERR_INVALID;
    std::lock_guard<std::mutex> lk(S->mu);
    auto f = S->reqs.find(id);
    if (f == S->reqs.end() || f->second->state != 4) return set_err(S->ctx, FBK_ERR_INVALID, "server: request has no table to take");
    Req* r = f->second.get();
    BatchIso* it = r->iso.get();
    fbk_table* t = it->table;
    it->table = nullptr;
    t->ctx = S->ctx;  // the table lives in the shared pool; the caller's context releases it
    free_iso_done(S->ctx, it);
    reserve_set(S, r, 0);
    r->state = 5;
    *out = t;
    return FBK_OK;
}

FBK_API fbk_status fbk_server_release_request(fbk_server* S, uint64_t id) {
    if (!S) return FBK_ERR_INVALID;
    std::lock_guard<std::mutex> lk(S->mu);
    auto f = S->reqs.find(id);
    if (f == S->reqs.end()) return FBK_ERR_INVALID;
    Req* r = f->second.get();
    if (r->state != 4 && r->state != -1 && r->state != 5) return set_err(S->ctx, FBK_ERR_BUSY, "server: request still in flight");
    free_iso_done(S->ctx, r->iso.get());
    reserve_set(S, r, 0);
    S->reqs.erase(f);
    S->cv.notify_all();
    return FBK_OK;
}

FBK_API fbk_status fbk_server_get_stats(fbk_server* S, fbk_server_stats* out) {
    if (!S || !out) return FBK_ERR_INVALID;
    std::lock_guard<std::mutex> lk(S->mu);
    *out = S->stats;
    out->reserved_bytes = S->reserved;
    out->ms_estimate = out->ms_phase_a = out->ms_phase_b = 0.0;
    for (const fbk_batch* B : S->wb) {
        out->ms_estimate += B->stats.ms_estimate;
        out->ms_phase_a += B->stats.ms_phase_a;
        out->ms_phase_b += B->stats.ms_phase_b;
    }
    return FBK_OK;
}

FBK_API fbk_status fbk_server_destroy(fbk_server* S) {
    if (!S) return FBK_OK;
    {
        std::lock_guard<std::mutex> lk(S->mu);
        S->stop = true;
        while (!S->queued.empty()) {
            Req* r = S->reqs[S->queued.front()].get();
            S->queued.pop_front();
            r->state = -1;
            r->status = FBK_ERR_BUSY;
            S->stats.failed++;
        }
        S->cv.notify_all();
    }
    for (auto& t : S->th) t.join();
    for (auto& kv : S->reqs)
        if (!S->wb.empty()) free_iso(S->wb[0], kv.second->iso.get());
    S->reqs.clear();
    for (fbk_batch* B : S->wb) fbk_batch_release(B);
    for (fbk_ctx* c : S->wctx) fbk_ctx_destroy(c);
    delete S;
    return FBK_OK;
}

}  // extern "C"
