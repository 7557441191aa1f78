// fbk_api.cu — host side of the C ABI: contexts, device pool, bank upload, and the
// CountMinSketch / HyperLogLog / solid-table objects with their build passes.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "fbk_device.cuh"
#include "fbk_internal.h"
#include "host/fbk_workers.h"

using namespace fbk;

// ===========================================================================
// errors, pool, timing
// ===========================================================================
namespace fbk {

fbk_status set_err(fbk_ctx* ctx, fbk_status st, const std::string& msg) {
    if (ctx) ctx->err = msg;
    return st;
}
fbk_status cuda_err(fbk_ctx* ctx, cudaError_t e, const char* what) {
    std::string m = std::string(what) + ": " + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ")";
    return set_err(ctx, e == cudaErrorMemoryAllocation ? FBK_ERR_OOM : FBK_ERR_CUDA, m);
}

bool DevicePool::init(uint64_t bytes, std::string& err) {
    bytes = (bytes + 255) & ~255ULL;
    cudaError_t e = cudaMalloc((void**)&base_, bytes);
    if (e != cudaSuccess) {
        err = std::string("pool cudaMalloc: ") + cudaGetErrorString(e);
        base_ = nullptr;
        return false;
    }
    size_ = bytes;
    free_.clear();
    live_.clear();
    free_[0] = bytes;
    used_bytes_ = 0;
    return true;
}
void DevicePool::release() {
    if (base_) cudaFree(base_);
    base_ = nullptr;
    size_ = used_bytes_ = 0;
    free_.clear();
    live_.clear();
}
void* DevicePool::alloc(uint64_t bytes) {
    std::lock_guard<std::mutex> g(mu_);
    bytes = std::max<uint64_t>(256, (bytes + 255) & ~255ULL);
    for (auto it = free_.begin(); it != free_.end(); ++it) {
        if (it->second >= bytes) {
            uint64_t off = it->first, sz = it->second;
            free_.erase(it);
            if (sz > bytes) free_[off + bytes] = sz - bytes;
            live_[off] = bytes;
            used_bytes_ += bytes;
            return base_ + off;
        }
    }
    return nullptr;
}
void DevicePool::free(void* p) {
    if (!p) return;
    std::lock_guard<std::mutex> g(mu_);
    uint64_t off = (uint64_t)((char*)p - base_);
    auto it = live_.find(off);
    if (it == live_.end()) return;
    uint64_t sz = it->second;
    live_.erase(it);
    used_bytes_ -= sz;
    auto nx = free_.lower_bound(off);
    if (nx != free_.end() && nx->first == off + sz) {
        sz += nx->second;
        free_.erase(nx);
    }
    auto pv = free_.lower_bound(off);
    if (pv != free_.begin()) {
        --pv;
        if (pv->first + pv->second == off) {
            pv->second += sz;
            return;
        }
    }
    free_[off] = sz;
}
uint64_t DevicePool::largest_free() const {
    std::lock_guard<std::mutex> g(mu_);
    uint64_t m = 0;
    for (auto& f : free_) m = std::max(m, f.second);
    return m;
}

void* dev_alloc(fbk_ctx* ctx, uint64_t bytes) {
    if (bytes == 0) bytes = 256;
    if (ctx->pool && ctx->pool->active()) return ctx->pool->alloc(bytes);
    void* p = nullptr;
    if (cudaMalloc(&p, bytes) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return p;
}
void dev_free(fbk_ctx* ctx, void* p) {
    if (!p) return;
    if (ctx->pool && ctx->pool->active()) ctx->pool->free(p);
    else cudaFree(p);
}

Launch launch_cfg(fbk_ctx* ctx, int block, int grid) {
    Launch L;
    L.block = block;
    L.grid = grid > 0 ? grid : ctx->num_sms * 4;
    L.stream = ctx->stream;
    L.sms = ctx->num_sms;
    return L;
}
Launch launch_cfg_persistent(fbk_ctx* ctx, int block, int grid) {
    Launch L = launch_cfg(ctx, block, grid);
    L.grid = grid;
    return L;
}

void time_begin(fbk_ctx* ctx, const char* name, TimedLaunch& t) {
    ctx->launches++;
    t.name = name;
    t.a = t.b = nullptr;
    if (!ctx->timing || ctx->capturing) return;
    for (cudaEvent_t* e : {&t.a, &t.b}) {
        if (!ctx->free_events.empty()) {
            *e = ctx->free_events.back();
            ctx->free_events.pop_back();
        } else {
            cudaEventCreate(e);
        }
    }
    cudaEventRecord(t.a, ctx->stream);
}
void time_end(fbk_ctx* ctx, TimedLaunch& t) {
    if (!ctx->timing || !t.a) return;
    cudaEventRecord(t.b, ctx->stream);
    ctx->pending.push_back(t);
}

static void collect_timing(fbk_ctx* ctx) {
    if (ctx->pending.empty()) return;
    cudaStreamSynchronize(ctx->stream);
    for (auto& t : ctx->pending) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, t.a, t.b);
        auto& acc = ctx->timed[t.name];
        acc.first += ms;
        acc.second += 1;
        ctx->free_events.push_back(t.a);
        ctx->free_events.push_back(t.b);
    }
    ctx->pending.clear();
}

fbk_status ctx_check_status(fbk_ctx* ctx, uint32_t* bits) {
    uint32_t* h = (uint32_t*)ctx->h_pinned;
    cudaError_t e = cudaMemcpyAsync(h, ctx->d_status, sizeof(uint32_t), cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return cuda_err(ctx, e, "status readback");
    *bits = h[0];
    return FBK_OK;
}

BankDev bank_view(const fbk_bank* b, uint64_t r_begin, uint64_t r_end, const uint64_t* keep_bits) {
    BankDev v;
    v.data = b->data;
    v.off = b->off;
    v.len = b->len;
    v.pair_idx = b->pair_idx;
    v.keep_bits = keep_bits;
    v.r_begin = r_begin;
    v.r_end = r_end;
    return v;
}

uint64_t f64_to_u64_sat(double x) {
    if (!(x > 0.0)) return 0;
    if (x >= 18446744073709551616.0) return UINT64_MAX;
    return (uint64_t)x;
}

double hll_estimate_from_sum(double sum, uint64_t zeros, uint32_t p) {
    const double m = (double)(1ULL << p);
    const double alpha_m = 0.7213 / (1.0 + 1.079 / m);
    const double raw = alpha_m * m * m / sum;
    if (raw <= 2.5 * m) {
        if (zeros > 0) return m * std::log(m / (double)zeros);
        return raw;
    } else if (raw <= (1.0 / 30.0) * 18446744073709551616.0) {
        return raw;
    }
    const double two64 = 18446744073709551616.0;
    return -two64 * std::log(1.0 - raw / two64);
}

}  // namespace fbk


// ===========================================================================
// status, context
// ===========================================================================
extern "C" {

FBK_API const char* fbk_status_str(fbk_status s) {
    switch (s) {
        case FBK_OK: return "ok";
        case FBK_ERR_INVALID: return "invalid argument";
        case FBK_ERR_CUDA: return "cuda error";
        case FBK_ERR_OOM: return "out of device memory";
        case FBK_ERR_TABLE_FULL: return "solid table full";
        case FBK_ERR_TIMEOUT: return "device wait timed out";
        case FBK_ERR_IO: return "i/o error";
        case FBK_ERR_FORMAT: return "malformed input";
        case FBK_ERR_EMPTY: return "no valid read pairs";
        case FBK_ERR_BUSY: return "busy";
        case FBK_ERR_NOT_READY: return "not ready";
        case FBK_ERR_NO_DEVICE: return "no cuda device";
        default: return "unknown status";
    }
}

FBK_API const char* fbk_version(void) { return "fastbact_gb300 0.1.0 (sm_103a)"; }

FBK_API fbk_status fbk_ctx_create(int device, uint64_t pool_bytes, fbk_ctx** out) {
    if (!out) return FBK_ERR_INVALID;
    *out = nullptr;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
        cudaGetLastError();
        return FBK_ERR_NO_DEVICE;
    }
    if (device < 0 || device >= n) return FBK_ERR_INVALID;
    fbk_ctx* c = new fbk_ctx();
    c->device = device;
    cudaError_t e = cudaSetDevice(device);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMalloc((void**)&c->d_status, 64);
    if (e == cudaSuccess) e = cudaMalloc((void**)&c->d_counts, 8 * sizeof(unsigned long long));
    if (e == cudaSuccess) e = cudaMallocHost(&c->h_pinned, 65536);
    if (e == cudaSuccess) e = cudaMemset(c->d_status, 0, 64);
    if (e != cudaSuccess) {
        fbk_ctx_destroy(c);
        return FBK_ERR_CUDA;
    }
    c->pool = std::make_shared<DevicePool>();
    if (pool_bytes > 0 && !c->pool->init(pool_bytes, c->err)) {
        fbk_ctx_destroy(c);
        return FBK_ERR_OOM;
    }
    *out = c;
    return FBK_OK;
}

FBK_API fbk_status fbk_ctx_destroy(fbk_ctx* c) {
    if (!c) return FBK_OK;
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    for (auto& t : c->pending) {
        cudaEventDestroy(t.a);
        cudaEventDestroy(t.b);
    }
    for (auto e : c->free_events) cudaEventDestroy(e);
    for (auto e : c->markers)
        if (e) cudaEventDestroy(e);
    c->pool.reset();  // the pool memory goes when its last context does
    if (c->d_status) cudaFree(c->d_status);
    if (c->d_counts) cudaFree(c->d_counts);
    if (c->h_pinned) cudaFreeHost(c->h_pinned);
    for (int i = 0; i < 2; ++i) {
        if (c->h_stage[i]) cudaFreeHost(c->h_stage[i]);
        if (c->stage_ev[i]) cudaEventDestroy(c->stage_ev[i]);
    }
    if (c->copy_stream) {
        cudaStreamSynchronize(c->copy_stream);
        cudaStreamDestroy(c->copy_stream);
    }
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
    return FBK_OK;
}

FBK_API fbk_status fbk_ctx_fork(fbk_ctx* parent, fbk_ctx** out) {
    if (!parent || !out) return FBK_ERR_INVALID;
    *out = nullptr;
    fbk_ctx* c = new fbk_ctx();
    c->device = parent->device;
    c->num_sms = parent->num_sms;
    c->pool = parent->pool;
    c->sweep_bytes = parent->sweep_bytes;
    c->bucket_bytes = parent->bucket_bytes;
    c->stripes = parent->stripes;
    c->load_factor = parent->load_factor;
    c->pass2_mode = parent->pass2_mode;
    c->record_factor = parent->record_factor;
    c->block_pass1 = parent->block_pass1;
    c->grid_pass1 = parent->grid_pass1;
    c->block_pass2 = parent->block_pass2;
    c->block_emit = parent->block_emit;
    c->grid_pass2 = parent->grid_pass2;
    c->block_misc = parent->block_misc;
    c->sketch_mode = parent->sketch_mode;
    c->ladder_ilp = parent->ladder_ilp;
    c->emit_lookahead = parent->emit_lookahead;
    c->upsert_queue = parent->upsert_queue;
    c->batch_pass1 = parent->batch_pass1;
    c->filter_sizing = parent->filter_sizing;
    c->filter_load = parent->filter_load;
    c->acc_filter = parent->acc_filter;
    c->upsert_all = parent->upsert_all;
    cudaError_t e = cudaSetDevice(c->device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMalloc((void**)&c->d_status, 64);
    if (e == cudaSuccess) e = cudaMalloc((void**)&c->d_counts, 8 * sizeof(unsigned long long));
    if (e == cudaSuccess) e = cudaMallocHost(&c->h_pinned, 65536);
    if (e == cudaSuccess) e = cudaMemset(c->d_status, 0, 64);
    if (e != cudaSuccess) {
        fbk_ctx_destroy(c);
        return cuda_err(parent, e, "fbk_ctx_fork");
    }
    *out = c;
    return FBK_OK;
}

FBK_API fbk_status fbk_ctx_pool_free(const fbk_ctx* ctx, uint64_t* free_bytes, uint64_t* largest_block) {
    if (!ctx || !free_bytes) return FBK_ERR_INVALID;
    if (ctx->pool && ctx->pool->active()) {
        *free_bytes = ctx->pool->free_bytes();
        if (largest_block) *largest_block = ctx->pool->largest_free();
    } else {
        size_t f = 0, t = 0;
        cudaSetDevice(ctx->device);
        cudaMemGetInfo(&f, &t);
        *free_bytes = f;
        if (largest_block) *largest_block = f;
    }
    return FBK_OK;
}

FBK_API fbk_status fbk_last_error(const fbk_ctx* ctx, char* buf, size_t len) {
    if (!ctx || !buf || len == 0) return FBK_ERR_INVALID;
    snprintf(buf, len, "%s", ctx->err.c_str());
    return FBK_OK;
}

FBK_API fbk_status fbk_ctx_sync(fbk_ctx* ctx) {
    if (!ctx) return FBK_ERR_INVALID;
    CK(ctx, cudaStreamSynchronize(ctx->stream));
    return FBK_OK;
}

FBK_API fbk_status fbk_ctx_set_timing(fbk_ctx* ctx, int enable) {
    if (!ctx) return FBK_ERR_INVALID;
    ctx->timing = enable != 0;
    return FBK_OK;
}

FBK_API fbk_status fbk_ctx_timing(fbk_ctx* ctx, const char* prefix, double* ms, uint64_t* launches) {
    if (!ctx || !prefix || !ms || !launches) return FBK_ERR_INVALID;
    collect_timing(ctx);
    double t = 0;
    uint64_t n = 0;
    size_t pl = strlen(prefix);
    for (auto& kv : ctx->timed)
        if (kv.first.compare(0, pl, prefix) == 0) {
            t += kv.second.first;
            n += kv.second.second;
        }
    *ms = t;
    *launches = n;
    return FBK_OK;
}

FBK_API fbk_status fbk_ctx_timing_reset(fbk_ctx* ctx) {
    if (!ctx) return FBK_ERR_INVALID;
    collect_timing(ctx);
    ctx->timed.clear();
    return FBK_OK;
}

FBK_API fbk_status fbk_ctx_event_record(fbk_ctx* ctx, int slot) {
    if (!ctx || slot < 0 || slot >= 16) return FBK_ERR_INVALID;
    if (!ctx->markers[slot]) CK(ctx, cudaEventCreate(&ctx->markers[slot]));
    CK(ctx, cudaEventRecord(ctx->markers[slot], ctx->stream));
    return FBK_OK;
}

FBK_API fbk_status fbk_ctx_event_elapsed(fbk_ctx* ctx, int a, int b, double* ms) {
    if (!ctx || !ms || a < 0 || a >= 16 || b < 0 || b >= 16 || !ctx->markers[a] || !ctx->markers[b]) return FBK_ERR_INVALID;
    CK(ctx, cudaEventSynchronize(ctx->markers[b]));
    float f = 0.f;
    CK(ctx, cudaEventElapsedTime(&f, ctx->markers[a], ctx->markers[b]));
    *ms = f;
    return FBK_OK;
}

FBK_API fbk_status fbk_ctx_set_tuning(fbk_ctx* ctx, const char* name, double v) {
    if (!ctx || !name) return FBK_ERR_INVALID;
    const std::string n(name);
    if (n == "sweep_bytes" && v >= 4096) ctx->sweep_bytes = (uint64_t)v;
    else if (n == "bucket_bytes" && v >= 4096) ctx->bucket_bytes = (uint64_t)v;
    else if (n == "stripes" && v >= 1 && v <= 256) ctx->stripes = (uint32_t)v;
    else if (n == "load_factor" && v >= 0.1 && v <= 0.9) ctx->load_factor = v;
    else if (n == "pass2_mode" && (v == 0 || v == 1)) ctx->pass2_mode = (int)v;
    else if (n == "record_factor" && v > 0 && v <= 16) ctx->record_factor = v;
    else if (n == "sketch_mode" && (v == 0 || v == 1)) ctx->sketch_mode = (int)v;
    else if (n == "ladder_ilp" && v >= 0 && v <= 5 && v == (int)v) ctx->ladder_ilp = (int)v;
    else if (n == "emit_lookahead" && v >= 0 && v <= 5 && v == (int)v) ctx->emit_lookahead = (int)v;
    else if (n == "upsert_queue" && (v == 0 || v == 1 || v == 2)) ctx->upsert_queue = (int)v;
    else if (n == "batch_pass1" && (v == 0 || v == 1 || v == 2)) ctx->batch_pass1 = (int)v;
    else if (n == "filter_sizing" && (v == 0 || v == 1)) ctx->filter_sizing = (int)v;
    else if (n == "filter_load" && v >= 0.02 && v <= 0.9) ctx->filter_load = v;
    else if (n == "acc_filter" && (v == 0 || v == 1 || v == 2)) ctx->acc_filter = (int)v;
    else if (n == "upsert_all" && (v == 0 || v == 1 || v == 2)) ctx->upsert_all = (int)v;
    // the pass kernels are compiled for blocks of at most 256 threads
    else if (n == "block_pass1" && v >= 32 && v <= 256 && ((int)v % 32) == 0) ctx->block_pass1 = (int)v;
    else if (n == "grid_pass1" && v >= 0) ctx->grid_pass1 = (int)v;
    else if (n == "block_pass2" && v >= 32 && v <= 256 && ((int)v % 32) == 0) ctx->block_pass2 = (int)v;
    else if (n == "block_emit" && v >= 32 && v <= 256 && ((int)v % 32) == 0) ctx->block_emit = (int)v;
    else if (n == "grid_pass2" && v >= 0) ctx->grid_pass2 = (int)v;
    else return set_err(ctx, FBK_ERR_INVALID, "unknown tuning name or value out of range: " + n);
    return FBK_OK;
}

FBK_API fbk_status fbk_ctx_get_tuning(const fbk_ctx* ctx, const char* name, double* v) {
    if (!ctx || !name || !v) return FBK_ERR_INVALID;
    const std::string n(name);
    if (n == "sweep_bytes") *v = (double)ctx->sweep_bytes;
    else if (n == "bucket_bytes") *v = (double)ctx->bucket_bytes;
    else if (n == "stripes") *v = ctx->stripes;
    else if (n == "load_factor") *v = ctx->load_factor;
    else if (n == "pass2_mode") *v = ctx->pass2_mode;
    else if (n == "record_factor") *v = ctx->record_factor;
    else if (n == "sketch_mode") *v = ctx->sketch_mode;
    else if (n == "ladder_ilp") *v = ctx->ladder_ilp;
    else if (n == "emit_lookahead") *v = ctx->emit_lookahead;
    else if (n == "upsert_queue") *v = ctx->upsert_queue;
    else if (n == "batch_pass1") *v = ctx->batch_pass1;
    else if (n == "filter_sizing") *v = ctx->filter_sizing;
    else if (n == "filter_load") *v = ctx->filter_load;
    else if (n == "acc_filter") *v = ctx->acc_filter;
    else if (n == "upsert_all") *v = ctx->upsert_all;
    else if (n == "block_pass1") *v = ctx->block_pass1;
    else if (n == "grid_pass1") *v = ctx->grid_pass1;
    else if (n == "block_pass2") *v = ctx->block_pass2;
    else if (n == "block_emit") *v = ctx->block_emit;
    else if (n == "grid_pass2") *v = ctx->grid_pass2;
    else return FBK_ERR_INVALID;
    return FBK_OK;
}

FBK_API fbk_status fbk_ctx_launch_count(const fbk_ctx* ctx, uint64_t* n) {
    if (!ctx || !n) return FBK_ERR_INVALID;
    *n = ctx->launches;
    return FBK_OK;
}

FBK_API fbk_status fbk_ctx_mem_info(const fbk_ctx* ctx, uint64_t* used, uint64_t* size) {
    if (!ctx || !used || !size) return FBK_ERR_INVALID;
    *used = ctx->pool ? ctx->pool->used() : 0;
    *size = ctx->pool ? ctx->pool->size() : 0;
    return FBK_OK;
}

}  // extern "C"

// ===========================================================================
// read bank
// ===========================================================================
namespace fbk {

static constexpr size_t STAGE_BYTES = 16u << 20;  // one staging slot
static constexpr size_t STAGE_MIN = 4u << 20;     // smaller pageable copies go direct
static constexpr size_t STAGE_PIECE = 1u << 20;   // host copy unit of the worker pool

static bool host_page_locked(const void* p) {
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return at.type == cudaMemoryTypeHost;
}

static cudaError_t stage_ready(fbk_ctx* ctx) {
    if (ctx->h_stage[0]) return cudaSuccess;
    cudaError_t e = cudaSuccess;
    for (int i = 0; i < 2 && e == cudaSuccess; ++i) {
        e = cudaMallocHost(&ctx->h_stage[i], STAGE_BYTES);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ctx->stage_ev[i], cudaEventDisableTiming);
    }
    return e;
}

static void pool_copy(void* dst, const void* src, size_t n) {
    host_parallel_for((n + STAGE_PIECE - 1) / STAGE_PIECE, [&](uint64_t i, unsigned) {
        const size_t o = i * STAGE_PIECE;
        std::memcpy((char*)dst + o, (const char*)src + o, std::min(STAGE_PIECE, n - o));
    });
}

cudaError_t copy_h2d(fbk_ctx* ctx, void* dst, const void* src, size_t bytes) {
    if (bytes == 0) return cudaSuccess;
    if (bytes < STAGE_MIN || host_page_locked(src))
        return cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, ctx->stream);
    cudaError_t e = stage_ready(ctx);
    for (size_t done = 0; e == cudaSuccess && done < bytes;) {
        const int slot = (int)((done / STAGE_BYTES) & 1);
        const size_t n = std::min(STAGE_BYTES, bytes - done);
        e = cudaEventSynchronize(ctx->stage_ev[slot]);  // the slot's previous DMA has finished
        if (e != cudaSuccess) break;
        pool_copy(ctx->h_stage[slot], (const char*)src + done, n);
        e = cudaMemcpyAsync((char*)dst + done, ctx->h_stage[slot], n, cudaMemcpyHostToDevice, ctx->stream);
        if (e == cudaSuccess) e = cudaEventRecord(ctx->stage_ev[slot], ctx->stream);
        done += n;
    }
    return e;
}

cudaError_t copy_d2h(fbk_ctx* ctx, void* dst, const void* src, size_t bytes) {
    if (bytes == 0) return cudaSuccess;
    if (bytes < STAGE_MIN || host_page_locked(dst)) {
        cudaError_t e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, ctx->stream);
        return e == cudaSuccess ? cudaStreamSynchronize(ctx->stream) : e;
    }
    cudaError_t e = stage_ready(ctx);
    const size_t nc = (bytes + STAGE_BYTES - 1) / STAGE_BYTES;
    auto issue = [&](size_t c) {
        const size_t o = c * STAGE_BYTES, n = std::min(STAGE_BYTES, bytes - o);
        cudaError_t x = cudaMemcpyAsync(ctx->h_stage[c & 1], (const char*)src + o, n, cudaMemcpyDeviceToHost, ctx->stream);
        return x == cudaSuccess ? cudaEventRecord(ctx->stage_ev[c & 1], ctx->stream) : x;
    };
    if (e == cudaSuccess) e = issue(0);
    for (size_t c = 0; e == cudaSuccess && c < nc; ++c) {
        // chunk c + 1 lands in the other slot, whose previous contents were copied out
        // in the last iteration, while chunk c is copied out of this one
        if (c + 1 < nc) e = issue(c + 1);
        if (e == cudaSuccess) e = cudaEventSynchronize(ctx->stage_ev[c & 1]);
        if (e != cudaSuccess) break;
        const size_t o = c * STAGE_BYTES;
        pool_copy((char*)dst + o, ctx->h_stage[c & 1], std::min(STAGE_BYTES, bytes - o));
    }
    return e;
}

void scan_arenas(const fbk_arena_view* arenas, int n_arenas, ArenaScan& sc) {
    struct Job { int a; uint64_t lo, hi; };
    std::vector<Job> jobs;
    for (int a = 0; a < n_arenas; ++a)
        for (uint64_t lo = 0; lo < arenas[a].n_seqs; lo += ArenaScan::BLOCK)
            jobs.push_back({a, lo, std::min(arenas[a].n_seqs, lo + ArenaScan::BLOCK)});
    sc.block_bases.assign(jobs.size(), 0);
    struct Part {
        uint64_t bases = 0, max_pair = 0, long_bases = 0;
        uint32_t max_len = 0;
        bool bad = false;
        std::vector<uint64_t> hist;
    };
    std::vector<Part> parts(host_threads());
    host_parallel_for(jobs.size(), [&](uint64_t j, unsigned t) {
        Part& P = parts[t];
        if (P.hist.empty()) P.hist.assign(ArenaScan::BINS, 0);
        const fbk_arena_view& v = arenas[jobs[j].a];
        const uint64_t cap = v.n_words * 32;
        uint64_t bases = 0;
        for (uint64_t i = jobs[j].lo; i < jobs[j].hi; ++i) {
            const uint32_t L = v.lengths[i];
            // every sequence must lie inside its arena's words: the kernels read only there
            P.bad |= L && v.offsets[i] + (uint64_t)L > cap;
            bases += L;
            P.max_len = std::max(P.max_len, L);
            if (v.pair_idx) P.max_pair = std::max<uint64_t>(P.max_pair, v.pair_idx[i]);
            if (L < ArenaScan::BINS - 1) P.hist[L]++;
            else P.long_bases += L;
        }
        sc.block_bases[j] = bases;
        P.bases += bases;
    });
    sc.hist.assign(ArenaScan::BINS, 0);
    for (const Part& P : parts) {
        if (P.hist.empty()) continue;
        sc.n_bases += P.bases;
        sc.max_pair = std::max(sc.max_pair, P.max_pair);
        sc.max_len = std::max(sc.max_len, P.max_len);
        sc.long_bases += P.long_bases;
        sc.bad |= P.bad;
        for (uint64_t L = 0; L <= std::min<uint64_t>(P.max_len, ArenaScan::BINS - 1); ++L) sc.hist[L] += P.hist[L];
    }
    for (int a = 0; a < n_arenas; ++a) sc.n_reads += arenas[a].n_seqs;
}

static cudaError_t copy_stream_of(fbk_ctx* ctx, cudaStream_t* s) {
    if (!ctx->copy_stream) {
        cudaError_t e = cudaStreamCreateWithFlags(&ctx->copy_stream, cudaStreamNonBlocking);
        if (e != cudaSuccess) return e;
    }
    *s = ctx->copy_stream;
    return cudaSuccess;
}

cudaError_t bank_wait(fbk_ctx* ctx, const fbk_bank* b) {
    return b && b->ready ? cudaStreamWaitEvent(ctx->stream, b->ready, 0) : cudaSuccess;
}

fbk_status bank_upload_impl(fbk_ctx* ctx, const fbk_arena_view* arenas, int n_arenas, fbk_bank** out, uint64_t chunk_bases,
                            bool async) {
    uint64_t n_words = 0;
    bool all_pairs = true;
    for (int a = 0; a < n_arenas; ++a) {
        const fbk_arena_view& v = arenas[a];
        if (v.n_seqs && (!v.offsets || !v.lengths)) return set_err(ctx, FBK_ERR_INVALID, "arena has sequences but no offsets/lengths");
        if (v.n_words && !v.data) return set_err(ctx, FBK_ERR_INVALID, "arena has words but no data pointer");
        if (v.n_seqs && !v.pair_idx) all_pairs = false;
        n_words += v.n_words;
    }
    ArenaScan sc;
    scan_arenas(arenas, n_arenas, sc);
    if (sc.bad) return set_err(ctx, FBK_ERR_INVALID, "sequence extends past the arena data");
    const uint64_t n_reads = sc.n_reads, n_bases = sc.n_bases, max_pair = sc.max_pair;
    const uint32_t max_len = sc.max_len;
    fbk_bank* b = new fbk_bank();
    b->ctx = ctx;
    b->n_reads = n_reads;
    b->n_words = n_words;
    b->n_bases = n_bases;
    b->max_len = max_len;
    b->n_pairs = all_pairs && n_reads ? max_pair + 1 : 0;
    b->data = (uint64_t*)dev_alloc(ctx, (n_words + 8) * 8);
    b->off = (uint64_t*)dev_alloc(ctx, std::max<uint64_t>(n_reads, 1) * 8);
    b->len = (uint32_t*)dev_alloc(ctx, std::max<uint64_t>(n_reads, 1) * 4);
    if (all_pairs && n_reads) b->pair_idx = (uint32_t*)dev_alloc(ctx, n_reads * 4);
    if (!b->data || !b->off || !b->len || (all_pairs && n_reads && !b->pair_idx)) {
        fbk_bank_release(b);
        return set_err(ctx, FBK_ERR_OOM, "device memory for the read bank");
    }
    uint64_t wbase = 0, rbase = 0;
    Launch L = launch_cfg(ctx, 256, 0);
    // An asynchronous upload (every arena buffer page-locked) copies and rebases on the
    // context's copy stream and records b->ready; the calls that read the bank order
    // the context's stream after it (bank_wait).
    if (async) {
        for (int a = 0; a < n_arenas && async; ++a) {
            const fbk_arena_view& v = arenas[a];
            async = (!v.n_words || host_page_locked(v.data)) &&
                    (!v.n_seqs || (host_page_locked(v.offsets) && host_page_locked(v.lengths) &&
                                   (!v.pair_idx || host_page_locked(v.pair_idx))));
        }
        cudaError_t e = async ? copy_stream_of(ctx, &L.stream) : cudaSuccess;
        if (e == cudaSuccess && async) e = cudaEventCreateWithFlags(&b->ready, cudaEventDisableTiming);
        if (e != cudaSuccess) {
            fbk_bank_release(b);
            return cuda_err(ctx, e, "bank upload stream");
        }
    }
    auto h2d = [&](void* dst, const void* src, size_t bytes) -> cudaError_t {
        if (!async) return copy_h2d(ctx, dst, src, bytes);
        return cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, L.stream);
    };
    for (int a = 0; a < n_arenas; ++a) {
        const fbk_arena_view& v = arenas[a];
        cudaError_t e = cudaSuccess;
        if (v.n_words) e = h2d(b->data + wbase, v.data, v.n_words * 8);
        if (e == cudaSuccess && v.n_seqs) e = h2d(b->off + rbase, v.offsets, v.n_seqs * 8);
        if (e == cudaSuccess && v.n_seqs) e = h2d(b->len + rbase, v.lengths, v.n_seqs * 4);
        if (e == cudaSuccess && v.n_seqs && b->pair_idx) e = h2d(b->pair_idx + rbase, v.pair_idx, v.n_seqs * 4);
        if (e == cudaSuccess && wbase && v.n_seqs) {
            TimedLaunch tl;
            time_begin(ctx, "bank_rebase", tl);
            e = launch_add_u64(L, b->off + rbase, v.n_seqs, wbase * 32);
            time_end(ctx, tl);
        }
        if (e != cudaSuccess) {
            fbk_bank_release(b);
            return cuda_err(ctx, e, "bank upload");
        }
        wbase += v.n_words;
        rbase += v.n_seqs;
        b->arena_reads.push_back(v.n_seqs);
    }
    cudaError_t e = cudaMemsetAsync(b->data + n_words, 0, 8 * 8, L.stream);
    if (e == cudaSuccess && async) e = cudaEventRecord(b->ready, L.stream);
    if (e != cudaSuccess) {
        fbk_bank_release(b);
        return cuda_err(ctx, e, "bank padding");
    }
    // Read ranges with fewer than chunk_bases bases: one launch over a range adds
    // at most (bases x weight) to any 32-bit counter, which the callers keep below
    // 2^32 - 2^17 (counters start each launch at <= 65535).  Greedy walk: a range
    // ends before the read that would bring it to chunk_bases; a block whose bases
    // cannot reach that is skipped whole.
    b->chunk_starts.push_back(0);
    uint64_t acc = 0, r = 0, j = 0;
    for (int a = 0; a < n_arenas; ++a)
        for (uint64_t lo = 0; lo < arenas[a].n_seqs; lo += ArenaScan::BLOCK, ++j) {
            const uint64_t hi = std::min(arenas[a].n_seqs, lo + ArenaScan::BLOCK);
            if (acc + sc.block_bases[j] < chunk_bases) {
                acc += sc.block_bases[j];
                r += hi - lo;
                continue;
            }
            for (uint64_t i = lo; i < hi; ++i, ++r) {
                if (acc && acc + arenas[a].lengths[i] >= chunk_bases) {
                    b->chunk_starts.push_back(r);
                    b->max_chunk = std::max(b->max_chunk, acc);
                    acc = 0;
                }
                acc += arenas[a].lengths[i];
            }
        }
    b->max_chunk = std::max(b->max_chunk, acc);
    b->chunk_starts.push_back(n_reads);
    // length histogram with bins 0 .. max_len (+1 spare); longer reads (>= 2^16 - 1)
    // are counted by their bases only
    const uint64_t bins = std::min<uint64_t>((uint64_t)max_len + 2, ArenaScan::BINS);
    b->len_hist.assign(sc.hist.begin(), sc.hist.begin() + bins);
    b->long_bases = sc.long_bases;
    for (uint64_t L = bins - 1; L < ArenaScan::BINS; ++L) b->long_bases += L * sc.hist[L];
    *out = b;
    return FBK_OK;
}

}  // namespace fbk

extern "C" {

FBK_API fbk_status fbk_bank_upload(fbk_ctx* ctx, const fbk_arena_view arenas[3], fbk_bank** out) {
    if (!ctx || !arenas || !out) return FBK_ERR_INVALID;
    CK(ctx, cudaSetDevice(ctx->device));
    return bank_upload_impl(ctx, arenas, 3, out);
}

FBK_API fbk_status fbk_bank_upload_async(fbk_ctx* ctx, const fbk_arena_view arenas[3], fbk_bank** out) {
    if (!ctx || !arenas || !out) return FBK_ERR_INVALID;
    CK(ctx, cudaSetDevice(ctx->device));
    return bank_upload_impl(ctx, arenas, 3, out, 1ull << 30, true);
}

FBK_API fbk_status fbk_bank_wait(const fbk_bank* b) {
    if (!b) return FBK_ERR_INVALID;
    if (b->ready) CK(b->ctx, cudaEventSynchronize(b->ready));
    return FBK_OK;
}

FBK_API fbk_status fbk_bank_info(const fbk_bank* b, uint64_t* n_reads, uint64_t* n_bases) {
    if (!b) return FBK_ERR_INVALID;
    if (n_reads) *n_reads = b->n_reads;
    if (n_bases) *n_bases = b->n_bases;
    return FBK_OK;
}

FBK_API fbk_status fbk_bank_release(fbk_bank* b) {
    if (!b) return FBK_OK;
    fbk_ctx* ctx = b->ctx;
    cudaStreamSynchronize(ctx->stream);
    if (b->ready) {
        cudaEventSynchronize(b->ready);
        cudaEventDestroy(b->ready);
    }
    dev_free(ctx, b->data);
    dev_free(ctx, b->off);
    dev_free(ctx, b->len);
    dev_free(ctx, b->pair_idx);
    delete b;
    return FBK_OK;
}

// ===========================================================================
// CountMinSketch
// ===========================================================================
FBK_API uint64_t fbk_cms_width_for_genome_size(uint64_t g) {
    if (g > (1ULL << 27) / 16) return 1ULL << 27;  // above the clamp (and no overflow of g * 16)
    uint64_t x = g * 16, t = 1;
    while (t < x) t <<= 1;
    return std::min<uint64_t>(std::max<uint64_t>(t, 1ULL << 21), 1ULL << 27);
}

FBK_API fbk_status fbk_cms_create(fbk_ctx* ctx, uint32_t log2w, uint32_t cbits, fbk_cms** out) {
    if (!ctx || !out || (cbits != 4 && cbits != 16) || log2w < 3 || log2w > 30)
        return set_err(ctx, FBK_ERR_INVALID, "cms: counter_bits must be 4 or 16 and 3 <= log2_width <= 30");
    CK(ctx, cudaSetDevice(ctx->device));
    fbk_cms* c = new fbk_cms();
    c->ctx = ctx;
    c->log2w = log2w;
    c->cbits = cbits;
    c->n = 4ULL << log2w;
    c->cnt = (uint32_t*)dev_alloc(ctx, c->n * 4);
    c->hll12 = (uint32_t*)dev_alloc(ctx, 4096 * 4);
    if (!c->cnt || !c->hll12) {
        dev_free(ctx, c->cnt);
        dev_free(ctx, c->hll12);
        delete c;
        return set_err(ctx, FBK_ERR_OOM, "device memory for the count-min sketch");
    }
    CK(ctx, cudaMemsetAsync(c->cnt, 0, c->n * 4, ctx->stream));
    CK(ctx, cudaMemsetAsync(c->hll12, 0, 4096 * 4, ctx->stream));
    *out = c;
    return FBK_OK;
}

FBK_API fbk_status fbk_cms_clear(fbk_cms* c) {
    if (!c) return FBK_ERR_INVALID;
    CK(c->ctx, cudaMemsetAsync(c->cnt, 0, c->n * 4, c->ctx->stream));
    CK(c->ctx, cudaMemsetAsync(c->hll12, 0, 4096 * 4, c->ctx->stream));
    return FBK_OK;
}

// Keeps every count <= 65535 between calls (exact below every cap).
static fbk_status cms_clamp(fbk_cms* c) {
    fbk_ctx* ctx = c->ctx;
    TIMED(ctx, "cms_clamp", launch_clamp_counters(launch_cfg(ctx, 256, 0), c->cnt, c->n));
    return FBK_OK;
}

static fbk_status cms_keys_op(fbk_cms* c, const uint64_t* keys, uint64_t n, uint32_t* est, int add) {
    if (!c || (n && !keys) || (!add && n && !est)) return FBK_ERR_INVALID;
    if (n == 0) return FBK_OK;
    fbk_ctx* ctx = c->ctx;
    const uint64_t chunk = 1ULL << 30;  // adds per launch stay far below 2^32 - 2^17
    uint64_t* dk = (uint64_t*)dev_alloc(ctx, std::min(n, chunk) * 8);
    uint32_t* de = add ? nullptr : (uint32_t*)dev_alloc(ctx, std::min(n, chunk) * 4);
    if (!dk || (!add && !de)) {
        dev_free(ctx, dk);
        dev_free(ctx, de);
        return set_err(ctx, FBK_ERR_OOM, "cms key buffer");
    }
    cudaError_t e = cudaSuccess;
    for (uint64_t s0 = 0; s0 < n && e == cudaSuccess; s0 += chunk) {
        const uint64_t m = std::min(chunk, n - s0);
        e = cudaMemcpyAsync(dk, keys + s0, m * 8, cudaMemcpyHostToDevice, ctx->stream);
        if (e == cudaSuccess) {
            TimedLaunch tl;
            time_begin(ctx, add ? "cms_add_keys" : "cms_estimate_keys", tl);
            // The final counts of a batch of adds do not depend on their order, so one
            // launch reproduces the sequential adds exactly.
            e = launch_cms_keys(launch_cfg(ctx, 256, 0), c->cnt, c->log2w, c->cap(), dk, m, de, add);
            time_end(ctx, tl);
        }
        if (e == cudaSuccess && add) e = launch_clamp_counters(launch_cfg(ctx, 256, 0), c->cnt, c->n);
        if (e == cudaSuccess && !add) e = cudaMemcpyAsync(est + s0, de, m * 4, cudaMemcpyDeviceToHost, ctx->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    }
    dev_free(ctx, dk);
    dev_free(ctx, de);
    if (e != cudaSuccess) return cuda_err(ctx, e, "cms key op");
    return FBK_OK;
}

FBK_API fbk_status fbk_cms_add_keys(fbk_cms* c, const uint64_t* keys, uint64_t n) { return cms_keys_op(c, keys, n, nullptr, 1); }
FBK_API fbk_status fbk_cms_estimate_keys(fbk_cms* c, const uint64_t* keys, uint64_t n, uint32_t* out) {
    return cms_keys_op(c, keys, n, out, 0);
}

static int nw_of(uint32_t key_bits) { return key_bits == 64 ? 1 : key_bits == 128 ? 2 : key_bits == 256 ? 4 : 0; }
static uint32_t max_k_of(uint32_t key_bits) { return key_bits == 64 ? 31 : key_bits == 128 ? 63 : 127; }

// Builds the subsampler bitmap for a bank on the device (nullptr when keeping all).
static fbk_status make_keep_bits(fbk_ctx* ctx, const fbk_bank* b, const fbk_subsample* ss, uint64_t** bits_out) {
    *bits_out = nullptr;
    if (!ss || !(ss->factor < 0.999)) return FBK_OK;
    if (!b->pair_idx || b->n_pairs == 0)
        return set_err(ctx, FBK_ERR_INVALID, "subsampling needs per-read pair indices in the bank");
    uint64_t nw = (b->n_pairs + 63) / 64;
    uint64_t* bits = (uint64_t*)dev_alloc(ctx, nw * 8);
    if (!bits) return set_err(ctx, FBK_ERR_OOM, "subsample bitmap");
    TIMED(ctx, "subsample", launch_subsample_mask(launch_cfg(ctx, 256, 0), b->n_pairs, ss->factor, ss->seed, bits));
    *bits_out = bits;
    return FBK_OK;
}

// Sweep plan: each sweep touches at most ctx->sweep_bytes of the sketch — several
// whole rows when they fit, else a column range of one row.  Fewer sweeps mean fewer
// scans of the bank; smaller slices stay resident in L2.
struct SweepPlan {
    uint32_t rows_per;   // rows per sweep (1, 2 or 4)
    uint64_t cols_per;   // columns per sweep (all when rows_per > 1)
};
static SweepPlan sweep_plan(const fbk_ctx* ctx, uint32_t log2w) {
    const uint64_t w = 1ULL << log2w, row_bytes = w * 4;
    SweepPlan sp;
    if (ctx->sweep_bytes >= 4 * row_bytes) sp = {4, w};
    else if (ctx->sweep_bytes >= 2 * row_bytes) sp = {2, w};
    else sp = {1, std::min(w, std::max<uint64_t>(1024, ctx->sweep_bytes / 4))};
    return sp;
}

static fbk_status pass1_impl(fbk_cms* c, const fbk_bank* b, uint32_t k, uint32_t key_bits, const uint64_t* keep_bits,
                             uint32_t mult) {
    fbk_ctx* ctx = c->ctx;
    const int nw = nw_of(key_bits);
    if (!nw || k < 1 || k > max_k_of(key_bits)) return set_err(ctx, FBK_ERR_INVALID, "k out of range for key_bits");
    if ((uint64_t)mult * b->max_chunk_bases() >= (1ULL << 32) - (1ULL << 17))
        return set_err(ctx, FBK_ERR_INVALID, "pass 1: read chunk too large for this weight");
    Launch L = launch_cfg_persistent(ctx, ctx->block_pass1, ctx->grid_pass1);
    const uint64_t w = 1ULL << c->log2w;
    const SweepPlan sp = sweep_plan(ctx, c->log2w);
    for (size_t ch = 0; ch + 1 < b->chunk_starts.size(); ++ch) {
        const BankDev bv = bank_view(b, b->chunk_starts[ch], b->chunk_starts[ch + 1], keep_bits);
        for (uint32_t row = 0; row < 4; row += sp.rows_per)
            for (uint64_t c0 = 0; c0 < w; c0 += sp.cols_per)
                TIMED(ctx, "pass1", launch_pass1_sweep(nw, L, bv, k, c->cnt, c->log2w, row, row + sp.rows_per, c0,
                                                       std::min(w, c0 + sp.cols_per), mult,
                                                       (row == 0 && c0 == 0) ? c->hll12 : nullptr));
        fbk_status st = cms_clamp(c);
        if (st) return st;
    }
    return FBK_OK;
}

// Distinct canonical keys added to the sketch by bank passes (p=12 HyperLogLog over
// the 1 key in 16 whose hash ends in four zero bits, about 1.6% standard error at
// isolate scale); only used to size the solid table.
static fbk_status cms_distinct(const fbk_cms* c, uint64_t* out) {
    fbk_ctx* ctx = c->ctx;
    uint32_t* h = (uint32_t*)ctx->h_pinned;
    CK(ctx, cudaMemcpyAsync(h, c->hll12, 4096 * 4, cudaMemcpyDeviceToHost, ctx->stream));
    CK(ctx, cudaStreamSynchronize(ctx->stream));
    double sum = 0.0;
    uint64_t zeros = 0;
    for (int i = 0; i < 4096; ++i) {
        sum += std::ldexp(1.0, -(int)h[i]);
        zeros += h[i] == 0;
    }
    // pass 1 counts 1 key in PASS1_HLL_SAMPLE (by hash)
    *out = (uint64_t)(hll_estimate_from_sum(sum, zeros, 12) * PASS1_HLL_SAMPLE * 1.08) + 4096;
    return FBK_OK;
}

FBK_API fbk_status fbk_cms_add_bank(fbk_cms* c, const fbk_bank* b, uint32_t k, uint32_t key_bits, const fbk_subsample* ss) {
    if (!c || !b) return FBK_ERR_INVALID;
    fbk_ctx* ctx = c->ctx;
    CK(ctx, cudaSetDevice(ctx->device));
    CK(ctx, bank_wait(ctx, b));
    uint64_t* keep = nullptr;
    fbk_status st = make_keep_bits(ctx, b, ss, &keep);
    if (st) return st;
    st = pass1_impl(c, b, k, key_bits, keep, 1);
    if (keep) {
        cudaStreamSynchronize(ctx->stream);
        dev_free(ctx, keep);
    }
    return st;
}

FBK_API fbk_status fbk_cms_build(fbk_ctx* ctx, const fbk_bank* b, uint32_t k, uint32_t key_bits, uint32_t log2_width,
                                 uint32_t counter_bits, fbk_cms** out) {
    if (!ctx || !b || !out) return FBK_ERR_INVALID;
    *out = nullptr;
    fbk_cms* c = nullptr;
    fbk_status st = fbk_cms_create(ctx, log2_width, counter_bits, &c);
    if (st) return st;
    st = fbk_cms_add_bank(c, b, k, key_bits, nullptr);
    if (st) {
        fbk_cms_release(c);
        return st;
    }
    *out = c;
    return FBK_OK;
}

// Prior contigs are counted with weights up to 1000 per push, so their bank is cut
// into ranges of fewer than 4M bases (1000 x 4M < 2^32 - 2^17).
static const uint64_t CONTIG_CHUNK_BASES = 4000000;

// Packs ASCII contigs into a one-arena device bank (ASCII_TO_2BIT, bitseq.rs:67-81).
static fbk_status contig_bank(fbk_ctx* ctx, const uint8_t* ascii, const uint64_t* offs, uint64_t n, fbk_bank** out) {
    std::vector<uint64_t> words, o(n);
    std::vector<uint32_t> l(n);
    uint64_t pos = 0;
    for (uint64_t i = 0; i < n; ++i) {
        uint64_t len = offs[i + 1] - offs[i];
        if (len >= CONTIG_CHUNK_BASES) return set_err(ctx, FBK_ERR_INVALID, "contig of 4M bases or more");
        o[i] = pos;
        l[i] = (uint32_t)len;
        words.resize((pos + len + 31) / 32 + 1, 0);
        for (uint64_t j = 0; j < len; ++j, ++pos) {
            uint8_t ch = ascii[offs[i] + j];
            uint64_t code = (ch == 'C' || ch == 'c') ? 1 : (ch == 'G' || ch == 'g') ? 2 : (ch == 'T' || ch == 't') ? 3 : 0;
            words[pos >> 5] |= code << ((pos & 31) * 2);
        }
    }
    fbk_arena_view v;
    v.data = words.data();
    v.n_words = words.size();
    v.offsets = o.data();
    v.lengths = l.data();
    v.n_seqs = n;
    v.pair_idx = nullptr;
    fbk_status st = bank_upload_impl(ctx, &v, 1, out, CONTIG_CHUNK_BASES);
    if (st == FBK_OK) cudaStreamSynchronize(ctx->stream);  // host vectors go out of scope
    return st;
}

FBK_API fbk_status fbk_cms_add_contigs(fbk_cms* c, const uint8_t* ascii, const uint64_t* offs, uint64_t n, uint32_t k,
                                       uint32_t key_bits) {
    if (!c || (n && (!ascii || !offs))) return FBK_ERR_INVALID;
    if (n == 0) return FBK_OK;
    fbk_ctx* ctx = c->ctx;
    fbk_bank* cb = nullptr;
    fbk_status st = contig_bank(ctx, ascii, offs, n, &cb);
    if (st) return st;
    st = pass1_impl(c, cb, k, key_bits, nullptr, 10);
    fbk_bank_release(cb);
    return st;
}

FBK_API fbk_status fbk_cms_nbytes(const fbk_cms* c, uint64_t* nbytes) {
    if (!c || !nbytes) return FBK_ERR_INVALID;
    *nbytes = c->cbits == 4 ? c->n / 2 : c->n * 2;
    return FBK_OK;
}

FBK_API fbk_status fbk_cms_export(fbk_cms* c, uint8_t* out, uint64_t nbytes) {
    uint64_t want = 0;
    if (!c || !out || fbk_cms_nbytes(c, &want) != FBK_OK || nbytes != want) return FBK_ERR_INVALID;
    fbk_ctx* ctx = c->ctx;
    uint8_t* d = (uint8_t*)dev_alloc(ctx, nbytes);
    if (!d) return set_err(ctx, FBK_ERR_OOM, "cms export buffer");
    cudaError_t e;
    {
        TimedLaunch tl;
        time_begin(ctx, "cms_export", tl);
        e = launch_cms_export((int)c->cbits, launch_cfg(ctx, 256, 0), c->cnt, c->n, d);
        time_end(ctx, tl);
    }
    if (e == cudaSuccess) e = copy_d2h(ctx, out, d, nbytes);
    dev_free(ctx, d);
    if (e != cudaSuccess) return cuda_err(ctx, e, "cms export");
    return FBK_OK;
}

FBK_API fbk_status fbk_cms_import(fbk_cms* c, const uint8_t* in, uint64_t nbytes) {
    uint64_t want = 0;
    if (!c || !in || fbk_cms_nbytes(c, &want) != FBK_OK || nbytes != want) return FBK_ERR_INVALID;
    fbk_ctx* ctx = c->ctx;
    uint8_t* d = (uint8_t*)dev_alloc(ctx, nbytes);
    if (!d) return set_err(ctx, FBK_ERR_OOM, "cms import buffer");
    cudaError_t e = copy_h2d(ctx, d, in, nbytes);
    if (e == cudaSuccess) {
        TimedLaunch tl;
        time_begin(ctx, "cms_import", tl);
        e = launch_cms_import((int)c->cbits, launch_cfg(ctx, 256, 0), c->cnt, c->n, d);
        time_end(ctx, tl);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    dev_free(ctx, d);
    if (e != cudaSuccess) return cuda_err(ctx, e, "cms import");
    return FBK_OK;
}

FBK_API fbk_status fbk_cms_merge(fbk_cms* dst, const fbk_cms* src) {
    if (!dst || !src || dst->cbits != src->cbits || dst->log2w != src->log2w) return FBK_ERR_INVALID;
    fbk_ctx* ctx = dst->ctx;
    if (src->ctx != ctx) CK(ctx, cudaStreamSynchronize(src->ctx->stream));
    TIMED(ctx, "cms_merge", launch_cms_merge(launch_cfg(ctx, 256, 0), dst->cnt, src->cnt, dst->n));
    return FBK_OK;
}

FBK_API fbk_status fbk_cms_counts_device(fbk_cms* c, uint32_t** counts, uint64_t* n) {
    if (!c || !counts || !n) return FBK_ERR_INVALID;
    *counts = c->cnt;
    *n = c->n;
    return FBK_OK;
}

FBK_API fbk_status fbk_cms_clamp_counts(fbk_cms* c) {
    if (!c) return FBK_ERR_INVALID;
    fbk_ctx* ctx = c->ctx;
    CK(ctx, cudaSetDevice(ctx->device));
    fbk_status st = cms_clamp(c);
    if (st == FBK_OK) CK(ctx, cudaStreamSynchronize(ctx->stream));
    return st;
}

FBK_API fbk_status fbk_cms_release(fbk_cms* c) {
    if (!c) return FBK_OK;
    cudaStreamSynchronize(c->ctx->stream);
    dev_free(c->ctx, c->cnt);
    dev_free(c->ctx, c->hll12);
    delete c;
    return FBK_OK;
}

// ===========================================================================
// HyperLogLog
// ===========================================================================
FBK_API fbk_status fbk_hll_create(fbk_ctx* ctx, uint32_t p, fbk_hll** out) {
    if (!ctx || !out || p < 4 || p > 18) return set_err(ctx, FBK_ERR_INVALID, "hll: 4 <= p <= 18");
    fbk_hll* h = new fbk_hll();
    h->ctx = ctx;
    h->p = p;
    h->regs = (uint32_t*)dev_alloc(ctx, (1ULL << p) * 4);
    if (!h->regs) {
        delete h;
        return set_err(ctx, FBK_ERR_OOM, "hll registers");
    }
    CK(ctx, cudaMemsetAsync(h->regs, 0, (1ULL << p) * 4, ctx->stream));
    *out = h;
    return FBK_OK;
}

static fbk_status hll_add(fbk_hll* h, const uint64_t* x, uint64_t n, int mix) {
    if (!h || (n && !x)) return FBK_ERR_INVALID;
    if (!n) return FBK_OK;
    fbk_ctx* ctx = h->ctx;
    uint64_t* d = (uint64_t*)dev_alloc(ctx, n * 8);
    if (!d) return set_err(ctx, FBK_ERR_OOM, "hll hash buffer");
    cudaError_t e = cudaMemcpyAsync(d, x, n * 8, cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) {
        TimedLaunch tl;
        time_begin(ctx, "hll_add", tl);
        e = launch_hll_add(launch_cfg(ctx, 256, 0), h->regs, h->p, d, n, mix);
        time_end(ctx, tl);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    dev_free(ctx, d);
    if (e != cudaSuccess) return cuda_err(ctx, e, "hll add");
    return FBK_OK;
}
FBK_API fbk_status fbk_hll_add_hashes(fbk_hll* h, const uint64_t* x, uint64_t n) { return hll_add(h, x, n, 0); }
FBK_API fbk_status fbk_hll_add_canonical_hashes(fbk_hll* h, const uint64_t* x, uint64_t n) { return hll_add(h, x, n, 1); }

FBK_API fbk_status fbk_hll_merge(fbk_hll* dst, const fbk_hll* src) {
    if (!dst || !src || dst->p != src->p) return FBK_ERR_INVALID;
    fbk_ctx* ctx = dst->ctx;
    TIMED(ctx, "hll_merge", launch_hll_merge(launch_cfg(ctx, 256, 0), dst->regs, src->regs, 1ULL << dst->p));
    return FBK_OK;
}

FBK_API fbk_status fbk_hll_export(fbk_hll* h, uint8_t* regs, uint64_t n) {
    if (!h || !regs || n != (1ULL << h->p)) return FBK_ERR_INVALID;
    std::vector<uint32_t> tmp(n);
    CK(h->ctx, cudaMemcpyAsync(tmp.data(), h->regs, n * 4, cudaMemcpyDeviceToHost, h->ctx->stream));
    CK(h->ctx, cudaStreamSynchronize(h->ctx->stream));
    for (uint64_t i = 0; i < n; ++i) regs[i] = (uint8_t)tmp[i];
    return FBK_OK;
}

FBK_API double fbk_hll_estimate_registers(const uint8_t* regs, uint32_t p) {
    if (!regs || p < 4 || p > 18) return std::nan("");
    const uint64_t n = 1ULL << p;
    double sum = 0.0;
    uint64_t zeros = 0;
    for (uint64_t i = 0; i < n; ++i) {
        sum += std::ldexp(1.0, -(int)regs[i]);
        zeros += regs[i] == 0;
    }
    return hll_estimate_from_sum(sum, zeros, p);
}

FBK_API fbk_status fbk_hll_estimate(fbk_hll* h, double* out) {
    if (!h || !out) return FBK_ERR_INVALID;
    std::vector<uint8_t> r(1ULL << h->p);
    fbk_status st = fbk_hll_export(h, r.data(), r.size());
    if (st) return st;
    *out = fbk_hll_estimate_registers(r.data(), h->p);
    return FBK_OK;
}

FBK_API fbk_status fbk_hll_release(fbk_hll* h) {
    if (!h) return FBK_OK;
    cudaStreamSynchronize(h->ctx->stream);
    dev_free(h->ctx, h->regs);
    delete h;
    return FBK_OK;
}

// ===========================================================================
// solid table
// ===========================================================================
static void table_free_storage(fbk_table* t) {
    fbk_ctx* ctx = t->ctx;
    if (t->tags != t->keys) dev_free(ctx, t->tags);
    dev_free(ctx, t->keys);
    dev_free(ctx, t->cnt);
    dev_free(ctx, t->cov);
    t->keys = t->tags = nullptr;
    t->cnt = t->cov = nullptr;
}
static void table_free_out(fbk_table* t) {
    dev_free(t->ctx, t->out_keys);
    dev_free(t->ctx, t->out_cov);
    dev_free(t->ctx, t->out_mask);
    t->out_keys = nullptr;
    t->out_cov = nullptr;
    t->out_mask = nullptr;
    t->out_cap = 0;
}

static TableDev table_dev(const fbk_table* t) {
    TableDev d;
    d.keys = t->keys;
    d.tags = t->tags;
    d.tag_stride = t->tags && t->tags == t->keys ? 4u : 1u;
    d.cnt = t->cnt;
    d.cov = t->cov;
    d.cap = t->cap;
    d.max_probe = (uint32_t)std::min<uint64_t>(t->cap, 1u << 16);
    d.spin_limit = 1u << 20;
    return d;
}

static fbk_status table_alloc(fbk_table* t, uint64_t cap, bool with_cov) {
    fbk_ctx* ctx = t->ctx;
    t->cap = cap;
    t->keys = (uint64_t*)dev_alloc(ctx, cap * 8 * t->nw);
    if (t->nw > 2) t->tags = tag_in_key(t->nw, t->k) ? t->keys : (uint64_t*)dev_alloc(ctx, cap * 8);
    t->cnt = (uint32_t*)dev_alloc(ctx, cap * 32);
    if (with_cov) t->cov = (uint32_t*)dev_alloc(ctx, cap * 4);
    if (!t->keys || (t->nw > 2 && !t->tags) || !t->cnt || (with_cov && !t->cov)) {
        table_free_storage(t);
        return set_err(ctx, FBK_ERR_OOM, "device memory for the solid table (capacity " + std::to_string(cap) + ")");
    }
    TIMED(ctx, "table_init", launch_table_init((int)t->nw, launch_cfg(ctx, 256, 0), table_dev(t)));
    CK(ctx, cudaMemsetAsync(t->cnt, 0, cap * 32, ctx->stream));
    if (with_cov) CK(ctx, cudaMemsetAsync(t->cov, 0, cap * 4, ctx->stream));
    return FBK_OK;
}

// Runs the conversion kernel, (re)allocating the compact output when needed.
static fbk_status table_convert(fbk_table* t, uint64_t* acc_keys, uint16_t* acc_cov, uint16_t* acc_edges, uint64_t acc_cap,
                                uint64_t* acc_digest = nullptr) {
    fbk_ctx* ctx = t->ctx;
    // the rows are rewritten (or reallocated): an asynchronous export of them must have
    // been read out
    if (t->exported) CK(ctx, cudaEventSynchronize(t->exported));
    for (int attempt = 0; attempt < 2; ++attempt) {
        CK(ctx, cudaMemsetAsync(ctx->d_counts, 0, 8 * sizeof(unsigned long long), ctx->stream));
        ConvOut o{};
        o.acc_digest = acc_digest != nullptr;
        o.keys = t->out_keys;
        o.cov = t->out_cov;
        o.mask = t->out_mask;
        o.cap_solid = t->out_cap;
        o.acc_keys = acc_keys;
        o.acc_cov = acc_cov;
        o.acc_edges = acc_edges;
        o.cap_acc = acc_cap;
        o.counts = ctx->d_counts;
        TIMED(ctx, "convert", launch_convert((int)t->nw, launch_cfg(ctx, 256, 0), table_dev(t), t->min_trans_cov, o));
        unsigned long long* h = (unsigned long long*)ctx->h_pinned;
        CK(ctx, cudaMemcpyAsync(h, ctx->d_counts, 6 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, ctx->stream));
        CK(ctx, cudaStreamSynchronize(ctx->stream));
        t->n_keys = h[0];
        t->n_solid = h[1];
        t->digest = h[2];
        t->pushes = h[3] + t->skipped_pushes;
        if (acc_digest) *acc_digest = h[5];
        if (t->n_solid <= t->out_cap) return FBK_OK;
        table_free_out(t);
        uint64_t cap = t->n_solid + 1024;
        t->out_keys = (uint64_t*)dev_alloc(ctx, cap * 8 * t->nw);
        t->out_cov = (uint16_t*)dev_alloc(ctx, cap * 2);
        t->out_mask = (uint8_t*)dev_alloc(ctx, cap);
        if (!t->out_keys || !t->out_cov || !t->out_mask) {
            table_free_out(t);
            return set_err(ctx, FBK_ERR_OOM, "solid table output");
        }
        t->out_cap = cap;
    }
    return FBK_OK;
}

// The pass-1 gate kept as a threshold ladder instead of counts (fbk_k_ladder.cu).
struct Ladder {
    uint32_t* bits = nullptr;
    uint32_t log2w = 0;
};

// Solidity bitmap of a bank (bit = first base of a window, 1 = passes the CMS gate):
// starts all ones, one sweep per row slice clears the failing windows.
static fbk_status solidity_bitmap(fbk_ctx* ctx, const fbk_bank* b, const fbk_cms* cms, const fbk_build_params* p, int nw,
                                  const uint64_t* keep_bits, uint32_t** bm_out, const Ladder* lad) {
    const uint64_t n_bm = b->n_words + 9;
    uint32_t* bm = (uint32_t*)dev_alloc(ctx, n_bm * 4);
    if (!bm) return set_err(ctx, FBK_ERR_OOM, "solidity bitmap");
    *bm_out = bm;
    CK(ctx, cudaMemsetAsync(bm, 0xFF, n_bm * 4, ctx->stream));
    Launch L = launch_cfg_persistent(ctx, ctx->block_pass2, ctx->grid_pass2);
    if (lad) {
        TIMED(ctx, "solid", launch_ladder_solid(nw, L, bank_view(b, 0, b->n_reads, keep_bits), p->k, lad->bits, lad->log2w,
                                                p->t_solid, bm));
        return FBK_OK;
    }
    const uint64_t w = 1ULL << cms->log2w;
    const SweepPlan sp = sweep_plan(ctx, cms->log2w);
    const BankDev bv = bank_view(b, 0, b->n_reads, keep_bits);
    for (uint32_t row = 0; row < 4; row += sp.rows_per)
        for (uint64_t c0 = 0; c0 < w; c0 += sp.cols_per)
            TIMED(ctx, "solid", launch_solid_sweep(nw, L, bv, p->k, cms->cnt, cms->log2w, row, row + sp.rows_per, c0,
                                                   std::min(w, c0 + sp.cols_per), p->t_solid, cms->cap(), bm));
    return FBK_OK;
}

// Record buckets of pass 2: bucket b covers home slots [b << shift, (b+1) << shift),
// a table range of about ctx->bucket_bytes, so a bucket's upserts stay in L2.
struct Buckets {
    fbk_ctx* ctx = nullptr;
    BucketDev d{};
    uint32_t* overflow = nullptr;      // 256 bytes: the overflow flag, then the work counter
    unsigned long long* work = nullptr;  // work items handed out by the persistent upsert
    ~Buckets() {
        if (!ctx) return;
        cudaStreamSynchronize(ctx->stream);
        dev_free(ctx, d.recs);
        dev_free(ctx, d.fill);
        dev_free(ctx, overflow);
    }
};

static fbk_status buckets_alloc(fbk_ctx* ctx, uint64_t cap, uint64_t slot_bytes, int nw, uint32_t k, uint64_t max_records,
                                Buckets& bk) {
    const RecFmt fmt = record_format(k, nw);
    // at most 64 buckets (the emit kernel's per-warp staging holds 64 counters)
    uint32_t shift = 0;
    while (shift < 40 && (2ULL << shift) * slot_bytes <= ctx->bucket_bytes) ++shift;
    while (((cap + (1ULL << shift) - 1) >> shift) > 64) ++shift;
    const uint32_t P = (uint32_t)((cap + (1ULL << shift) - 1) >> shift);
    const uint32_t S = std::max<uint32_t>(1, std::min<uint32_t>(256, ctx->stripes));
    const uint64_t per_stripe = (uint64_t)(ctx->record_factor * (double)max_records / ((double)P * S)) +
                                (ctx->record_factor >= 1.0 ? 4096 : 0);
    bk.ctx = ctx;
    bk.d.shift = shift;
    bk.d.n_buckets = P;
    bk.d.stripes = S;
    bk.d.stripe_cap = per_stripe;
    bk.d.rw = fmt.rw;
    bk.d.ws = fmt.ws;
    bk.d.packed = fmt.packed;
    bk.d.recs = (uint64_t*)dev_alloc(ctx, (uint64_t)P * S * per_stripe * 8 * fmt.rw);
    bk.d.fill = (unsigned long long*)dev_alloc(ctx, (uint64_t)P * S * 8);
    bk.overflow = (uint32_t*)dev_alloc(ctx, 256);
    bk.work = bk.overflow ? (unsigned long long*)(bk.overflow + 2) : nullptr;
    bk.d.overflow = bk.overflow;
    if (!bk.d.recs || !bk.d.fill || !bk.overflow) return set_err(ctx, FBK_ERR_OOM, "pass-2 record buckets");
    CK(ctx, cudaMemsetAsync(bk.overflow, 0, 4, ctx->stream));
    return FBK_OK;
}

// Capacity of a filtered pass's table, chosen after bucket 0 of P is counted: the keys
// that pass the filter in bucket 0 are about the counters at or above min_trans_cov
// (keys that share a counter add a few percent), the buckets split the keys by hash
// evenly, and the table gets 30% headroom over that estimate at the load of tuning
// filter_load, a multiple of P slots, never more than the capacity from the distinct
// estimate.  Allocates and initialises the table.
static fbk_status size_filtered_table(fbk_table* t, const RecordFilter& flt, uint32_t n_buckets, uint64_t cap_distinct) {
    fbk_ctx* ctx = t->ctx;
    unsigned long long* d_n = ctx->d_counts + 7;
    CK(ctx, cudaMemsetAsync(d_n, 0, 8, ctx->stream));
    TIMED(ctx, "pass2_count", launch_count_at_least(launch_cfg(ctx, 256, 0), flt.cnt, 1ULL << flt.log2m, flt.min_records, d_n));
    CK(ctx, cudaMemcpyAsync(ctx->h_pinned, d_n, 8, cudaMemcpyDeviceToHost, ctx->stream));
    CK(ctx, cudaStreamSynchronize(ctx->stream));
    const uint64_t n0 = *(const unsigned long long*)ctx->h_pinned;
    const double keys = 1.3 * (double)n0 * (double)n_buckets;
    uint64_t cap = (uint64_t)(keys / ctx->filter_load) + 1024;
    cap = (cap + n_buckets - 1) / n_buckets * n_buckets;
    if (cap > cap_distinct) cap = cap_distinct;
    return table_alloc(t, cap, false);
}

// Pass 2 for every read chunk (and the prior contigs), with retries at twice the
// capacity when the probe limit is hit.  Reads go through record buckets; if a
// bucket stripe overflows, the chunk is redone by the direct sweep.
static fbk_status solid_build_impl(fbk_ctx* ctx, const fbk_bank* b, const fbk_cms* cms, const fbk_build_params* p,
                                   const uint64_t* keep_bits, const fbk_bank* contigs, uint64_t distinct_hint,
                                   fbk_table** out, const Ladder* lad = nullptr) {
    const int nw = nw_of(p->key_bits);
    if (!nw || p->k < 1 || p->k > max_k_of(p->key_bits)) return set_err(ctx, FBK_ERR_INVALID, "k out of range for key_bits");
    if (p->t_solid > 0xFFFF || p->min_trans_cov > 0xFFFF) return set_err(ctx, FBK_ERR_INVALID, "thresholds must fit u16");
    if (2 * b->max_chunk_bases() >= (1ULL << 32) - (1ULL << 17))
        return set_err(ctx, FBK_ERR_INVALID, "pass 2: read chunk too large");
    uint64_t cap;
    if (p->table_log2_cap) {
        if (p->table_log2_cap < 10 || p->table_log2_cap > 34) return set_err(ctx, FBK_ERR_INVALID, "table_log2_cap out of range");
        cap = 1ULL << p->table_log2_cap;
    } else {
        cap = std::max<uint64_t>(1024, (uint64_t)((double)distinct_hint / ctx->load_factor) + 1024);
    }
    // With a ladder gate and record buckets, the emit kernel evaluates the gate
    // itself; the bitmap is built only if a direct sweep is needed.
    uint32_t* bm = nullptr;
    struct BmGuard {
        fbk_ctx* c;
        uint32_t** p;
        ~BmGuard() {
            cudaStreamSynchronize(c->stream);
            dev_free(c, *p);
        }
    } bmg{ctx, &bm};
    const bool inline_gate = lad && ctx->pass2_mode == 1;
    struct DevBuf {
        fbk_ctx* c = nullptr;
        void* p = nullptr;
        void alloc(fbk_ctx* ctx, uint64_t bytes) {
            if (!p) {
                c = ctx;
                p = dev_alloc(ctx, bytes);
            }
        }
        ~DevBuf() {
            if (!p) return;
            cudaStreamSynchronize(c->stream);
            dev_free(c, p);
        }
    } fbuf;
    auto need_bitmap = [&]() -> fbk_status {
        if (bm) return FBK_OK;
        fbk_status s2 = solidity_bitmap(ctx, b, cms, p, nw, keep_bits, &bm, lad);
        if (s2) {
            dev_free(ctx, bm);
            bm = nullptr;
        }
        return s2;
    };
    fbk_status st = inline_gate ? FBK_OK : need_bitmap();
    if (st) return st;
    fbk_table* t = new fbk_table();
    t->ctx = ctx;
    t->nw = (uint32_t)nw;
    t->k = p->k;
    t->min_trans_cov = p->min_trans_cov;
    const uint64_t slot_bytes = 8ULL * nw + (nw > 2 ? 8 : 0) + 32 + (contigs ? 4 : 0);
    const uint64_t max_records = std::min(b->windows(p->k, p->k + 1), b->max_chunk_bases());
    const bool use_buckets = max_records && ctx->pass2_mode == 1;
    // the record filter needs every record of the pass in one bucket pass: one
    // read chunk and no prior contigs (their pushes weigh 1000)
    const bool filter = use_buckets && acc_filter_on(ctx->acc_filter, nw, distinct_hint, max_records) && !contigs &&
                        b->chunk_starts.size() == 2 && p->min_trans_cov >= 2;
    for (int attempt = 0; attempt < 4; ++attempt) {
        // A filtered pass holds only the keys that pass the filter, typically a small
        // part of the distinct k-mers: its first attempt sizes the table once the first
        // bucket is counted (the record buckets do not depend on the capacity), from the
        // counters that reach min_trans_cov.  A table that fills up reruns at the
        // capacity from the distinct estimate.
        const bool late_table = filter && attempt == 0 && ctx->filter_sizing && !p->table_log2_cap;
        if (!late_table) st = table_alloc(t, cap, contigs != nullptr);
        if (st) {
            table_free_out(t);
            delete t;
            return st;
        }
        if (!t->out_keys) {
            // Converted rows are a subset of the distinct keys: size the output from
            // the estimate (table_convert grows it and reruns if the estimate was low).
            const uint64_t oc = std::min<uint64_t>(cap, (uint64_t)(1.1 * (double)distinct_hint) + 4096);
            t->out_keys = (uint64_t*)dev_alloc(ctx, oc * 8 * t->nw);
            t->out_cov = (uint16_t*)dev_alloc(ctx, oc * 2);
            t->out_mask = (uint8_t*)dev_alloc(ctx, oc);
            if (!t->out_keys || !t->out_cov || !t->out_mask) table_free_out(t);
            else t->out_cap = oc;
        }
        CK(ctx, cudaMemsetAsync(ctx->d_status, 0, 4, ctx->stream));
        TableDev td = table_dev(t);
        Launch L = launch_cfg_persistent(ctx, ctx->block_pass2, ctx->grid_pass2);
        Launch Lc = launch_cfg(ctx, 256, 0);
        auto clamp = [&]() -> cudaError_t {
            cudaError_t e = launch_clamp_counters(Lc, t->cnt, t->cap * 8);
            if (e == cudaSuccess && t->cov) e = launch_clamp_counters(Lc, t->cov, t->cap);
            return e;
        };
        Buckets bk;
        // the buckets (their count and the table range each covers) follow the capacity
        // from the distinct estimate in every attempt
        st = use_buckets ? buckets_alloc(ctx, cap, slot_bytes, nw, p->k, max_records, bk) : FBK_OK;
        RecordFilter flt{};
        if (filter && st == FBK_OK) {
            // one counter per record or more, at most 2^23 (32 MB: stays in L2)
            uint32_t log2m = 11;
            while (log2m < 23 && (1ULL << log2m) < max_records / bk.d.n_buckets) ++log2m;
            fbuf.alloc(ctx, (1ULL << log2m) * 4 + 8);
            if (!fbuf.p) st = set_err(ctx, FBK_ERR_OOM, "pass-2 record filter");
            flt.cnt = (uint32_t*)fbuf.p;
            flt.log2m = log2m;
            flt.min_records = p->min_trans_cov;
            flt.skipped = (unsigned long long*)((char*)fbuf.p + (1ULL << log2m) * 4);
            if (st == FBK_OK) CK(ctx, cudaMemsetAsync(flt.skipped, 0, 8, ctx->stream));
        }
        if (st) {
            table_free_storage(t);
            table_free_out(t);
            delete t;
            return st;
        }
        bool first_launch = true;
        for (size_t c = 0; c + 1 < b->chunk_starts.size() && use_buckets; ++c) {
            if (!first_launch) TIMED(ctx, "clamp", clamp());
            first_launch = false;
            const BankDev bv = bank_view(b, b->chunk_starts[c], b->chunk_starts[c + 1], keep_bits);
            CK(ctx, cudaMemsetAsync(bk.d.fill, 0, (uint64_t)bk.d.n_buckets * bk.d.stripes * 8, ctx->stream));
            if (inline_gate)
                TIMED(ctx, "pass2_emit", launch_emit_ladder(nw, launch_cfg_persistent(ctx, ctx->block_emit, ctx->grid_pass2), bv,
                                                            p->k, lad->bits, lad->log2w, p->t_solid, td, bk.d,
                                                            emit_form(ctx, nw)));
            else
                TIMED(ctx, "pass2_emit", launch_emit(nw, L, bv, p->k, bm, 1, td, bk.d));
            if (!filter && ctx->upsert_all) {
                // every bucket in one persistent launch
                CK(ctx, cudaMemsetAsync(bk.work, 0, 8, ctx->stream));
                TIMED(ctx, "pass2_upsert", launch_upsert_all(nw, L, bk.d, 1, 1, td, ctx->d_status, bk.work, ctx->upsert_all));
            } else {
                for (uint32_t bu = 0; bu < bk.d.n_buckets; ++bu) {
                    if (filter) {
                        CK(ctx, cudaMemsetAsync(flt.cnt, 0, (1ULL << flt.log2m) * 4, ctx->stream));
                        TIMED(ctx, "pass2_count", launch_count_records(nw, L, bk.d, bu, flt));
                    }
                    if (late_table && bu == 0) {
                        st = size_filtered_table(t, flt, bk.d.n_buckets, cap);
                        if (st) {
                            table_free_out(t);
                            delete t;
                            return st;
                        }
                        td = table_dev(t);
                    }
                    TIMED(ctx, "pass2_upsert", launch_upsert(nw, L, bk.d, bu, 1, 1, td, ctx->d_status, flt, ctx->upsert_queue));
                }
            }
        }
        uint32_t ovf = use_buckets ? 0 : 1;  // without buckets every chunk takes the direct sweep
        t->filtered = false;
        t->skipped_pushes = 0;
        if (use_buckets) {
            CK(ctx, cudaMemcpyAsync(ctx->h_pinned, bk.overflow, 4, cudaMemcpyDeviceToHost, ctx->stream));
            if (filter) CK(ctx, cudaMemcpyAsync((char*)ctx->h_pinned + 8, flt.skipped, 8, cudaMemcpyDeviceToHost, ctx->stream));
            CK(ctx, cudaStreamSynchronize(ctx->stream));
            ovf = *(uint32_t*)ctx->h_pinned;
            if (filter && !ovf) {
                t->filtered = true;
                t->skipped_pushes = *(uint64_t*)((char*)ctx->h_pinned + 8);
            }
        }
        if (ovf && max_records) {
            st = need_bitmap();
            if (st) {
                table_free_storage(t);
                table_free_out(t);
                delete t;
                return st;
            }
            if (use_buckets) {
                // A stripe ran out of room: recount every chunk with the direct sweep.
                table_free_storage(t);
                st = table_alloc(t, cap, contigs != nullptr);
                if (st) {
                    table_free_out(t);
                    delete t;
                    return st;
                }
                td = table_dev(t);
            }
            for (size_t c = 0; c + 1 < b->chunk_starts.size(); ++c) {
                if (c > 0) TIMED(ctx, "clamp", clamp());
                TIMED(ctx, "pass2_direct", launch_pass2_sweep(nw, L, bank_view(b, b->chunk_starts[c], b->chunk_starts[c + 1], keep_bits),
                                                              p->k, bm, 1, 0, t->cap, 1, 1, td, ctx->d_status));
            }
        }
        if (contigs) {
            // +1000 per edge push and +100 cov (build.rs:203-240)
            for (size_t c = 0; c + 1 < contigs->chunk_starts.size(); ++c) {
                TIMED(ctx, "clamp", clamp());
                TIMED(ctx, "pass2_contigs",
                      launch_pass2_sweep(nw, L, bank_view(contigs, contigs->chunk_starts[c], contigs->chunk_starts[c + 1], nullptr),
                                         p->k, nullptr, 0, 0, t->cap, 1000, 100, td, ctx->d_status));
            }
        }
        uint32_t bits = 0;
        st = ctx_check_status(ctx, &bits);
        if (st) {
            table_free_storage(t);
            table_free_out(t);
            delete t;
            return st;
        }
        if (bits & ST_SPIN_TIMEOUT) {
            table_free_storage(t);
            table_free_out(t);
            delete t;
            return set_err(ctx, FBK_ERR_TIMEOUT, "solid table: a bounded wait for a key publication gave up");
        }
        if (!(bits & ST_TABLE_FULL)) {
            st = table_convert(t, nullptr, nullptr, nullptr, 0);
            if (st) {
                table_free_storage(t);
                table_free_out(t);
                delete t;
                return st;
            }
            *out = t;
            return FBK_OK;
        }
        table_free_storage(t);
        cap *= 2;
    }
    table_free_out(t);
    delete t;
    return set_err(ctx, FBK_ERR_TABLE_FULL, "solid table still full after growing it 3 times");
}

static fbk_status contig_bank_opt(fbk_ctx* ctx, const uint8_t* ascii, const uint64_t* offs, uint64_t n, fbk_bank** out) {
    *out = nullptr;
    if (n == 0) return FBK_OK;
    if (!ascii || !offs) return set_err(ctx, FBK_ERR_INVALID, "contigs: null buffers");
    return contig_bank(ctx, ascii, offs, n, out);
}

FBK_API fbk_status fbk_solid_build(fbk_ctx* ctx, const fbk_bank* b, const fbk_cms* cms, const fbk_build_params* p,
                                   const fbk_subsample* ss, const uint8_t* contig_ascii, const uint64_t* contig_offs,
                                   uint64_t n_contigs, fbk_table** out) {
    if (!ctx || !b || !cms || !p || !out) return FBK_ERR_INVALID;
    CK(ctx, cudaSetDevice(ctx->device));
    CK(ctx, bank_wait(ctx, b));
    uint64_t* keep = nullptr;
    fbk_status st = make_keep_bits(ctx, b, ss, &keep);
    if (st) return st;
    fbk_bank* cb = nullptr;
    st = contig_bank_opt(ctx, contig_ascii, contig_offs, n_contigs, &cb);
    uint64_t distinct = 0;
    if (st == FBK_OK && !p->table_log2_cap) st = cms_distinct(cms, &distinct);
    if (st == FBK_OK) st = solid_build_impl(ctx, b, cms, p, keep, cb, distinct + (cb ? cb->n_bases : 0), out);
    cudaStreamSynchronize(ctx->stream);
    if (cb) fbk_bank_release(cb);
    dev_free(ctx, keep);
    return st;
}

// Build front end when the caller does not ask for the sketch: pass 1 keeps only
// the gate pass 2 reads (a t_solid-level ladder, fbk_k_ladder.cu) in one sweep per read
// chunk, the solidity bitmap takes one sweep, pass 2 and the conversion are unchanged.
static fbk_status build_front_ladder(fbk_ctx* ctx, const fbk_bank* b, const fbk_build_params* p, const fbk_subsample* ss,
                                     uint32_t log2w, fbk_table** out) {
    const int nw = nw_of(p->key_bits);
    if (!nw || p->k < 1 || p->k > max_k_of(p->key_bits)) return set_err(ctx, FBK_ERR_INVALID, "k out of range for key_bits");
    if (log2w < 1 || log2w > 30) return set_err(ctx, FBK_ERR_INVALID, "cms_log2_width out of range");
    Ladder lad;
    lad.log2w = log2w;
    const uint64_t lad_bytes = (uint64_t)p->t_solid * (4ULL << log2w) / 8 + 256;
    lad.bits = (uint32_t*)dev_alloc(ctx, lad_bytes);
    uint32_t* hll = (uint32_t*)dev_alloc(ctx, 4096 * 4);
    uint64_t* keep = nullptr;
    fbk_status st = (!lad.bits || !hll) ? set_err(ctx, FBK_ERR_OOM, "sketch gate") : FBK_OK;
    if (st == FBK_OK) st = make_keep_bits(ctx, b, ss, &keep);
    if (st == FBK_OK) {
        cudaError_t e = cudaMemsetAsync(lad.bits, 0, lad_bytes, ctx->stream);
        if (e == cudaSuccess) e = cudaMemsetAsync(hll, 0, 4096 * 4, ctx->stream);
        if (e != cudaSuccess) st = cuda_err(ctx, e, "sketch gate clear");
    }
    Launch L = launch_cfg_persistent(ctx, ctx->block_pass1, ctx->grid_pass1);
    for (size_t c = 0; st == FBK_OK && c + 1 < b->chunk_starts.size(); ++c) {
        TimedLaunch tl;
        time_begin(ctx, "pass1", tl);
        cudaError_t e = launch_ladder_pass1(nw, L, bank_view(b, b->chunk_starts[c], b->chunk_starts[c + 1], keep), p->k, lad.bits,
                                            log2w, p->t_solid, hll, ladder_form(ctx, nw));
        time_end(ctx, tl);
        if (e != cudaSuccess) st = cuda_err(ctx, e, "pass1 ladder");
    }
    uint64_t distinct = 0;
    if (st == FBK_OK && !p->table_log2_cap) {
        fbk_cms view;
        view.ctx = ctx;
        view.hll12 = hll;
        st = cms_distinct(&view, &distinct);
        view.hll12 = nullptr;
    }
    if (st == FBK_OK) st = solid_build_impl(ctx, b, nullptr, p, keep, nullptr, distinct, out, &lad);
    cudaStreamSynchronize(ctx->stream);
    dev_free(ctx, keep);
    dev_free(ctx, hll);
    dev_free(ctx, lad.bits);
    return st;
}

FBK_API fbk_status fbk_build_front(fbk_ctx* ctx, const fbk_bank* b, const fbk_build_params* p, const fbk_subsample* ss,
                                   const uint8_t* contig_ascii, const uint64_t* contig_offs, uint64_t n_contigs,
                                   fbk_table** out, fbk_cms** cms_out) {
    if (!ctx || !b || !p || !out) return FBK_ERR_INVALID;
    CK(ctx, cudaSetDevice(ctx->device));
    CK(ctx, bank_wait(ctx, b));
    uint32_t log2w = p->cms_log2_width;
    if (!log2w) {
        // build.rs:74-84: explicit genome size (floored at 50 kb), else read bases / 60
        uint64_t g = p->genome_size ? std::max<uint64_t>(p->genome_size, 50000) : std::max<uint64_t>(b->n_bases / 60, 50000);
        uint64_t w = fbk_cms_width_for_genome_size(g);
        log2w = 0;
        while ((1ULL << log2w) < w) ++log2w;
    }
    const uint32_t cap = p->counter_bits == 4 ? 15u : 0xFFFFu;
    if (!cms_out && n_contigs == 0 && ctx->sketch_mode == 1 && p->t_solid >= 1 && p->t_solid <= LADDER_MAX_LEVELS &&
        p->t_solid <= cap && p->counter_bits != 0 && (p->counter_bits == 4 || p->counter_bits == 16))
        return build_front_ladder(ctx, b, p, ss, log2w, out);
    fbk_cms* cms = nullptr;
    fbk_status st = fbk_cms_create(ctx, log2w, p->counter_bits, &cms);
    if (st) return st;
    uint64_t* keep = nullptr;
    fbk_bank* cb = nullptr;
    st = make_keep_bits(ctx, b, ss, &keep);
    if (st == FBK_OK) st = contig_bank_opt(ctx, contig_ascii, contig_offs, n_contigs, &cb);
    if (st == FBK_OK) st = pass1_impl(cms, b, p->k, p->key_bits, keep, 1);
    if (st == FBK_OK && cb) st = pass1_impl(cms, cb, p->k, p->key_bits, nullptr, 10);
    uint64_t distinct = 0;
    if (st == FBK_OK && !p->table_log2_cap) st = cms_distinct(cms, &distinct);
    if (st == FBK_OK) st = solid_build_impl(ctx, b, cms, p, keep, cb, distinct, out);
    cudaStreamSynchronize(ctx->stream);
    if (cb) fbk_bank_release(cb);
    dev_free(ctx, keep);
    if (st == FBK_OK && cms_out) *cms_out = cms;
    else fbk_cms_release(cms);
    return st;
}

FBK_API fbk_status fbk_table_info(const fbk_table* t, uint64_t* n_keys, uint64_t* n_solid, uint64_t* capacity) {
    if (!t) return FBK_ERR_INVALID;
    if (n_keys) *n_keys = t->n_keys;
    if (n_solid) *n_solid = t->n_solid;
    if (capacity) *capacity = t->cap;
    return FBK_OK;
}

FBK_API fbk_status fbk_table_export(fbk_table* t, uint64_t* keys, uint16_t* cov, uint8_t* mask, uint64_t cap, uint64_t* n_out) {
    if (!t || !n_out) return FBK_ERR_INVALID;
    fbk_ctx* ctx = t->ctx;
    uint64_t n = std::min(cap, t->n_solid);
    if (n && (!keys || !cov || !mask)) return FBK_ERR_INVALID;
    if (n) {
        CK(ctx, copy_d2h(ctx, keys, t->out_keys, n * 8 * t->nw));
        CK(ctx, copy_d2h(ctx, cov, t->out_cov, n * 2));
        CK(ctx, copy_d2h(ctx, mask, t->out_mask, n));
    }
    *n_out = t->n_solid;
    return FBK_OK;
}

FBK_API fbk_status fbk_table_export_async(fbk_table* t, uint64_t* keys, uint16_t* cov, uint8_t* mask, uint64_t cap, uint64_t* n_out) {
    if (!t || !n_out) return FBK_ERR_INVALID;
    fbk_ctx* ctx = t->ctx;
    uint64_t n = std::min(cap, t->n_solid);
    if (n && (!keys || !cov || !mask)) return FBK_ERR_INVALID;
    if (n && (!host_page_locked(keys) || !host_page_locked(cov) || !host_page_locked(mask)))
        return set_err(ctx, FBK_ERR_INVALID, "fbk_table_export_async: the row buffers must be page-locked host memory");
    CK(ctx, cudaSetDevice(ctx->device));
    cudaStream_t cs = nullptr;
    CK(ctx, copy_stream_of(ctx, &cs));
    if (!t->converted) CK(ctx, cudaEventCreateWithFlags(&t->converted, cudaEventDisableTiming));
    if (!t->exported) CK(ctx, cudaEventCreateWithFlags(&t->exported, cudaEventDisableTiming));
    // the copies start once the work queued on the context's stream (the conversion) is done
    CK(ctx, cudaEventRecord(t->converted, ctx->stream));
    CK(ctx, cudaStreamWaitEvent(cs, t->converted, 0));
    if (n) {
        CK(ctx, cudaMemcpyAsync(keys, t->out_keys, n * 8 * t->nw, cudaMemcpyDeviceToHost, cs));
        CK(ctx, cudaMemcpyAsync(cov, t->out_cov, n * 2, cudaMemcpyDeviceToHost, cs));
        CK(ctx, cudaMemcpyAsync(mask, t->out_mask, n, cudaMemcpyDeviceToHost, cs));
    }
    CK(ctx, cudaEventRecord(t->exported, cs));
    *n_out = t->n_solid;
    return FBK_OK;
}

FBK_API fbk_status fbk_table_export_wait(fbk_table* t) {
    if (!t) return FBK_ERR_INVALID;
    if (t->exported) CK(t->ctx, cudaEventSynchronize(t->exported));
    return FBK_OK;
}

FBK_API fbk_status fbk_table_export_acc(fbk_table* t, uint64_t* keys, uint16_t* cov, uint16_t* edges, uint64_t cap, uint64_t* n_out) {
    if (!t || !n_out) return FBK_ERR_INVALID;
    fbk_ctx* ctx = t->ctx;
    if (!t->cnt) return set_err(ctx, FBK_ERR_INVALID, "the accumulator slots of this table were released after conversion");
    uint64_t n = std::min(cap, t->n_keys);
    uint64_t* dk = nullptr;
    uint16_t *dc = nullptr, *de = nullptr;
    if (n) {
        if (!keys || !cov || !edges) return FBK_ERR_INVALID;
        dk = (uint64_t*)dev_alloc(ctx, n * 8 * t->nw);
        dc = (uint16_t*)dev_alloc(ctx, n * 2);
        de = (uint16_t*)dev_alloc(ctx, n * 16);
        if (!dk || !dc || !de) {
            dev_free(ctx, dk);
            dev_free(ctx, dc);
            dev_free(ctx, de);
            return set_err(ctx, FBK_ERR_OOM, "accumulator export buffers");
        }
    }
    fbk_status st = table_convert(t, dk, dc, de, n);
    if (st == FBK_OK && n) {
        cudaError_t e = copy_d2h(ctx, keys, dk, n * 8 * t->nw);
        if (e == cudaSuccess) e = copy_d2h(ctx, cov, dc, n * 2);
        if (e == cudaSuccess) e = copy_d2h(ctx, edges, de, n * 16);
        if (e != cudaSuccess) st = cuda_err(ctx, e, "accumulator export");
    }
    dev_free(ctx, dk);
    dev_free(ctx, dc);
    dev_free(ctx, de);
    *n_out = t->n_keys;
    return st;
}

FBK_API fbk_status fbk_table_flags(const fbk_table* t, uint32_t* flags) {
    if (!t || !flags) return FBK_ERR_INVALID;
    *flags = t->filtered ? FBK_TABLE_ACC_FILTERED : 0u;
    return FBK_OK;
}

FBK_API fbk_status fbk_table_pushes(const fbk_table* t, uint64_t* pushes) {
    if (!t || !pushes) return FBK_ERR_INVALID;
    *pushes = t->pushes;
    return FBK_OK;
}

FBK_API fbk_status fbk_table_export_acc_owned(fbk_table* t, uint32_t world, uint64_t* rows, uint64_t cap_rows,
                                              uint64_t* owner_counts) {
    if (!t || !owner_counts || world == 0 || world > 65536) return FBK_ERR_INVALID;
    fbk_ctx* ctx = t->ctx;
    if (!t->cnt) return set_err(ctx, FBK_ERR_INVALID, "the accumulator slots of this table were released after conversion");
    CK(ctx, cudaSetDevice(ctx->device));
    const uint64_t n = t->n_keys;
    if (n > cap_rows || (n && !rows)) return set_err(ctx, FBK_ERR_INVALID, "owner rows: buffer smaller than the accumulator");
    const int nw = (int)t->nw;
    uint64_t* dk = n ? (uint64_t*)dev_alloc(ctx, n * 8 * nw) : nullptr;
    uint16_t* dc = n ? (uint16_t*)dev_alloc(ctx, n * 2) : nullptr;
    uint16_t* de = n ? (uint16_t*)dev_alloc(ctx, n * 16) : nullptr;
    unsigned long long* cnt = (unsigned long long*)dev_alloc(ctx, (uint64_t)world * 16);
    fbk_status st = (n && (!dk || !dc || !de)) || !cnt ? set_err(ctx, FBK_ERR_OOM, "owner rows: staging") : FBK_OK;
    if (st == FBK_OK) st = table_convert(t, dk, dc, de, n);
    if (st == FBK_OK) {
        const Launch L = launch_cfg(ctx, 256, 0);
        cudaError_t e = cudaMemsetAsync(cnt, 0, (uint64_t)world * 8, ctx->stream);
        if (e == cudaSuccess) e = launch_owner_hist(nw, L, dk, n, world, cnt);
        std::vector<unsigned long long> h(world);
        if (e == cudaSuccess) e = cudaMemcpyAsync(h.data(), cnt, (uint64_t)world * 8, cudaMemcpyDeviceToHost, ctx->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
        if (e == cudaSuccess) {
            std::vector<unsigned long long> start(world);
            unsigned long long acc = 0;
            for (uint32_t o = 0; o < world; ++o) {
                start[o] = acc;
                acc += h[o];
                owner_counts[o] = h[o];
            }
            unsigned long long* cursor = cnt + world;
            e = cudaMemcpyAsync(cursor, start.data(), (uint64_t)world * 8, cudaMemcpyHostToDevice, ctx->stream);
            if (e == cudaSuccess) e = launch_owner_scatter(nw, L, dk, de, n, world, cursor, rows);
            if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
        }
        if (e != cudaSuccess) st = cuda_err(ctx, e, "owner rows");
    }
    cudaStreamSynchronize(ctx->stream);
    dev_free(ctx, dk);
    dev_free(ctx, dc);
    dev_free(ctx, de);
    dev_free(ctx, cnt);
    return st;
}

FBK_API fbk_status fbk_table_from_acc_rows(fbk_ctx* ctx, uint32_t k, uint32_t key_bits, uint32_t min_trans_cov,
                                           const uint64_t* rows, uint64_t n, fbk_table** out) {
    if (!ctx || !out || (n && !rows)) return FBK_ERR_INVALID;
    *out = nullptr;
    const int nw = nw_of(key_bits);
    if (!nw || k < 1 || k > max_k_of(key_bits)) return set_err(ctx, FBK_ERR_INVALID, "k out of range for key_bits");
    if (min_trans_cov > 0xFFFF) return set_err(ctx, FBK_ERR_INVALID, "min_trans_cov must fit u16");
    CK(ctx, cudaSetDevice(ctx->device));
    fbk_table* t = new fbk_table();
    t->ctx = ctx;
    t->nw = (uint32_t)nw;
    t->k = k;
    t->min_trans_cov = min_trans_cov;
    uint64_t cap = std::max<uint64_t>(1024, (uint64_t)((double)n / ctx->load_factor) + 1024);
    for (int attempt = 0; attempt < 4; ++attempt) {
        fbk_status st = table_alloc(t, cap, false);
        if (st == FBK_OK && !t->out_keys) {
            const uint64_t oc = n + 4096;  // converted rows are a subset of the keys
            t->out_keys = (uint64_t*)dev_alloc(ctx, oc * 8 * nw);
            t->out_cov = (uint16_t*)dev_alloc(ctx, oc * 2);
            t->out_mask = (uint8_t*)dev_alloc(ctx, oc);
            if (!t->out_keys || !t->out_cov || !t->out_mask) table_free_out(t);
            else t->out_cap = oc;
        }
        if (st == FBK_OK) {
            cudaError_t e = cudaMemsetAsync(ctx->d_status, 0, 4, ctx->stream);
            if (e == cudaSuccess)
                e = launch_rows_upsert(nw, launch_cfg(ctx, 256, 0), rows, n, table_dev(t), ctx->d_status);
            if (e != cudaSuccess) st = cuda_err(ctx, e, "rows upsert");
        }
        uint32_t bits = 0;
        if (st == FBK_OK) st = ctx_check_status(ctx, &bits);
        if (st == FBK_OK && (bits & ST_SPIN_TIMEOUT))
            st = set_err(ctx, FBK_ERR_TIMEOUT, "solid table: a bounded wait for a key publication gave up");
        if (st == FBK_OK && !(bits & ST_TABLE_FULL)) {
            st = table_convert(t, nullptr, nullptr, nullptr, 0);
            if (st == FBK_OK) {
                *out = t;
                return FBK_OK;
            }
        }
        table_free_storage(t);
        if (st != FBK_OK) {
            table_free_out(t);
            delete t;
            return st;
        }
        cap *= 2;
    }
    table_free_out(t);
    delete t;
    return set_err(ctx, FBK_ERR_TABLE_FULL, "solid table still full after growing it 3 times");
}

FBK_API fbk_status fbk_table_acc_digest(fbk_table* t, uint64_t* digest, uint64_t* n_keys) {
    if (!t || !digest) return FBK_ERR_INVALID;
    fbk_ctx* ctx = t->ctx;
    if (!t->cnt) return set_err(ctx, FBK_ERR_INVALID, "the accumulator slots of this table were released after conversion");
    CK(ctx, cudaSetDevice(ctx->device));
    fbk_status st = table_convert(t, nullptr, nullptr, nullptr, 0, digest);
    if (st == FBK_OK && n_keys) *n_keys = t->n_keys;
    return st;
}

FBK_API fbk_status fbk_table_digest(fbk_table* t, uint64_t* digest, uint64_t* n_solid) {
    if (!t || !digest) return FBK_ERR_INVALID;
    *digest = t->digest;
    if (n_solid) *n_solid = t->n_solid;
    return FBK_OK;
}

FBK_API fbk_status fbk_table_release(fbk_table* t) {
    if (!t) return FBK_OK;
    cudaStreamSynchronize(t->ctx->stream);
    for (cudaEvent_t* e : {&t->exported, &t->converted})
        if (*e) {
            cudaEventSynchronize(*e);
            cudaEventDestroy(*e);
        }
    table_free_storage(t);
    table_free_out(t);
    delete t;
    return FBK_OK;
}

// ===========================================================================
// subsampler, ntHash / canonical k-mer dumps
// ===========================================================================
FBK_API fbk_status fbk_subsample_mask(fbk_ctx* ctx, uint64_t n_pairs, const fbk_subsample* ss, uint64_t* keep_bits) {
    if (!ctx || !ss || (n_pairs && !keep_bits)) return FBK_ERR_INVALID;
    if (!n_pairs) return FBK_OK;
    const uint64_t nw = (n_pairs + 63) / 64;
    uint64_t* d = (uint64_t*)dev_alloc(ctx, nw * 8);
    if (!d) return set_err(ctx, FBK_ERR_OOM, "subsample bitmap");
    cudaError_t e;
    {
        TimedLaunch tl;
        time_begin(ctx, "subsample", tl);
        e = launch_subsample_mask(launch_cfg(ctx, 256, 0), n_pairs, ss->factor, ss->seed, d);
        time_end(ctx, tl);
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(keep_bits, d, nw * 8, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    dev_free(ctx, d);
    if (e != cudaSuccess) return cuda_err(ctx, e, "subsample mask");
    return FBK_OK;
}

// Uploads one arena and the per-read window bases for the dump kernels.
static fbk_status dump_prep(fbk_ctx* ctx, const fbk_arena_view* arena, uint32_t k, fbk_bank** bank, uint64_t** kbase,
                            uint64_t* total) {
    fbk_status st = bank_upload_impl(ctx, arena, 1, bank);
    if (st) return st;
    std::vector<uint64_t> kb(arena->n_seqs + 1, 0);
    for (uint64_t i = 0; i < arena->n_seqs; ++i) kb[i + 1] = kb[i] + (arena->lengths[i] >= k ? arena->lengths[i] - k + 1 : 0);
    *total = kb.back();
    *kbase = (uint64_t*)dev_alloc(ctx, kb.size() * 8);
    if (!*kbase) {
        fbk_bank_release(*bank);
        return set_err(ctx, FBK_ERR_OOM, "window base offsets");
    }
    CK(ctx, cudaMemcpyAsync(*kbase, kb.data(), kb.size() * 8, cudaMemcpyHostToDevice, ctx->stream));
    CK(ctx, cudaStreamSynchronize(ctx->stream));
    return FBK_OK;
}

FBK_API fbk_status fbk_nthash_arena(fbk_ctx* ctx, const fbk_arena_view* arena, uint32_t k, uint64_t* out, uint64_t cap, uint64_t* n_out) {
    if (!ctx || !arena || !n_out || k == 0) return FBK_ERR_INVALID;
    CK(ctx, cudaSetDevice(ctx->device));
    fbk_bank* b = nullptr;
    uint64_t* kbase = nullptr;
    uint64_t total = 0;
    fbk_status st = dump_prep(ctx, arena, k, &b, &kbase, &total);
    if (st) return st;
    *n_out = total;
    if (total > cap || (total && !out)) {
        fbk_bank_release(b);
        dev_free(ctx, kbase);
        return total > cap ? set_err(ctx, FBK_ERR_INVALID, "output buffer too small") : FBK_ERR_INVALID;
    }
    uint64_t* d = (uint64_t*)dev_alloc(ctx, std::max<uint64_t>(total, 1) * 8);
    cudaError_t e = d ? cudaSuccess : cudaErrorMemoryAllocation;
    if (e == cudaSuccess) {
        TimedLaunch tl;
        time_begin(ctx, "nthash_dump", tl);
        e = launch_nthash_arena(launch_cfg(ctx, 256, 0), bank_view(b, 0, b->n_reads, nullptr), kbase, k, d);
        time_end(ctx, tl);
    }
    if (e == cudaSuccess && total) e = cudaMemcpyAsync(out, d, total * 8, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    dev_free(ctx, d);
    dev_free(ctx, kbase);
    fbk_bank_release(b);
    if (e != cudaSuccess) return cuda_err(ctx, e, "nthash dump");
    return FBK_OK;
}

FBK_API fbk_status fbk_canonical_kmers_arena(fbk_ctx* ctx, const fbk_arena_view* arena, uint32_t k, uint32_t key_bits,
                                             uint64_t* out_words, uint8_t* out_is_rc, uint64_t cap, uint64_t* n_out) {
    const int nw = nw_of(key_bits);
    if (!ctx || !arena || !n_out || !nw || k == 0 || k > max_k_of(key_bits)) return FBK_ERR_INVALID;
    CK(ctx, cudaSetDevice(ctx->device));
    fbk_bank* b = nullptr;
    uint64_t* kbase = nullptr;
    uint64_t total = 0;
    fbk_status st = dump_prep(ctx, arena, k, &b, &kbase, &total);
    if (st) return st;
    *n_out = total;
    if (total > cap || (total && (!out_words || !out_is_rc))) {
        fbk_bank_release(b);
        dev_free(ctx, kbase);
        return total > cap ? set_err(ctx, FBK_ERR_INVALID, "output buffer too small") : FBK_ERR_INVALID;
    }
    uint64_t* d = (uint64_t*)dev_alloc(ctx, std::max<uint64_t>(total, 1) * 8 * nw);
    uint8_t* dr = (uint8_t*)dev_alloc(ctx, std::max<uint64_t>(total, 1));
    cudaError_t e = (d && dr) ? cudaSuccess : cudaErrorMemoryAllocation;
    if (e == cudaSuccess) {
        TimedLaunch tl;
        time_begin(ctx, "canon_dump", tl);
        e = launch_canon_arena(nw, launch_cfg(ctx, 256, 0), bank_view(b, 0, b->n_reads, nullptr), kbase, k, d, dr);
        time_end(ctx, tl);
    }
    if (e == cudaSuccess && total) e = cudaMemcpyAsync(out_words, d, total * 8 * nw, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess && total) e = cudaMemcpyAsync(out_is_rc, dr, total, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    dev_free(ctx, d);
    dev_free(ctx, dr);
    dev_free(ctx, kbase);
    fbk_bank_release(b);
    if (e != cudaSuccess) return cuda_err(ctx, e, "canonical k-mer dump");
    return FBK_OK;
}

}  // extern "C"

// Entry points of the table and pass helpers for the multi-isolate host code.
namespace fbk {
int key_words(uint32_t key_bits) { return nw_of(key_bits); }
uint32_t key_k_max(uint32_t key_bits) { return max_k_of(key_bits); }
fbk_status keep_bits_for(fbk_ctx* ctx, const fbk_bank* b, const fbk_subsample* ss, uint64_t** bits_out) {
    return make_keep_bits(ctx, b, ss, bits_out);
}
TableDev tbl_dev(const fbk_table* t) { return table_dev(t); }
fbk_status tbl_alloc(fbk_table* t, uint64_t cap, bool with_cov) { return table_alloc(t, cap, with_cov); }
void tbl_free_storage(fbk_table* t) { table_free_storage(t); }
void tbl_free_out(fbk_table* t) { table_free_out(t); }
fbk_status tbl_convert(fbk_table* t) { return table_convert(t, nullptr, nullptr, nullptr, 0); }
fbk_status solid_build(fbk_ctx* ctx, const fbk_bank* b, const fbk_cms* cms, const fbk_build_params* p, const uint64_t* keep_bits,
                       uint64_t distinct_hint, fbk_table** out) {
    return solid_build_impl(ctx, b, cms, p, keep_bits, nullptr, distinct_hint, out);
}
fbk_status solid_build_ladder(fbk_ctx* ctx, const fbk_bank* b, uint32_t* ladder, uint32_t log2w, const fbk_build_params* p,
                              const uint64_t* keep_bits, uint64_t distinct_hint, fbk_table** out) {
    Ladder lad;
    lad.bits = ladder;
    lad.log2w = log2w;
    return solid_build_impl(ctx, b, nullptr, p, keep_bits, nullptr, distinct_hint, out, &lad);
}
}  // namespace fbk
