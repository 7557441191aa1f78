// fbk_noalloc.cu — the genome-estimator sample loop for callers that cannot
// allocate device memory.
//
// Some callers cannot call cudaMalloc: hosts whose device memory is owned by another
// runtime's allocator (a Rust or Go service with its own pool, a framework that has
// reserved the whole GPU, so a cudaMalloc of ours would fail or fragment its pool),
// and latency-critical loops that must not take the allocator's locks or trigger the
// implicit device synchronisation a cudaFree can cause.  fbk_estimate_sample_noalloc
// serves them: it needs no context and makes no allocating call.  Its scratch memory
// is the file-scope device array below, FBK_NOALLOC_SCRATCH_BYTES (8 MiB) in size,
// which every GPU that loads this library holds until the process exits.
//
// It is a blocking call: it copies the caller's host buffers to the array on the
// caller's stream, waits for the stream (cudaStreamSynchronize) and evaluates the
// estimator's checkpoints on the host.  So it cannot be recorded into a CUDA graph;
// a call made on a stream that is being captured fails (the synchronisation is
// refused there) and ends that capture.
//
// The sizes that fit: at most 20000 read pairs (40000 reads), at most 2^23 bases in
// the sample, a count-min sketch of at most 2^18 columns per row, HyperLogLog
// precision at most 14.  Larger requests are rejected with FBK_ERR_INVALID and a
// message; nothing is copied or launched for them.
//
// The first call on a device looks up the array's device address with
// cudaGetSymbolAddress (with that device current) and caches it.  Every call on a
// device shares the same array and leaves its contents behind; each call
// re-initialises every region it reads before use (the first-occurrence table, the
// register segments, the padding after the packed reads).  Calls whose GPU work
// overlaps — different streams, or different host threads without ordering — race on
// the array, so serialise them.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>

#include "fbk_device.cuh"
#include "fbk_internal.h"

namespace {

constexpr uint64_t SCRATCH_BYTES = 8ull << 20;  // FBK_NOALLOC_SCRATCH_BYTES in fbk.h
constexpr uint64_t MAX_PAIRS = 20000;
constexpr uint64_t MAX_BASES = 1ull << 23;
constexpr uint32_t MAX_LOG2W = 18;
constexpr uint32_t MAX_P = 14;
constexpr uint32_t MAX_SEGS = 1 + (MAX_PAIRS - 6000 + 1999) / 2000;  // 8

static __device__ __align__(256) unsigned char g_scratch[SCRATCH_BYTES];

constexpr int MAX_DEVICES = 64;
std::mutex g_mu;
unsigned char* g_ptr[MAX_DEVICES] = {};
int g_sms[MAX_DEVICES] = {};

// Exclusive prefix of the per-read window counts (one block; n <= 40000).
__global__ void k_window_bases(const uint32_t* __restrict__ len, uint64_t n, uint32_t k, uint64_t* __restrict__ kbase) {
    __shared__ uint64_t s_carry;
    __shared__ uint64_t s_warp[32];
    if (threadIdx.x == 0) s_carry = 0;
    __syncthreads();
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (uint64_t base = 0; base < n; base += blockDim.x) {
        const uint64_t i = base + threadIdx.x;
        const uint64_t v = (i < n && len[i] >= k) ? (uint64_t)(len[i] - k + 1) : 0;
        uint64_t x = v;
        for (int o = 1; o < 32; o <<= 1) {
            const uint64_t y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= (uint32_t)o) x += y;
        }
        if (lane == 31) s_warp[warp] = x;
        __syncthreads();
        if (warp == 0) {
            uint64_t w = lane < (blockDim.x >> 5) ? s_warp[lane] : 0;
            for (int o = 1; o < 32; o <<= 1) {
                const uint64_t y = __shfl_up_sync(0xffffffffu, w, o);
                if (lane >= (uint32_t)o) w += y;
            }
            if (lane < (blockDim.x >> 5)) s_warp[lane] = w;
        }
        __syncthreads();
        const uint64_t before = (warp ? s_warp[warp - 1] : 0) + s_carry;
        if (i < n) kbase[i] = before + x - v;
        __syncthreads();
        if (threadIdx.x == blockDim.x - 1) s_carry = before + x;
        __syncthreads();
    }
    if (threadIdx.x == 0) kbase[n] = s_carry;
}

// u32 registers of one segment -> u8 (register values are at most 65 - p).
__global__ void k_narrow(const uint32_t* __restrict__ src, uint8_t* __restrict__ dst, uint64_t m) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m; i += (uint64_t)gridDim.x * blockDim.x)
        dst[i] = (uint8_t)src[i];
}

// compute_dynamic_kmers (src/ingest/estimator.rs:104-161) into a fixed array.
int ladder(uint64_t median_len, uint64_t* out) {
    const uint64_t min_k = median_len < 75 ? 21 : 31;
    const uint64_t effective_len = (median_len * 16) / 10;
    uint64_t max_k = fbk::f64_to_u64_sat((double)effective_len * 0.85);
    max_k = std::min<uint64_t>(std::max(max_k, min_k), 127);
    if (max_k % 2 == 0) max_k -= 1;
    int n = 0;
    if (max_k <= min_k) {
        out[n++] = min_k;
        return n;
    }
    if (median_len >= 100) {
        out[n++] = min_k;
        if (max_k > 73) out[n++] = 63;
        out[n++] = max_k;
        return n;
    }
    uint64_t step = (max_k - min_k) / 2;
    if (step % 2 == 1) step += 1;
    if (step < 6) step = 6;
    for (uint64_t k = min_k; k <= max_k && n < 8; k += step) out[n++] = k;
    if (out[n - 1] != max_k && max_k > out[n - 1]) {
        if (max_k - out[n - 1] >= 10 && n < 8) out[n++] = max_k;
        else out[n - 1] = max_k;
    }
    return n;
}

inline uint64_t up256(uint64_t x) { return (x + 255) & ~255ull; }

}  // namespace

using namespace fbk;

extern "C" FBK_API fbk_status fbk_estimate_sample_noalloc(int device, void* stream_handle, const fbk_arena_view* sample,
                                                          uint64_t n_pairs, const fbk_count_stats* stats,
                                                          const fbk_estimator_params* prm, fbk_genome_estimate* out,
                                                          uint8_t* regs_total, uint8_t* regs_solid, char* err,
                                                          size_t errlen) {
    auto fail = [&](fbk_status st, const char* msg) {
        if (err && errlen) snprintf(err, errlen, "%s", msg);
        return st;
    };
    if (!sample || !stats || !prm || !out) return fail(FBK_ERR_INVALID, "null argument");
    if (device < 0 || device >= MAX_DEVICES) return fail(FBK_ERR_INVALID, "device index out of range");
    const uint32_t k = prm->k, p = prm->hll_p, log2w = prm->cms_log2_width;
    if (k == 0 || p < 4 || log2w < 3) return fail(FBK_ERR_INVALID, "estimator parameters out of range");
    if (p > MAX_P) return fail(FBK_ERR_INVALID, "hll_p above 14 does not fit the fixed scratch");
    if (log2w > MAX_LOG2W) return fail(FBK_ERR_INVALID, "cms_log2_width above 18 does not fit the fixed scratch");
    if (sample->n_seqs < 2 * n_pairs) return fail(FBK_ERR_INVALID, "sample holds fewer than 2*n_pairs reads");
    const uint64_t sample_target = std::min(std::min(prm->max_pairs, prm->sample_cap), stats->exact_read_pairs);
    const uint64_t n_use = std::min(sample_target, n_pairs);
    if (n_use == 0) return fail(FBK_ERR_EMPTY, "Input FASTQ files contain 0 valid read pairs");
    if (n_use > MAX_PAIRS) return fail(FBK_ERR_INVALID, "more than 20000 sampled pairs do not fit the fixed scratch");
    const uint64_t n_reads = 2 * n_use;

    // Sample extent, m_sample at every checkpoint and the window total, without any
    // host or device allocation.
    uint64_t end_base = 0, windows = 0;
    uint64_t m_at[MAX_SEGS + 1] = {};
    for (uint64_t r = 0; r < n_reads; ++r) {
        const uint32_t L = sample->lengths[r];
        if (L && sample->offsets[r] + L > sample->n_words * 32) return fail(FBK_ERR_INVALID, "sequence extends past the arena data");
        end_base = std::max<uint64_t>(end_base, sample->offsets[r] + L);
        windows += L >= k ? L - k + 1 : 0;
        if (r & 1) {
            const uint64_t pc = (r >> 1) + 1;  // pairs done
            if (pc >= 6000 && (pc - 6000) % 2000 == 0) m_at[(pc - 6000) / 2000] = windows;
        }
    }
    if (end_base > MAX_BASES) return fail(FBK_ERR_INVALID, "more than 2^23 sample bases do not fit the fixed scratch");
    if (windows >= 0xFFFFFFFFull) return fail(FBK_ERR_INVALID, "estimator sample holds 2^32 or more k-mers");
    const uint64_t m_final = windows;
    const uint64_t n_words = (end_base + 31) / 32;
    const uint64_t m = 1ull << p;
    const uint32_t n_segs = n_use <= 6000 ? 1u : (uint32_t)(1 + (n_use - 6000 + 1999) / 2000);

    // scratch layout
    const uint64_t o_data = 0;
    const uint64_t o_off = o_data + up256((n_words + 8) * 8);
    const uint64_t o_len = o_off + up256(n_reads * 8);
    const uint64_t o_kbase = o_len + up256(n_reads * 4);
    const uint64_t o_first = o_kbase + up256((n_reads + 1) * 8);
    const uint64_t o_rt = o_first + up256((4ull << log2w) * 4);
    const uint64_t o_rs = o_rt + up256((uint64_t)n_segs * m * 4);
    const uint64_t o_sums = o_rs + up256((uint64_t)n_segs * m * 4);
    const uint64_t o_zeros = o_sums + up256(2ull * n_segs * 8);
    const uint64_t o_u8 = o_zeros + up256(2ull * n_segs * 8);
    const uint64_t total = o_u8 + up256(2 * m);
    if (total > SCRATCH_BYTES) return fail(FBK_ERR_INVALID, "request does not fit the 8 MiB fixed scratch");

    // once per device, with that device current: the array's device address
    int prev = -1;
    if (cudaGetDevice(&prev) != cudaSuccess) return fail(FBK_ERR_NO_DEVICE, "cudaGetDevice failed");
    if (cudaSetDevice(device) != cudaSuccess) return fail(FBK_ERR_NO_DEVICE, "cudaSetDevice failed");
    unsigned char* base;
    int sms;
    {
        std::lock_guard<std::mutex> g(g_mu);
        if (!g_ptr[device]) {
            void* ptr = nullptr;
            cudaError_t e = cudaGetSymbolAddress(&ptr, g_scratch);
            if (e != cudaSuccess || !ptr) {
                cudaSetDevice(prev);
                return fail(FBK_ERR_CUDA, "cudaGetSymbolAddress of the fixed scratch failed");
            }
            int n = 0;
            if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) n = 1;
            g_ptr[device] = (unsigned char*)ptr;
            g_sms[device] = n;
        }
        base = g_ptr[device];
        sms = g_sms[device];
    }
    cudaStream_t st = (cudaStream_t)stream_handle;
    uint64_t* d_data = (uint64_t*)(base + o_data);
    uint64_t* d_off = (uint64_t*)(base + o_off);
    uint32_t* d_len = (uint32_t*)(base + o_len);
    uint64_t* d_kbase = (uint64_t*)(base + o_kbase);
    uint32_t* d_first = (uint32_t*)(base + o_first);
    uint32_t* d_rt = (uint32_t*)(base + o_rt);
    uint32_t* d_rs = (uint32_t*)(base + o_rs);
    double* d_sums = (double*)(base + o_sums);
    unsigned long long* d_zeros = (unsigned long long*)(base + o_zeros);
    uint8_t* d_u8 = base + o_u8;

    cudaError_t e = cudaMemcpyAsync(d_data, sample->data, n_words * 8, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(d_data + n_words, 0, 8 * 8, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_off, sample->offsets, n_reads * 8, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_len, sample->lengths, n_reads * 4, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(d_first, 0xFF, (4ull << log2w) * 4, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(d_rt, 0, (uint64_t)n_segs * m * 4, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(d_rs, 0, (uint64_t)n_segs * m * 4, st);
    if (e == cudaSuccess) {
        k_window_bases<<<1, 1024, 0, st>>>(d_len, n_reads, k, d_kbase);
        e = cudaGetLastError();
    }
    BankDev bv;
    bv.data = d_data;
    bv.off = d_off;
    bv.len = d_len;
    bv.pair_idx = nullptr;
    bv.keep_bits = nullptr;
    bv.r_begin = 0;
    bv.r_end = n_reads;
    Launch L{};
    L.grid = sms * 4;
    L.block = 256;
    L.stream = st;
    L.sms = sms;
    if (e == cudaSuccess) e = launch_est_firstpos(L, bv, d_kbase, k, d_first, log2w);
    if (e == cudaSuccess) e = launch_est_hll(L, bv, d_kbase, k, d_first, log2w, p, n_segs, d_rt, d_rs);
    if (e == cudaSuccess) e = launch_est_prefix(L, d_rt, p, n_segs);
    if (e == cudaSuccess) e = launch_est_prefix(L, d_rs, p, n_segs);
    if (e == cudaSuccess) e = launch_est_sums(L, d_rt, d_rs, p, n_segs, d_sums, d_zeros);
    double h_sums[2 * MAX_SEGS];
    unsigned long long h_zeros[2 * MAX_SEGS];
    if (e == cudaSuccess) e = cudaMemcpyAsync(h_sums, d_sums, 2ull * n_segs * 8, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(h_zeros, d_zeros, 2ull * n_segs * 8, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
        cudaSetDevice(prev);
        return fail(FBK_ERR_CUDA, cudaGetErrorString(e));
    }

    // checkpoints and post-math: src/ingest/estimator.rs:366-439
    auto est = [&](int which, uint32_t seg) { return hll_estimate_from_sum(h_sums[which * n_segs + seg], h_zeros[which * n_segs + seg], p); };
    uint32_t final_seg = n_segs - 1;
    uint64_t pairs_done = n_use, m_sample = m_final;
    for (uint32_t j = 0; j < n_segs; ++j) {
        const uint64_t P = 6000 + 2000ull * j;
        if (P > n_use) break;
        const uint64_t u1 = f64_to_u64_sat(std::round(est(0, j)));
        const uint64_t u2 = f64_to_u64_sat(std::round(est(1, j)));
        const uint64_t e1 = u1 > u2 ? u1 - u2 : 0;
        const uint64_t m_tr = m_at[j] > e1 ? m_at[j] - e1 : 0;
        const double lam = u2 > 0 ? (double)m_tr / (double)u2 : 0.0;
        if (lam >= 15.0) {
            final_seg = j;
            pairs_done = P;
            m_sample = m_at[j];
            break;
        }
    }
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
    memset(out, 0, sizeof(*out));
    out->genome_size = est_g;
    out->exact_read_pairs = stats->exact_read_pairs;
    out->total_bases = stats->total_bases;
    out->median_read_len = stats->median_read_len;
    out->max_read_len = stats->max_read_len;
    out->estimated_cov = estimated_cov;
    out->subsample_factor = ssf;
    out->n_kmers = (uint64_t)ladder(stats->median_read_len, out->kmers);
    out->confidence = conf;
    out->u_ge_1 = u_ge_1;
    out->u_ge_2 = u_ge_2;
    out->sample_kmer_depth = lambda_s;
    out->pairs_sampled = pairs_done;
    out->m_sample = m_sample;

    for (int which = 0; which < 2 && e == cudaSuccess; ++which) {
        uint8_t* dst = which == 0 ? regs_total : regs_solid;
        if (!dst) continue;
        const uint32_t* src = (which == 0 ? d_rt : d_rs) + (uint64_t)final_seg * m;
        k_narrow<<<std::max(1, sms), 256, 0, st>>>(src, d_u8 + which * m, m);
        e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaMemcpyAsync(dst, d_u8 + which * m, m, cudaMemcpyDeviceToHost, st);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    cudaSetDevice(prev);
    if (e != cudaSuccess) return fail(FBK_ERR_CUDA, cudaGetErrorString(e));
    return FBK_OK;
}
