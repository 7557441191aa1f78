// fbk_ingest_dev.cu — ingest_reads_ext_with_seed (src/ingest/trim_merge.rs:307-417) on
// the device: the two FASTQ files' bytes in, a device ReadBank out.
//
//   1. line index: each block counts the newlines of a 4 KiB chunk; after a host prefix
//      over chunks, each block writes the positions of its newlines (block scan);
//   2. records: line 4r is the header of record r, 4r+1 its sequence, 4r+3 its
//      qualities (plain 4-line FASTQ, the form the host reader and the generator use;
//      a trailing '\r' is dropped from every line);
//   3. one thread per pair applies the subsampler, adapter and quality trimming and
//      the overlap merge (trim_merge.rs:17-238) and records what the pair becomes;
//   4. after a host prefix over pairs, one thread per pair writes its reads' 2-bit
//      codes (ASCII_TO_2BIT, bitseq.rs:67-81) into the arenas (merged, pe_forward,
//      pe_reverse), concatenated as a device bank.
// The result equals the host ingest byte for byte (tests compare the banks).
#include <algorithm>
#include <cstring>
#include <vector>

#include "fbk_device.cuh"
#include "fbk_internal.h"

using namespace fbk;

namespace {

constexpr uint32_t CHUNK = 4096;

__global__ void k_nl_count(const uint8_t* __restrict__ t, uint64_t n, uint32_t* cnt) {
    __shared__ uint32_t s;
    if (threadIdx.x == 0) s = 0;
    __syncthreads();
    const uint64_t c0 = (uint64_t)blockIdx.x * CHUNK;
    uint32_t m = 0;
    for (uint64_t i = c0 + threadIdx.x; i < c0 + CHUNK && i < n; i += blockDim.x) m += t[i] == '\n';
    atomicAdd(&s, m);
    __syncthreads();
    if (threadIdx.x == 0) cnt[blockIdx.x] = s;
}

// Positions of the newlines of each chunk, in order: thread j scans bytes
// [c0 + 16 j, c0 + 16 j + 16); a block scan of the per-thread counts orders them.
__global__ void __launch_bounds__(256) k_nl_pos(const uint8_t* __restrict__ t, uint64_t n, const uint64_t* __restrict__ pre,
                                                uint64_t* pos) {
    __shared__ uint32_t s_warp[8];
    const uint64_t c0 = (uint64_t)blockIdx.x * CHUNK + (uint64_t)threadIdx.x * 16;
    uint32_t m = 0;
    for (uint64_t i = c0; i < c0 + 16 && i < n; ++i) m += t[i] == '\n';
    const uint32_t lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    uint32_t x = m;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= (uint32_t)o) x += y;
    }
    if (lane == 31) s_warp[w] = x;
    __syncthreads();
    uint32_t before = 0;
    for (uint32_t j = 0; j < w; ++j) before += s_warp[j];
    uint64_t o = pre[blockIdx.x] + before + x - m;
    for (uint64_t i = c0; i < c0 + 16 && i < n; ++i)
        if (t[i] == '\n') pos[o++] = i;
}

struct Fq {
    const uint8_t* t;
    const uint64_t* nl;  // newline positions
    uint64_t n_lines;
};

// Line j: [start, end) without the newline and a trailing '\r'.
__device__ __forceinline__ void line_span(const Fq& f, uint64_t j, uint64_t& a, uint64_t& e) {
    a = j == 0 ? 0 : f.nl[j - 1] + 1;
    e = f.nl[j];
    if (e > a && f.t[e - 1] == '\r') --e;
}

__device__ __forceinline__ uint8_t up(uint8_t c) { return (c >= 'a' && c <= 'z') ? (uint8_t)(c - 32) : c; }
__device__ __forceinline__ uint32_t code_of(uint8_t c) {  // ASCII_TO_2BIT
    c = up(c);
    return c == 'C' ? 1u : c == 'G' ? 2u : c == 'T' ? 3u : 0u;
}
// Complement for the merge's reverse complement of R2: a base other than ACGT becomes
// 'A' when R2 has at most 512 bases (trim_merge.rs:152-162) and 'T' when it is longer
// (reverse_complement_ascii, bitseq.rs:90-98, reads it as A and complements it).
__device__ __forceinline__ uint8_t rc_char(uint8_t c, uint64_t l2) {
    return (c == 'A' || c == 'a')   ? 'T'
           : (c == 'C' || c == 'c') ? 'G'
           : (c == 'G' || c == 'g') ? 'C'
           : (c == 'T' || c == 't') ? 'A'
                                    : (l2 <= 512 ? 'A' : 'T');
}

__constant__ uint8_t c_truseq[14] = "AGATCGGAAGAGC";
__constant__ uint8_t c_nextera[20] = "AGATGTGTATAAGAGACAG";
__constant__ uint8_t c_nextera_rc[20] = "CTGTCTCTTATACACATCT";

__device__ bool adapter_hit(const uint8_t* w, const uint8_t* ad) {
    int mm = 0;
    for (int j = 0; j < 10; ++j)
        if (up(w[j]) != ad[j] && ++mm > 1) return false;
    return true;
}
// trim_merge.rs:17-76
__device__ uint64_t d_trim_adapter(const uint8_t* s, uint64_t len) {
    if (len < 10) return len;
    const uint64_t start = len > 100 ? len - 100 : 0;
    for (uint64_t i = start; i + 10 <= len; ++i) {
        const uint8_t b0 = up(s[i]), b1 = up(s[i + 1]);
        const bool agat = b0 == 'A' || b1 == 'G', ctgt = b0 == 'C' || b1 == 'T';
        if (!agat && !ctgt) continue;
        if (agat && (adapter_hit(s + i, c_truseq) || adapter_hit(s + i, c_nextera))) return i;
        if (ctgt && adapter_hit(s + i, c_nextera_rc)) return i;
    }
    return len;
}
// trim_merge.rs:79-115 (-1 = None)
__device__ int64_t d_trim_quality(const uint8_t* q, uint64_t len, uint64_t qlen, uint32_t min_qual, uint64_t min_len) {
    if (len < min_len || qlen != len) return -1;
    uint64_t cut = len;
    const uint64_t ws = 4;
    if (qlen >= ws) {
        auto wsum = [&](uint64_t c) {
            uint64_t s = 0;
            for (uint64_t i = c - ws; i < c; ++i) s += q[i] > 33 ? q[i] - 33 : 0;
            return s;
        };
        if (wsum(cut) >= (uint64_t)min_qual * ws) return (int64_t)len;
        while (cut >= ws) {
            if (wsum(cut) / ws >= min_qual) break;
            cut -= 1;
        }
    }
    if (cut < min_len) return -1;
    return (int64_t)cut;
}
// trim_merge.rs:135-238, the overlap search: best overlap (0 = none) and its mismatches
__device__ uint64_t d_merge_overlap(const uint8_t* r1, uint64_t l1, const uint8_t* r2, uint64_t l2, uint64_t min_overlap,
                                    double ratio) {
    if (l1 < min_overlap || l2 < min_overlap) return 0;
    const uint64_t max_d = l1 < l2 ? l1 : l2;
    uint64_t best_d = 0;
    double best = -__longlong_as_double(0x7ff0000000000000LL);  // -inf
    for (int64_t dd = (int64_t)max_d; dd >= (int64_t)min_overlap; --dd) {
        const uint64_t d = (uint64_t)dd;
        const uint8_t* s1 = r1 + (l1 - d);
        const uint64_t allowed = (uint64_t)((double)d * ratio);
        uint64_t mm = 0;
        for (uint64_t i = 0; i < d; ++i)
            if (up(s1[i]) != up(rc_char(r2[l2 - 1 - i], l2)) && ++mm > allowed) break;
        if (mm <= allowed) {
            const double score = (double)d - 2.5 * (double)mm;
            if (score > best) {
                best = score;
                best_d = d;
            }
        }
        if ((double)d <= best) break;
    }
    return best_d >= min_overlap ? best_d : 0;
}

struct IngestArgs {
    Fq f1, f2;
    uint64_t n_pairs;
    double factor;
    uint64_t keep_threshold;
    int subsample, trim, merge;
    uint64_t min_len, seed;
    uint32_t min_qual;
};

// What a pair becomes: kind 0 dropped (or subsampled out), 1 merged, 2 unmerged; t1, t2
// the trimmed lengths and ov the merge overlap (merged length t1 + t2 - ov); raw = l1 + l2.
__global__ void k_pair_decide(IngestArgs A, uint8_t* kind, uint32_t* ta, uint32_t* tb, uint32_t* ov, uint32_t* raw, uint8_t* err) {
    for (uint64_t p = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; p < A.n_pairs; p += (uint64_t)gridDim.x * blockDim.x) {
        uint64_t h1a, h1e, s1a, s1e, p1a, p1e, q1a, q1e, h2a, h2e, s2a, s2e, p2a, p2e, q2a, q2e;
        line_span(A.f1, 4 * p, h1a, h1e);
        line_span(A.f1, 4 * p + 1, s1a, s1e);
        line_span(A.f1, 4 * p + 2, p1a, p1e);
        line_span(A.f1, 4 * p + 3, q1a, q1e);
        line_span(A.f2, 4 * p, h2a, h2e);
        line_span(A.f2, 4 * p + 1, s2a, s2e);
        line_span(A.f2, 4 * p + 2, p2a, p2e);
        line_span(A.f2, 4 * p + 3, q2a, q2e);
        const uint64_t l1 = s1e - s1a, l2 = s2e - s2a;
        raw[p] = (uint32_t)(l1 + l2);
        kind[p] = 0;
        ta[p] = tb[p] = ov[p] = 0;
        const bool bad = h1e == h1a || A.f1.t[h1a] != '@' || p1e == p1a || A.f1.t[p1a] != '+' || q1e - q1a != l1 || h2e == h2a ||
                         A.f2.t[h2a] != '@' || p2e == p2a || A.f2.t[p2a] != '+' || q2e - q2a != l2;
        if (bad) {
            *err = 1;
            continue;
        }
        const uint64_t idx1 = p + 1;  // 1-based input pair (trim_merge.rs:324-348)
        if (A.subsample && smix(idx1 ^ A.seed) > A.keep_threshold) continue;
        const uint8_t *s1 = A.f1.t + s1a, *q1 = A.f1.t + q1a, *s2 = A.f2.t + s2a, *q2 = A.f2.t + q2a;
        uint64_t t1 = l1, t2 = l2;
        if (A.trim) {
            const uint64_t a1 = d_trim_adapter(s1, l1), a2 = d_trim_adapter(s2, l2);
            const int64_t x1 = d_trim_quality(q1, a1, a1, A.min_qual, A.min_len);
            const int64_t x2 = d_trim_quality(q2, a2, a2, A.min_qual, A.min_len);
            if (x1 < 0 || x2 < 0) continue;
            t1 = (uint64_t)x1;
            t2 = (uint64_t)x2;
        } else if (l1 < A.min_len || l2 < A.min_len) {
            continue;
        }
        ta[p] = (uint32_t)t1;
        tb[p] = (uint32_t)t2;
        const uint64_t d = A.merge ? d_merge_overlap(s1, t1, s2, t2, 15, 0.10) : 0;
        ov[p] = (uint32_t)d;
        kind[p] = d ? 1 : 2;
    }
}

struct WriteArgs {
    uint64_t* data;      // all arenas' words, arena a from word wbase[a]
    uint64_t* off;       // bank-global base offsets
    uint32_t* len;
    uint32_t* pair_idx;
    uint64_t wbase[3];
    uint64_t rbase[3];   // first read of each arena
};

__device__ __forceinline__ void put_code(uint64_t* data, uint64_t g, uint32_t c) {
    if (c) atomicOr((unsigned long long*)&data[g >> 5], (unsigned long long)c << ((g & 31) << 1));
}

__global__ void k_pair_write(IngestArgs A, WriteArgs W, const uint8_t* __restrict__ kind, const uint32_t* __restrict__ ta,
                             const uint32_t* __restrict__ tb, const uint32_t* __restrict__ ov, const uint64_t* __restrict__ read_no,
                             const uint64_t* __restrict__ base_no) {
    for (uint64_t p = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; p < A.n_pairs; p += (uint64_t)gridDim.x * blockDim.x) {
        const uint8_t kd = kind[p];
        if (!kd) continue;
        uint64_t s1a, s1e, q1a, q1e, s2a, s2e, q2a, q2e;
        line_span(A.f1, 4 * p + 1, s1a, s1e);
        line_span(A.f1, 4 * p + 3, q1a, q1e);
        line_span(A.f2, 4 * p + 1, s2a, s2e);
        line_span(A.f2, 4 * p + 3, q2a, q2e);
        const uint8_t *s1 = A.f1.t + s1a, *q1 = A.f1.t + q1a, *s2 = A.f2.t + s2a, *q2 = A.f2.t + q2a;
        const uint32_t pair0 = (uint32_t)p;
        const uint64_t t1 = ta[p], t2 = tb[p];
        if (kd == 1) {
            // merged read (trim_merge.rs:214-237): r1 prefix, the overlap base by base
            // (agreeing bases, else the higher quality), then rc(r2) past the overlap
            const uint64_t d = ov[p], m = t1 + t2 - d;
            const uint64_t r = W.rbase[0] + read_no[p];
            const uint64_t g0 = W.wbase[0] * 32 + base_no[p];
            W.off[r] = g0;
            W.len[r] = (uint32_t)m;
            W.pair_idx[r] = pair0;
            uint64_t g = g0;
            for (uint64_t i = 0; i < t1 - d; ++i) put_code(W.data, g++, code_of(s1[i]));
            for (uint64_t i = 0; i < d; ++i) {
                const uint8_t b1 = s1[t1 - d + i], b2 = rc_char(s2[t2 - 1 - i], t2);
                const uint8_t qa = q1[t1 - d + i], qb = q2[t2 - 1 - i];
                const uint8_t c = (up(b1) == up(b2)) ? up(b1) : (qa >= qb ? up(b1) : up(b2));
                put_code(W.data, g++, code_of(c));
            }
            for (uint64_t i = d; i < t2; ++i) put_code(W.data, g++, code_of(rc_char(s2[t2 - 1 - i], t2)));
        } else {
            const uint64_t r1i = W.rbase[1] + read_no[p], r2i = W.rbase[2] + read_no[p];
            const uint64_t g1 = W.wbase[1] * 32 + base_no[p], g2 = W.wbase[2] * 32 + base_no[A.n_pairs + p];
            W.off[r1i] = g1;
            W.len[r1i] = (uint32_t)t1;
            W.pair_idx[r1i] = pair0;
            W.off[r2i] = g2;
            W.len[r2i] = (uint32_t)t2;
            W.pair_idx[r2i] = pair0;
            for (uint64_t i = 0; i < t1; ++i) put_code(W.data, g1 + i, code_of(s1[i]));
            for (uint64_t i = 0; i < t2; ++i) put_code(W.data, g2 + i, code_of(s2[i]));
        }
    }
}

struct DBufs {
    fbk_ctx* c;
    std::vector<void*> p;
    void* get(uint64_t b) {
        void* q = dev_alloc(c, std::max<uint64_t>(b, 8));
        if (q) p.push_back(q);
        return q;
    }
    ~DBufs() {
        cudaStreamSynchronize(c->stream);
        for (void* q : p) dev_free(c, q);
    }
};

// Uploads one FASTQ text (adding the final newline it may lack) and indexes its lines.
fbk_status index_lines(fbk_ctx* ctx, DBufs& B, const uint8_t* text, uint64_t len, Fq& f) {
    const bool add_nl = len && text[len - 1] != '\n';
    const uint64_t n = len + (add_nl ? 1 : 0);
    uint8_t* t = (uint8_t*)B.get(n);
    const uint64_t n_chunks = (n + CHUNK - 1) / CHUNK;
    uint32_t* cnt = (uint32_t*)B.get(n_chunks * 4);
    uint64_t* pre = (uint64_t*)B.get(n_chunks * 8);
    if (!t || !cnt || !pre) return set_err(ctx, FBK_ERR_OOM, "FASTQ text on the device");
    if (len) CK(ctx, cudaMemcpyAsync(t, text, len, cudaMemcpyHostToDevice, ctx->stream));
    if (add_nl) CK(ctx, cudaMemsetAsync(t + len, '\n', 1, ctx->stream));
    f.t = t;
    f.n_lines = 0;
    f.nl = nullptr;
    if (!n) return FBK_OK;
    TIMED(ctx, "ingest_lines", (k_nl_count<<<(unsigned)n_chunks, 256, 0, ctx->stream>>>(t, n, cnt), cudaGetLastError()));
    std::vector<uint32_t> hc(n_chunks);
    std::vector<uint64_t> hp(n_chunks);
    CK(ctx, cudaMemcpyAsync(hc.data(), cnt, n_chunks * 4, cudaMemcpyDeviceToHost, ctx->stream));
    CK(ctx, cudaStreamSynchronize(ctx->stream));
    uint64_t total = 0;
    for (uint64_t i = 0; i < n_chunks; ++i) {
        hp[i] = total;
        total += hc[i];
    }
    uint64_t* pos = (uint64_t*)B.get(total * 8);
    if (!pos) return set_err(ctx, FBK_ERR_OOM, "FASTQ line index");
    CK(ctx, cudaMemcpyAsync(pre, hp.data(), n_chunks * 8, cudaMemcpyHostToDevice, ctx->stream));
    TIMED(ctx, "ingest_lines", (k_nl_pos<<<(unsigned)n_chunks, 256, 0, ctx->stream>>>(t, n, pre, pos), cudaGetLastError()));
    f.nl = pos;
    f.n_lines = total;
    return FBK_OK;
}

}  // namespace

extern "C" {

FBK_API fbk_status fbk_ingest_fastq_device(fbk_ctx* ctx, const uint8_t* r1, uint64_t r1_len, const uint8_t* r2, uint64_t r2_len,
                                           double subsample_factor, uint64_t min_len, uint32_t min_qual, int enable_trim,
                                           int enable_merge, uint64_t seed, fbk_bank** out, fbk_ingest_stats* stats) {
    if (!ctx || !out || (r1_len && !r1) || (r2_len && !r2)) return FBK_ERR_INVALID;
    *out = nullptr;
    CK(ctx, cudaSetDevice(ctx->device));
    DBufs B{ctx, {}};
    Fq f1{}, f2{};
    fbk_status st = index_lines(ctx, B, r1, r1_len, f1);
    if (st == FBK_OK) st = index_lines(ctx, B, r2, r2_len, f2);
    if (st) return st;
    if (f1.n_lines % 4 || f2.n_lines % 4)
        return set_err(ctx, FBK_ERR_FORMAT, "device ingest reads plain 4-line FASTQ records (a record is incomplete or blank lines "
                                            "separate records; the host ingest reads those)");
    if (f1.n_lines != f2.n_lines) return set_err(ctx, FBK_ERR_FORMAT, "Mismatched paired-end FASTQ mate counts between R1 and R2");
    const uint64_t n_pairs = f1.n_lines / 4;
    if (n_pairs >= (1ULL << 32)) return set_err(ctx, FBK_ERR_INVALID, "device ingest: 2^32 or more pairs");
    IngestArgs A{};
    A.f1 = f1;
    A.f2 = f2;
    A.n_pairs = n_pairs;
    A.factor = subsample_factor;
    A.subsample = subsample_factor < 0.999;
    const double x = subsample_factor * 18446744073709551616.0;
    A.keep_threshold = !(x > 0.0) ? 0 : x >= 18446744073709551616.0 ? UINT64_MAX : (uint64_t)x;
    A.trim = enable_trim != 0;
    A.merge = enable_merge != 0;
    A.min_len = min_len;
    A.min_qual = min_qual;
    A.seed = seed;
    uint8_t* kind = (uint8_t*)B.get(n_pairs);
    uint32_t* ta = (uint32_t*)B.get(n_pairs * 4);
    uint32_t* tb = (uint32_t*)B.get(n_pairs * 4);
    uint32_t* ov = (uint32_t*)B.get(n_pairs * 4);
    uint32_t* raw = (uint32_t*)B.get(n_pairs * 4);
    uint8_t* err = (uint8_t*)B.get(8);
    if (!kind || !ta || !tb || !ov || !raw || !err) return set_err(ctx, FBK_ERR_OOM, "device ingest pair state");
    CK(ctx, cudaMemsetAsync(err, 0, 8, ctx->stream));
    Launch L = launch_cfg(ctx, 128, 0);
    if (n_pairs)
        TIMED(ctx, "ingest_decide", (k_pair_decide<<<L.grid, L.block, 0, L.stream>>>(A, kind, ta, tb, ov, raw, err), cudaGetLastError()));
    std::vector<uint8_t> hk(n_pairs), herr(1);
    std::vector<uint32_t> h1(n_pairs), h2(n_pairs), hov(n_pairs), hr(n_pairs);
    if (n_pairs) {
        CK(ctx, cudaMemcpyAsync(hk.data(), kind, n_pairs, cudaMemcpyDeviceToHost, ctx->stream));
        CK(ctx, cudaMemcpyAsync(h1.data(), ta, n_pairs * 4, cudaMemcpyDeviceToHost, ctx->stream));
        CK(ctx, cudaMemcpyAsync(h2.data(), tb, n_pairs * 4, cudaMemcpyDeviceToHost, ctx->stream));
        CK(ctx, cudaMemcpyAsync(hov.data(), ov, n_pairs * 4, cudaMemcpyDeviceToHost, ctx->stream));
        CK(ctx, cudaMemcpyAsync(hr.data(), raw, n_pairs * 4, cudaMemcpyDeviceToHost, ctx->stream));
    }
    CK(ctx, cudaMemcpyAsync(herr.data(), err, 1, cudaMemcpyDeviceToHost, ctx->stream));
    CK(ctx, cudaStreamSynchronize(ctx->stream));
    if (herr[0]) return set_err(ctx, FBK_ERR_FORMAT, "Corrupted FASTQ record (header, '+' line or quality length)");
    // read and base numbers of every pair in each arena (pair order = push order) and
    // the IngestStats (trim_merge.rs:307-417)
    fbk_ingest_stats S{};
    std::vector<uint64_t> read_no(n_pairs, 0), base_no(2 * n_pairs, 0);
    uint64_t nr[3] = {0, 0, 0}, nb[3] = {0, 0, 0};
    std::vector<uint32_t> lens[3];
    for (uint64_t p = 0; p < n_pairs; ++p) {
        S.input_read_pairs++;
        S.bases_before_trim += hr[p];
        if (!hk[p]) continue;
        S.retained_read_pairs++;
        S.bases_after_trim += (uint64_t)h1[p] + h2[p];
        if (hk[p] == 1) {
            const uint64_t m = (uint64_t)h1[p] + h2[p] - hov[p];
            read_no[p] = nr[0]++;
            base_no[p] = nb[0];
            nb[0] += m;
            lens[0].push_back((uint32_t)m);
            S.merged_pairs_count++;
            S.merged_bases += m;
        } else {
            read_no[p] = nr[1]++;
            nr[2]++;
            base_no[p] = nb[1];
            base_no[n_pairs + p] = nb[2];
            nb[1] += h1[p];
            nb[2] += h2[p];
            lens[1].push_back(h1[p]);
            lens[2].push_back(h2[p]);
            S.unmerged_pairs_count++;
        }
    }
    if (nr[0] + nr[1] + nr[2] == 0)
        return set_err(ctx, FBK_ERR_EMPTY, "No valid reads survived trimming and quality filtering (check input FASTQ files)");
    const uint64_t aw[3] = {(nb[0] + 31) / 32, (nb[1] + 31) / 32, (nb[2] + 31) / 32};
    const uint64_t n_words = aw[0] + aw[1] + aw[2];
    const uint64_t n_reads = nr[0] + nr[1] + nr[2];
    fbk_bank* bk = new fbk_bank();
    bk->ctx = ctx;
    bk->data = (uint64_t*)dev_alloc(ctx, (n_words + 8) * 8);
    bk->off = (uint64_t*)dev_alloc(ctx, n_reads * 8);
    bk->len = (uint32_t*)dev_alloc(ctx, n_reads * 4);
    bk->pair_idx = (uint32_t*)dev_alloc(ctx, n_reads * 4);
    uint64_t* d_read = (uint64_t*)B.get(n_pairs * 8);
    uint64_t* d_base = (uint64_t*)B.get(2 * n_pairs * 8);
    if (!bk->data || !bk->off || !bk->len || !bk->pair_idx || !d_read || !d_base) {
        fbk_bank_release(bk);
        return set_err(ctx, FBK_ERR_OOM, "device memory for the read bank");
    }
    WriteArgs W{};
    W.data = bk->data;
    W.off = bk->off;
    W.len = bk->len;
    W.pair_idx = bk->pair_idx;
    W.wbase[0] = 0;
    W.wbase[1] = aw[0];
    W.wbase[2] = aw[0] + aw[1];
    W.rbase[0] = 0;
    W.rbase[1] = nr[0];
    W.rbase[2] = nr[0] + nr[1];
    cudaError_t e = cudaMemsetAsync(bk->data, 0, (n_words + 8) * 8, ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_read, read_no.data(), n_pairs * 8, cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_base, base_no.data(), 2 * n_pairs * 8, cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) {
        TimedLaunch tl;
        time_begin(ctx, "ingest_write", tl);
        k_pair_write<<<L.grid, L.block, 0, L.stream>>>(A, W, kind, ta, tb, ov, d_read, d_base);
        e = cudaGetLastError();
        time_end(ctx, tl);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) {
        fbk_bank_release(bk);
        return cuda_err(ctx, e, "device ingest write");
    }
    // bank bookkeeping as bank_upload_impl keeps it
    bk->n_reads = n_reads;
    bk->n_words = n_words;
    bk->n_bases = nb[0] + nb[1] + nb[2];
    bk->n_pairs = n_pairs;
    uint32_t max_len = 0;
    for (int a = 0; a < 3; ++a) {
        bk->arena_reads.push_back(nr[a]);
        for (uint32_t L0 : lens[a]) max_len = std::max(max_len, L0);
    }
    bk->max_len = max_len;
    bk->chunk_starts.push_back(0);
    uint64_t acc = 0, r = 0;
    for (int a = 0; a < 3; ++a)
        for (uint32_t L0 : lens[a]) {
            if (acc && acc + L0 >= (1ull << 30)) {
                bk->chunk_starts.push_back(r);
                bk->max_chunk = std::max(bk->max_chunk, acc);
                acc = 0;
            }
            acc += L0;
            ++r;
        }
    bk->max_chunk = std::max(bk->max_chunk, acc);
    bk->chunk_starts.push_back(n_reads);
    const uint64_t bins = std::min<uint64_t>((uint64_t)max_len + 2, 1ULL << 16);
    bk->len_hist.assign(bins, 0);
    for (int a = 0; a < 3; ++a)
        for (uint32_t L0 : lens[a]) {
            if (L0 < bins - 1) bk->len_hist[L0]++;
            else bk->long_bases += L0;
        }
    if (stats) *stats = S;
    *out = bk;
    return FBK_OK;
}

// Copies a device bank back (for checks and hand-off): words (n_words), base offsets
// (bank-global), lengths and pair indices (n_reads each; any may be NULL).
FBK_API fbk_status fbk_bank_export(const fbk_bank* b, uint64_t* words, uint64_t* offsets, uint32_t* lengths, uint32_t* pair_idx) {
    if (!b) return FBK_ERR_INVALID;
    fbk_ctx* ctx = b->ctx;
    CK(ctx, bank_wait(ctx, b));
    if (words && b->n_words) CK(ctx, cudaMemcpyAsync(words, b->data, b->n_words * 8, cudaMemcpyDeviceToHost, ctx->stream));
    if (offsets && b->n_reads) CK(ctx, cudaMemcpyAsync(offsets, b->off, b->n_reads * 8, cudaMemcpyDeviceToHost, ctx->stream));
    if (lengths && b->n_reads) CK(ctx, cudaMemcpyAsync(lengths, b->len, b->n_reads * 4, cudaMemcpyDeviceToHost, ctx->stream));
    if (pair_idx && b->n_reads) {
        if (!b->pair_idx) return set_err(ctx, FBK_ERR_INVALID, "bank has no pair indices");
        CK(ctx, cudaMemcpyAsync(pair_idx, b->pair_idx, b->n_reads * 4, cudaMemcpyDeviceToHost, ctx->stream));
    }
    CK(ctx, cudaStreamSynchronize(ctx->stream));
    return FBK_OK;
}

FBK_API fbk_status fbk_bank_words(const fbk_bank* b, uint64_t* n_words) {
    if (!b || !n_words) return FBK_ERR_INVALID;
    *n_words = b->n_words;
    return FBK_OK;
}

FBK_API fbk_status fbk_bank_arena_counts(const fbk_bank* b, uint64_t* counts3) {
    if (!b || !counts3) return FBK_ERR_INVALID;
    for (int a = 0; a < 3; ++a) counts3[a] = a < (int)b->arena_reads.size() ? b->arena_reads[a] : 0;
    return FBK_OK;
}

}  // extern "C"
