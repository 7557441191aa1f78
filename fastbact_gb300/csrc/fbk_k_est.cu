// fbk_k_est.cu — genome-estimator kernels (src/ingest/estimator.rs:296-379) and
// small device utilities (HLL, CMS key ops, subsampler, ntHash / k-mer dumps).
//
// The reference estimator is sequential: k-mer occurrence t (pairs in order, R1
// then R2, windows in order) does cms.add_and_estimate(raw) and adds splitmix64(raw)
// to hll_solid when the estimate is >= 2.  After the add at t the counter (r, col)
// holds min(15, #{t' <= t touching it}), so "estimate >= 2" holds exactly when, for
// every row r, some t' < t touched (r, col_r(raw_t)).  The device form is therefore
//   A: first[r][col] = min t over all occurrences touching the counter (atomicMin)
//   B: solid(t) = for all r: first[r][col_r(raw_t)] < t
// which reproduces hll_solid bit for bit regardless of thread order.  The early stop
// (every 2000 pairs from 6000 on, estimator.rs:366-375) needs the HLL registers at
// each checkpoint: B writes per-segment register maxima, a prefix max over segments
// gives the registers at every checkpoint, and one thread per checkpoint sums
// 2^-reg in register order in f64 — the exact operation sequence of
// HyperLogLog::estimate (sketch.rs:88-96) — so the host finishes with the same bits.
#include "fbk_device.cuh"
#include "fbk_kernels.cuh"

namespace fbk {

// pair index (0-based) -> checkpoint segment: segment 0 covers pairs 1..6000 of the
// 1-based pair count, segment j >= 1 covers 6000+2000(j-1)+1 .. 6000+2000j.
__device__ __forceinline__ uint32_t est_segment(uint64_t pair0) {
    const uint64_t pc = pair0 + 1;
    return pc <= 6000 ? 0u : (uint32_t)(1 + (pc - 6001) / 2000);
}

__global__ void __launch_bounds__(256) k_est_firstpos(BankDev b, const uint64_t* __restrict__ kbase, uint32_t k,
                                                      uint32_t* __restrict__ first, uint32_t log2w) {
    const uint32_t lane = threadIdx.x & 31;
    const uint64_t gw = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    for (uint64_t r = b.r_begin + gw; r < b.r_end; r += nwarps) {
        const uint32_t len = b.len[r];
        if (len < k) continue;
        const uint64_t off = b.off[r], t0 = kbase[r];
        // lane takes a run of consecutive windows and rolls the hash along it
        const uint32_t nk = len - k + 1, run = (nk + 31) >> 5;
        const uint32_t lo = lane * run < nk ? lane * run : nk, hi = lo + run < nk ? lo + run : nk;
        nthash_run(b.data, off, k, lo, hi, [&](uint32_t i, uint64_t raw) {
            const uint32_t t = (uint32_t)(t0 + i);
#pragma unroll
            for (int rr = 0; rr < 4; ++rr) {
                uint32_t* p = first + cms_index(raw, rr, log2w);
                if (*(volatile uint32_t*)p > t) atomicMin(p, t);
            }
        });
    }
}

__global__ void __launch_bounds__(256) k_est_hll(BankDev b, const uint64_t* __restrict__ kbase, uint32_t k,
                                                 const uint32_t* __restrict__ first, uint32_t log2w, uint32_t p,
                                                 uint32_t n_segs, uint32_t* __restrict__ regs_total,
                                                 uint32_t* __restrict__ regs_solid) {
    const uint32_t lane = threadIdx.x & 31;
    const uint64_t gw = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    const uint64_t m = 1ULL << p;
    for (uint64_t r = b.r_begin + gw; r < b.r_end; r += nwarps) {
        const uint32_t len = b.len[r];
        if (len < k) continue;
        const uint64_t off = b.off[r], t0 = kbase[r];
        uint32_t seg = est_segment(r >> 1);  // reads are R1,R2 interleaved per pair
        if (seg >= n_segs) seg = n_segs - 1;
        uint32_t* rt = regs_total + (uint64_t)seg * m;
        uint32_t* rs = regs_solid + (uint64_t)seg * m;
        const uint32_t nk = len - k + 1, run = (nk + 31) >> 5;
        const uint32_t lo = lane * run < nk ? lane * run : nk, hi = lo + run < nk ? lo + run : nk;
        nthash_run(b.data, off, k, lo, hi, [&](uint32_t i, uint64_t raw) {
            const uint32_t t = (uint32_t)(t0 + i);
            bool solid = true;
#pragma unroll
            for (int rr = 0; rr < 4; ++rr) solid &= __ldcg(first + cms_index(raw, rr, log2w)) < t;
            uint32_t idx, rho;
            hll_idx_rho(smix(raw), p, idx, rho);
            // Registers only grow, so a stale read that is already >= rho is safe to skip.
            if (*(volatile uint32_t*)&rt[idx] < rho) atomicMax(&rt[idx], rho);
            if (solid && *(volatile uint32_t*)&rs[idx] < rho) atomicMax(&rs[idx], rho);
        });
    }
}

// In-place prefix max over segments, one thread per register.
__global__ void k_est_prefix(uint32_t* regs, uint64_t m, uint32_t n_segs) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m; i += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t v = regs[i];
        for (uint32_t s = 1; s < n_segs; ++s) {
            uint32_t x = regs[(uint64_t)s * m + i];
            v = x > v ? x : v;
            regs[(uint64_t)s * m + i] = v;
        }
    }
}

// One block per (sketch, segment end): the f64 sum of 2^-reg in register order and
// the number of zero registers (sketch.rs:88-96).  With m = 2^p registers all <= V =
// 53 - p, every partial sum of the sequence is a multiple of 2^-V no larger than 2^p,
// i.e. fits 53 bits: the sequential f64 sum is then exact and equals the integer sum
// of 2^(V - reg) (taken by the block in any order, at most 2^53) times 2^-V.  A sketch
// holding a larger register (V = 39 for p = 14: a hash with 39 or more leading zeros
// after its index bits) is summed sequentially by one thread, in register order, with
// 2^-v built exactly from its bits.
__global__ void __launch_bounds__(256) k_est_sums(const uint32_t* regs_total, const uint32_t* regs_solid, uint32_t p,
                                                  uint32_t n_segs, double* sums, unsigned long long* zeros) {
    const uint64_t m = 1ULL << p;
    const uint32_t V = 53 - p;
    __shared__ unsigned long long s_sum[8], s_zero[8];
    __shared__ uint32_t s_big;
    const uint32_t i = blockIdx.x;
    if (i >= 2 * n_segs) return;
    const uint32_t* r = (i < n_segs ? regs_total : regs_solid) + (uint64_t)(i % n_segs) * m;
    if (threadIdx.x == 0) s_big = 0;
    __syncthreads();
    unsigned long long acc = 0, z = 0;
    bool big = false;
    for (uint64_t j = threadIdx.x; j < m; j += blockDim.x) {
        const uint32_t v = r[j];
        big |= v > V;
        acc += v <= V ? 1ULL << (V - v) : 0ULL;
        z += (v == 0);
    }
    if (big) atomicOr(&s_big, 1u);
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        acc += __shfl_down_sync(0xffffffffu, acc, off);
        z += __shfl_down_sync(0xffffffffu, z, off);
    }
    if ((threadIdx.x & 31) == 0) {
        s_sum[threadIdx.x >> 5] = acc;
        s_zero[threadIdx.x >> 5] = z;
    }
    __syncthreads();
    if (threadIdx.x != 0) return;
    unsigned long long tot = 0, tz = 0;
    for (uint32_t w = 0; w < (blockDim.x >> 5); ++w) {
        tot += s_sum[w];
        tz += s_zero[w];
    }
    zeros[i] = tz;
    if (!s_big) {
        sums[i] = ldexp(__ull2double_rn(tot), -(int)V);  // tot <= 2^53: both steps exact
        return;
    }
    double s = 0.0;
    for (uint64_t j = 0; j < m; ++j) s = __dadd_rn(s, __longlong_as_double((long long)(1023 - (int)r[j]) << 52));
    sums[i] = s;
}

// HyperLogLog::add_hash / add_canonical_hash (sketch.rs:49-70) over device hashes.
__global__ void k_hll_add(uint32_t* regs, uint32_t p, const uint64_t* __restrict__ h, uint64_t n, int mix) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t x = mix ? smix(h[i]) : h[i];
        uint32_t idx, rho;
        hll_idx_rho(x, p, idx, rho);
        if (*(volatile uint32_t*)&regs[idx] < rho) atomicMax(&regs[idx], rho);
    }
}
__global__ void k_hll_merge(uint32_t* dst, const uint32_t* src, uint64_t n) {  // sketch.rs:73-80
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        dst[i] = src[i] > dst[i] ? src[i] : dst[i];
}

// Subsampler bitmap: bit q = pair q (0-based) kept; the reference's pair_idx is q+1
// (trim_merge.rs:333,343-347) and keep_threshold = (factor * 2^64) as u64.
__global__ void k_subsample(uint64_t n_pairs, uint64_t threshold, uint64_t seed, int keep_all, uint64_t* bits) {
    const uint64_t n_words = (n_pairs + 63) / 64;
    for (uint64_t w = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; w < n_words; w += (uint64_t)gridDim.x * blockDim.x) {
        uint64_t v = 0;
        for (uint32_t b = 0; b < 64; ++b) {
            const uint64_t q = w * 64 + b;
            if (q >= n_pairs) break;
            const bool keep = keep_all || smix((q + 1) ^ seed) <= threshold;
            v |= (uint64_t)keep << b;
        }
        bits[w] = v;
    }
}

// CountMinSketch::add / estimate (sketch.rs:191-246) over device keys, on the exact
// u32 counts: add is a RED.ADD per row, estimate the minimum over rows capped at cap.
__global__ void k_cms_keys(uint32_t* cnt, uint32_t log2w, uint32_t cap, const uint64_t* __restrict__ keys, uint64_t n,
                           uint32_t* est, int add) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t key = keys[i];
        if (add) {
#pragma unroll
            for (int r = 0; r < 4; ++r) atomicAdd(cnt + cms_index(key, r, log2w), 1u);
        } else {
            uint32_t m = cap;
#pragma unroll
            for (int r = 0; r < 4; ++r) {
                const uint32_t c = cnt[cms_index(key, r, log2w)];
                m = c < m ? c : m;
            }
            est[i] = m;
        }
    }
}

// dst = min(65535, dst + src): counts stay exact below every cap (<= 65535).
__global__ void k_cms_merge(uint32_t* dst, const uint32_t* src, uint64_t n) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t v = (uint64_t)dst[i] + src[i];
        dst[i] = v > 0xFFFFu ? 0xFFFFu : (uint32_t)v;
    }
}

// Reference layout: nibble byte b holds counters 2b (low) and 2b+1 (high), capped at
// 15 (sketch.rs:131-157); u16 mode writes min(65535, count) little-endian.
__global__ void k_cms_export_nib(const uint32_t* __restrict__ cnt, uint64_t n_bytes, uint8_t* out) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n_bytes; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint2 v = reinterpret_cast<const uint2*>(cnt)[i];
        const uint32_t lo = v.x < 15u ? v.x : 15u, hi = v.y < 15u ? v.y : 15u;
        out[i] = (uint8_t)(lo | (hi << 4));
    }
}
__global__ void k_cms_export_u16(const uint32_t* __restrict__ cnt, uint64_t n, uint16_t* out) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t v = cnt[i];
        out[i] = (uint16_t)(v < 0xFFFFu ? v : 0xFFFFu);
    }
}

// Inverse of the exports: counters from reference-layout bytes.
__global__ void k_cms_import_nib(uint32_t* __restrict__ cnt, uint64_t n_bytes, const uint8_t* __restrict__ in) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n_bytes; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t v = in[i];
        reinterpret_cast<uint2*>(cnt)[i] = make_uint2(v & 15u, v >> 4);
    }
}
__global__ void k_cms_import_u16(uint32_t* __restrict__ cnt, uint64_t n, const uint16_t* __restrict__ in) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) cnt[i] = in[i];
}

__global__ void __launch_bounds__(256) k_nthash_arena(BankDev b, const uint64_t* __restrict__ kbase, uint32_t k, uint64_t* out) {
    const uint32_t lane = threadIdx.x & 31;
    const uint64_t gw = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    for (uint64_t r = b.r_begin + gw; r < b.r_end; r += nwarps) {
        const uint32_t len = b.len[r];
        if (len < k) continue;
        const uint32_t nk = len - k + 1, run = (nk + 31) >> 5;
        const uint32_t lo = lane * run < nk ? lane * run : nk, hi = lo + run < nk ? lo + run : nk;
        const uint64_t o = kbase[r];
        nthash_run(b.data, b.off[r], k, lo, hi, [&](uint32_t i, uint64_t h) { out[o + i] = h; });
    }
}

template <int NW>
__global__ void __launch_bounds__(256) k_canon_arena(BankDev b, const uint64_t* __restrict__ kbase, uint32_t k,
                                                     uint64_t* out, uint8_t* out_rc) {
    const uint32_t lane = threadIdx.x & 31;
    const uint64_t gw = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    for (uint64_t r = b.r_begin + gw; r < b.r_end; r += nwarps) {
        const uint32_t len = b.len[r];
        if (len < k) continue;
        for (uint32_t i = lane; i < len - k + 1; i += 32) {
            Key<NW> can;
            bool rc;
            window_canonical<NW>(b.data, b.off[r] + i, k, can, rc);
            const uint64_t t = kbase[r] + i;
#pragma unroll
            for (int j = 0; j < NW; ++j) out[t * NW + j] = can.w[j];
            out_rc[t] = rc;
        }
    }
}

__global__ void k_add_u64(uint64_t* p, uint64_t n, uint64_t add) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) p[i] += add;
}

// ---------------------------------------------------------------------------
cudaError_t launch_est_firstpos(const Launch& L, const BankDev& b, const uint64_t* kbase, uint32_t k, uint32_t* first,
                                uint32_t log2w) {
    k_est_firstpos<<<L.grid, L.block, 0, L.stream>>>(b, kbase, k, first, log2w);
    return cudaGetLastError();
}
cudaError_t launch_est_hll(const Launch& L, const BankDev& b, const uint64_t* kbase, uint32_t k, const uint32_t* first,
                           uint32_t log2w, uint32_t p, uint32_t n_segs, uint32_t* regs_total, uint32_t* regs_solid) {
    k_est_hll<<<L.grid, L.block, 0, L.stream>>>(b, kbase, k, first, log2w, p, n_segs, regs_total, regs_solid);
    return cudaGetLastError();
}
cudaError_t launch_est_prefix(const Launch& L, uint32_t* regs, uint32_t p, uint32_t n_segs) {
    k_est_prefix<<<L.grid, L.block, 0, L.stream>>>(regs, 1ULL << p, n_segs);
    return cudaGetLastError();
}
cudaError_t launch_est_sums(const Launch& L, const uint32_t* regs_total, const uint32_t* regs_solid, uint32_t p,
                            uint32_t n_segs, double* sums, unsigned long long* zeros) {
    k_est_sums<<<2 * n_segs, 256, 0, L.stream>>>(regs_total, regs_solid, p, n_segs, sums, zeros);
    return cudaGetLastError();
}
cudaError_t launch_hll_add(const Launch& L, uint32_t* regs, uint32_t p, const uint64_t* hashes, uint64_t n, int mix) {
    k_hll_add<<<L.grid, L.block, 0, L.stream>>>(regs, p, hashes, n, mix);
    return cudaGetLastError();
}
cudaError_t launch_hll_merge(const Launch& L, uint32_t* dst, const uint32_t* src, uint64_t n) {
    k_hll_merge<<<L.grid, L.block, 0, L.stream>>>(dst, src, n);
    return cudaGetLastError();
}
cudaError_t launch_subsample_mask(const Launch& L, uint64_t n_pairs, double factor, uint64_t seed, uint64_t* bits) {
    // keep_threshold = (factor * (u64::MAX as f64)) as u64, saturating (trim_merge.rs:325)
    const double x = factor * 18446744073709551616.0;
    const uint64_t thr = !(x > 0.0) ? 0 : x >= 18446744073709551616.0 ? ~0ULL : (uint64_t)x;
    const int keep_all = !(factor < 0.999);
    k_subsample<<<L.grid, L.block, 0, L.stream>>>(n_pairs, thr, seed, keep_all, bits);
    return cudaGetLastError();
}
cudaError_t launch_cms_keys(const Launch& L, uint32_t* cnt, uint32_t log2w, uint32_t cap, const uint64_t* keys, uint64_t n,
                            uint32_t* est_out, int add) {
    k_cms_keys<<<L.grid, L.block, 0, L.stream>>>(cnt, log2w, cap, keys, n, est_out, add);
    return cudaGetLastError();
}
cudaError_t launch_cms_merge(const Launch& L, uint32_t* dst, const uint32_t* src, uint64_t n) {
    k_cms_merge<<<L.grid, L.block, 0, L.stream>>>(dst, src, n);
    return cudaGetLastError();
}
cudaError_t launch_cms_export(int cb, const Launch& L, const uint32_t* cnt, uint64_t n, uint8_t* out) {
    if (cb == 4) k_cms_export_nib<<<L.grid, L.block, 0, L.stream>>>(cnt, n / 2, out);
    else k_cms_export_u16<<<L.grid, L.block, 0, L.stream>>>(cnt, n, reinterpret_cast<uint16_t*>(out));
    return cudaGetLastError();
}
cudaError_t launch_cms_import(int cb, const Launch& L, uint32_t* cnt, uint64_t n, const uint8_t* in) {
    if (cb == 4) k_cms_import_nib<<<L.grid, L.block, 0, L.stream>>>(cnt, n / 2, in);
    else k_cms_import_u16<<<L.grid, L.block, 0, L.stream>>>(cnt, n, reinterpret_cast<const uint16_t*>(in));
    return cudaGetLastError();
}
cudaError_t launch_nthash_arena(const Launch& L, const BankDev& b, const uint64_t* kbase, uint32_t k, uint64_t* out) {
    k_nthash_arena<<<L.grid, L.block, 0, L.stream>>>(b, kbase, k, out);
    return cudaGetLastError();
}
cudaError_t launch_canon_arena(int nw, const Launch& L, const BankDev& b, const uint64_t* kbase, uint32_t k,
                               uint64_t* out_words, uint8_t* out_rc) {
    if (nw == 1) k_canon_arena<1><<<L.grid, L.block, 0, L.stream>>>(b, kbase, k, out_words, out_rc);
    else if (nw == 2) k_canon_arena<2><<<L.grid, L.block, 0, L.stream>>>(b, kbase, k, out_words, out_rc);
    else k_canon_arena<4><<<L.grid, L.block, 0, L.stream>>>(b, kbase, k, out_words, out_rc);
    return cudaGetLastError();
}
cudaError_t launch_add_u64(const Launch& L, uint64_t* p, uint64_t n, uint64_t add) {
    k_add_u64<<<L.grid, L.block, 0, L.stream>>>(p, n, add);
    return cudaGetLastError();
}

}  // namespace fbk
