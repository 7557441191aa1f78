// fbk_k_batch.cu — multi-isolate forms of the build kernels (one launch per phase
// for every isolate of a wave).
//
// The reads of all isolates in a wave form one global index R: isolate i owns
// R in [read_base[i], read_base[i+1]).  Warps stride over R exactly like the
// single-isolate kernels stride over one bank, so at any moment the resident warps
// work on a narrow band of R — one or two isolates — and the sketch or table slice
// they touch stays L2-resident.  A warp's R only grows, so it finds its isolate by
// walking forward through read_base (shared memory) and reloads the isolate's
// descriptor only when it crosses a boundary.
#include "fbk_device.cuh"
#include "fbk_kernels.cuh"
#include "fbk_table.cuh"

namespace fbk {

__device__ __forceinline__ uint32_t iso_walk(const unsigned long long* s_base, uint32_t n_iso, uint32_t i, uint64_t R) {
    while (i + 1 < n_iso && R >= s_base[i + 1]) ++i;
    return i;
}

__device__ __forceinline__ uint32_t load_bases(const unsigned long long* read_base, uint32_t n_iso, unsigned long long* s_base) {
    for (uint32_t i = threadIdx.x; i <= n_iso; i += blockDim.x) s_base[i] = read_base[i];
    __syncthreads();
    return 0;
}

// Pass 1 (build.rs:90-116) for rows [r0, r1) of every isolate's sketch, plus the
// p=12 HyperLogLog of its keys when do_hll.  Only keys whose hash has its low
// log2(BATCH_HLL_SAMPLE) bits zero enter the registers (the host scales the estimate
// back; it only sizes the table).  The registers (16 KB per isolate) are read
// through L2, where the atomics land, so an atomicMax is issued only when it raises
// a register.  (A read through the non-coherent cache would keep returning zeros and
// turn every sampled key into an atomic on 4096 hot words.)
template <int NW>
__global__ void __launch_bounds__(256) k_batch_pass1(const IsoDev* __restrict__ iso, const unsigned long long* __restrict__ read_base,
                                                     uint32_t n_iso, uint32_t k, uint32_t r0, uint32_t r1, int do_hll) {
    __shared__ unsigned long long s_base[BATCH_MAX_ISO + 1];
    load_bases(read_base, n_iso, s_base);
    const uint64_t total = s_base[n_iso];
    const uint32_t lane = threadIdx.x & 31;
    const uint64_t gw = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    uint32_t ci = 0, cur = 0xFFFFFFFFu;
    BankDev b{};
    uint32_t* cnt = nullptr;
    uint32_t* hll = nullptr;
    uint64_t wmask = 0, base = 0;
    uint32_t log2w = 0;
    for (uint64_t R = gw; R < total; R += nwarps) {
        ci = iso_walk(s_base, n_iso, ci, R);
        if (ci != cur) {
            cur = ci;
            b = iso[ci].b;
            cnt = iso[ci].cnt;
            log2w = iso[ci].log2w;
            wmask = (1ULL << log2w) - 1;
            hll = do_hll ? iso[ci].hll12 : nullptr;
            base = s_base[ci];
        }
        const uint64_t r = R - base;
        const uint32_t len = b.len[r];
        if (len < k || !bank_keep(b, r)) continue;
        const uint64_t off = b.off[r];
        const uint32_t nk = len - k + 1;
        for (uint32_t i = lane; i < nk; i += 32) {
            Key<NW> can;
            bool rc;
            window_canonical<NW>(b.data, off + i, k, can, rc);
            const uint64_t key = key_fold<NW>(can);
            for (uint32_t row = r0; row < r1; ++row) {
                const uint64_t col = smix(key ^ cms_seed((int)row)) & wmask;
                atomicAdd(cnt + ((uint64_t)row << log2w) + col, 1u);
            }
            const uint64_t h0 = smix(key ^ cms_seed(0));
            if (hll && (h0 & (BATCH_HLL_SAMPLE - 1)) == 0) {
                uint32_t idx, rho;
                hll_idx_rho(h0, 12, idx, rho);
                if (__ldcg(&hll[idx]) < rho) atomicMax(&hll[idx], rho);
            }
        }
    }
}

// Solidity bitmap (build.rs:259-267) for rows [r0, r1) of every isolate: a window's
// bit is cleared when its capped count in any of these rows is below t_solid.
template <int NW>
__global__ void __launch_bounds__(256) k_batch_solid(const IsoDev* __restrict__ iso, const unsigned long long* __restrict__ read_base,
                                                     uint32_t n_iso, uint32_t k, uint32_t r0, uint32_t r1) {
    __shared__ unsigned long long s_base[BATCH_MAX_ISO + 1];
    load_bases(read_base, n_iso, s_base);
    const uint64_t total = s_base[n_iso];
    const uint32_t lane = threadIdx.x & 31;
    const uint64_t gw = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    uint32_t ci = 0, cur = 0xFFFFFFFFu;
    BankDev b{};
    const uint32_t* cnt = nullptr;
    uint32_t* bm = nullptr;
    uint64_t wmask = 0, base = 0;
    uint32_t log2w = 0, t_solid = 0, cap = 0;
    for (uint64_t R = gw; R < total; R += nwarps) {
        ci = iso_walk(s_base, n_iso, ci, R);
        if (ci != cur) {
            cur = ci;
            b = iso[ci].b;
            cnt = iso[ci].cnt;
            bm = iso[ci].bm;
            log2w = iso[ci].log2w;
            wmask = (1ULL << log2w) - 1;
            t_solid = iso[ci].t_solid;
            cap = iso[ci].cap;
            base = s_base[ci];
        }
        const uint64_t r = R - base;
        const uint32_t len = b.len[r];
        if (len < k + 1 || !bank_keep(b, r)) continue;
        const uint64_t off = b.off[r];
        const uint32_t nk = len - k + 1;
        for (uint32_t it = 0; it < ((nk + 31) >> 5); ++it) {
            const uint32_t q = (it << 5) + lane;
            bool clr = false;
            if (q < nk) {
                Key<NW> can;
                bool rc;
                window_canonical<NW>(b.data, off + q, k, can, rc);
                const uint64_t key = key_fold<NW>(can);
                for (uint32_t row = r0; row < r1; ++row) {
                    const uint64_t col = smix(key ^ cms_seed((int)row)) & wmask;
                    uint32_t c = __ldg(cnt + ((uint64_t)row << log2w) + col);
                    c = c < cap ? c : cap;
                    clr |= c < t_solid;
                }
            }
            const uint32_t m = __ballot_sync(0xffffffffu, clr);
            if (lane == 0 && m) {
                const uint64_t g0 = off + ((uint64_t)it << 5);
                const uint32_t sh = (uint32_t)(g0 & 31);
                atomicAnd(&bm[g0 >> 5], ~(m << sh));
                if (sh) atomicAnd(&bm[(g0 >> 5) + 1], ~(m >> (32 - sh)));
            }
        }
    }
}

// Ladder forms (fbk_k_ladder.cu has the single-isolate kernels and the argument):
// level j of (row, col) is set once the count reached j + 1; the top level is t_solid.
template <int NW>
__global__ void __launch_bounds__(256, 4) k_batch_lpass1(const IsoDev* __restrict__ iso, const unsigned long long* __restrict__ read_base,
                                                         uint32_t n_iso, uint32_t k) {
    __shared__ unsigned long long s_base[BATCH_MAX_ISO + 1];
    load_bases(read_base, n_iso, s_base);
    const uint64_t total = s_base[n_iso];
    const uint32_t lane = threadIdx.x & 31;
    const uint64_t gw = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    uint32_t ci = 0, cur = 0xFFFFFFFFu;
    BankDev b{};
    uint32_t* lad = nullptr;
    uint32_t* top = nullptr;
    uint32_t* hll = nullptr;
    uint64_t wmask = 0, base = 0, level_words = 0;
    uint32_t log2w = 0, t = 1;
    for (uint64_t R = gw; R < total; R += nwarps) {
        ci = iso_walk(s_base, n_iso, ci, R);
        if (ci != cur) {
            cur = ci;
            b = iso[ci].b;
            lad = iso[ci].lad;
            log2w = iso[ci].log2w;
            t = iso[ci].t_solid;
            wmask = (1ULL << log2w) - 1;
            level_words = (4ULL << log2w) >> 5;
            top = lad + (uint64_t)(t - 1) * level_words;
            hll = iso[ci].hll12;
            base = s_base[ci];
        }
        const uint64_t r = R - base;
        const uint32_t len = b.len[r];
        if (len < k || !bank_keep(b, r)) continue;
        const uint64_t off = b.off[r];
        const uint32_t nk = len - k + 1;
        for (uint32_t it = 0; it < ((nk + 31) >> 5); ++it) {
            const uint32_t q = (it << 5) + lane;
            if (q >= nk) continue;
            Key<NW> can;
            bool rc;
            window_canonical<NW>(b.data, off + q, k, can, rc);
            const uint64_t key = key_fold<NW>(can);
            const uint64_t h0 = smix(key ^ cms_seed(0));
            uint32_t wd[4], mk[4];
            bool climb[4];
#pragma unroll
            for (int row = 0; row < 4; ++row) {
                const uint64_t h = row == 0 ? h0 : smix(key ^ cms_seed(row));
                const uint32_t bit = ((uint32_t)row << log2w) + (uint32_t)(h & wmask);
                wd[row] = bit >> 5;
                mk[row] = 1u << (bit & 31);
            }
#pragma unroll
            for (int row = 0; row < 4; ++row) climb[row] = !(__ldcg(top + wd[row]) & mk[row]);
            ladder_climb<4>(lad, level_words, t, wd, mk, climb);
            if ((h0 & (BATCH_HLL_SAMPLE - 1)) == 0) {
                uint32_t idx, rho;
                hll_idx_rho(h0, 12, idx, rho);
                if (__ldcg(&hll[idx]) < rho) atomicMax(&hll[idx], rho);
            }
        }
    }
}

// Exact number of pass-2 records of every isolate (windows that are solid and have
// a solid neighbour inside their read), which sizes the record buckets, and the
// k-mer occurrences of the two passes over kept reads: n_records[0] records,
// [1] windows of reads with len >= k, [2] windows of reads with len >= k + 1.
__global__ void __launch_bounds__(256) k_batch_count(const IsoDev* __restrict__ iso, const unsigned long long* __restrict__ read_base,
                                                     uint32_t n_iso, uint32_t k) {
    __shared__ unsigned long long s_base[BATCH_MAX_ISO + 1];
    load_bases(read_base, n_iso, s_base);
    const uint64_t total = s_base[n_iso];
    const uint32_t lane = threadIdx.x & 31;
    const uint64_t gw = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    uint32_t ci = 0, cur = 0xFFFFFFFFu;
    BankDev b{};
    const uint32_t* bm = nullptr;
    uint64_t base = 0;
    unsigned long long acc = 0, w1 = 0, w2 = 0;
    for (uint64_t R = gw; R < total; R += nwarps) {
        ci = iso_walk(s_base, n_iso, ci, R);
        if (ci != cur) {
            if (lane == 0 && cur != 0xFFFFFFFFu) {
                atomicAdd(iso[cur].n_records, acc);
                atomicAdd(iso[cur].n_records + 1, w1);
                atomicAdd(iso[cur].n_records + 2, w2);
            }
            acc = w1 = w2 = 0;
            cur = ci;
            b = iso[ci].b;
            bm = iso[ci].bm;
            base = s_base[ci];
        }
        const uint64_t r = R - base;
        const uint32_t len = b.len[r];
        if (len < k || !bank_keep(b, r)) continue;
        w1 += len - k + 1;
        if (len < k + 1) continue;
        w2 += len - k + 1;
        if (!bm) continue;  // a ladder gate: the records are bounded by the windows
        const uint64_t off = b.off[r];
        const uint32_t nk = len - k + 1;
        for (uint32_t q = lane; q < ((nk + 31) & ~31u); q += 32) {
            bool e = false;
            if (q < nk) {
                const uint64_t g = off + q;
                e = bm_bit(bm, g) && ((q > 0 && bm_bit(bm, g - 1)) || (q + 1 < nk && bm_bit(bm, g + 1)));
            }
            acc += __popc(__ballot_sync(0xffffffffu, e));
        }
    }
    if (lane == 0 && cur != 0xFFFFFFFFu) {
        atomicAdd(iso[cur].n_records, acc);
        atomicAdd(iso[cur].n_records + 1, w1);
        atomicAdd(iso[cur].n_records + 2, w2);
    }
}

// Pass 2, record form (build.rs:242-289): the records of every isolate go to that
// isolate's buckets; a warp flushes its staging buffer when it moves to the next
// isolate.
template <int NW>
__global__ void __launch_bounds__(256) k_batch_emit(const IsoDev* __restrict__ iso, const unsigned long long* __restrict__ read_base,
                                                    uint32_t n_iso, uint32_t k, uint32_t stripes) {
    extern __shared__ uint64_t emit_smem[];
    __shared__ unsigned long long s_base[BATCH_MAX_ISO + 1];
    load_bases(read_base, n_iso, s_base);
    const uint64_t total = s_base[n_iso];
    const uint32_t lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    uint64_t* buf = emit_smem + (uint64_t)wib * EMIT_WARP_WORDS(NW);
    uint8_t* bbuf = reinterpret_cast<uint8_t*>(buf + emit_buf(NW) * (NW + 1));
    uint16_t* rank = reinterpret_cast<uint16_t*>(bbuf + emit_buf(NW));
    uint32_t* hist = reinterpret_cast<uint32_t*>(rank + emit_buf(NW));
    unsigned long long* gbase = reinterpret_cast<unsigned long long*>(hist + EMIT_MAX_BUCKETS);
    uint16_t* perm = reinterpret_cast<uint16_t*>(gbase + EMIT_MAX_BUCKETS);
    const uint64_t gw = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    const uint32_t stripe = (uint32_t)(gw % stripes);
    uint32_t ci = 0, cur = 0xFFFFFFFFu, n_buf = 0;
    BankDev b{};
    const uint32_t* bm = nullptr;
    BucketDev bk{};
    uint64_t base = 0;
    for (uint64_t R = gw; R < total; R += nwarps) {
        ci = iso_walk(s_base, n_iso, ci, R);
        if (ci != cur) {
            if (n_buf) {
                __syncwarp();
                emit_flush<NW>(bk, stripe, lane, buf, bbuf, n_buf, hist, gbase, rank, perm);
                n_buf = 0;
            }
            cur = ci;
            b = iso[ci].b;
            bm = iso[ci].bm;
            bk = iso[ci].bk;
            base = s_base[ci];
        }
        const uint64_t r = R - base;
        const uint32_t len = b.len[r];
        if (len < k + 1 || !bank_keep(b, r)) continue;
        const uint64_t off = b.off[r];
        const uint32_t nk = len - k + 1;
        for (uint32_t it = 0; it < ((nk + 31) >> 5); ++it) {
            const uint32_t q = (it << 5) + lane;
            bool emit = false;
            Key<NW> key;
            uint32_t info = 0, bucket = 0;
            if (q < nk) {
                const uint64_t g = off + q;
                const bool sq = bm_bit(bm, g);
                const bool sl = q > 0 && bm_bit(bm, g - 1);
                const bool sr = q + 1 < nk && bm_bit(bm, g + 1);
                emit = sq && (sl || sr);
                if (emit) {
                    bool rc;
                    window_canonical<NW>(b.data, g, k, key, rc);
                    if (sr) info |= 8u | (base_at(b.data, g + k) + (rc ? 4u : 0u));
                    if (sl) info |= (8u | ((3u - base_at(b.data, g - 1)) + (rc ? 0u : 4u))) << 4;
                    bucket = bucket_of(key_fold<NW>(key), bk.n_buckets);
                }
            }
            const uint32_t active = __ballot_sync(0xffffffffu, emit);
            if (emit) {
                const uint32_t pos = n_buf + __popc(active & ((1u << lane) - 1));
                rec_put<NW>(buf + pos * (NW + 1), key, info, bk);
                bbuf[pos] = (uint8_t)bucket;
            }
            n_buf += __popc(active);
            if (n_buf > emit_buf(NW) - 32) {
                __syncwarp();
                emit_flush<NW>(bk, stripe, lane, buf, bbuf, n_buf, hist, gbase, rank, perm);
                n_buf = 0;
            }
        }
    }
    __syncwarp();
    if (n_buf) emit_flush<NW>(bk, stripe, lane, buf, bbuf, n_buf, hist, gbase, rank, perm);
}

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
template <class K>
static int grid_of(K kernel, const Launch& L, size_t smem) {
    if (L.grid > 0) return L.grid;
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, L.block, smem) != cudaSuccess || per_sm < 1) per_sm = 1;
    return per_sm * (L.sms > 0 ? L.sms : 1);
}

template <int NW>
static cudaError_t bpass1(const Launch& L, const IsoDev* iso, const unsigned long long* rb, uint32_t n, uint32_t k, uint32_t r0,
                          uint32_t r1, int hll) {
    k_batch_pass1<NW><<<grid_of(k_batch_pass1<NW>, L, 0), L.block, 0, L.stream>>>(iso, rb, n, k, r0, r1, hll);
    return cudaGetLastError();
}
cudaError_t launch_batch_pass1(int nw, const Launch& L, const IsoDev* iso, const unsigned long long* read_base, uint32_t n_iso,
                               uint32_t k, uint32_t r0, uint32_t r1, int do_hll) {
    if (n_iso > BATCH_MAX_ISO) return cudaErrorInvalidValue;
    if (nw == 1) return bpass1<1>(L, iso, read_base, n_iso, k, r0, r1, do_hll);
    if (nw == 2) return bpass1<2>(L, iso, read_base, n_iso, k, r0, r1, do_hll);
    return bpass1<4>(L, iso, read_base, n_iso, k, r0, r1, do_hll);
}

template <int NW>
static cudaError_t bsolid(const Launch& L, const IsoDev* iso, const unsigned long long* rb, uint32_t n, uint32_t k, uint32_t r0,
                          uint32_t r1) {
    k_batch_solid<NW><<<grid_of(k_batch_solid<NW>, L, 0), L.block, 0, L.stream>>>(iso, rb, n, k, r0, r1);
    return cudaGetLastError();
}
cudaError_t launch_batch_solid(int nw, const Launch& L, const IsoDev* iso, const unsigned long long* read_base, uint32_t n_iso,
                               uint32_t k, uint32_t r0, uint32_t r1) {
    if (n_iso > BATCH_MAX_ISO) return cudaErrorInvalidValue;
    if (nw == 1) return bsolid<1>(L, iso, read_base, n_iso, k, r0, r1);
    if (nw == 2) return bsolid<2>(L, iso, read_base, n_iso, k, r0, r1);
    return bsolid<4>(L, iso, read_base, n_iso, k, r0, r1);
}

template <int NW>
static cudaError_t blp1(const Launch& L, const IsoDev* iso, const unsigned long long* rb, uint32_t n, uint32_t k) {
    k_batch_lpass1<NW><<<grid_of(k_batch_lpass1<NW>, L, 0), L.block, 0, L.stream>>>(iso, rb, n, k);
    return cudaGetLastError();
}
cudaError_t launch_batch_lpass1(int nw, const Launch& L, const IsoDev* iso, const unsigned long long* read_base, uint32_t n_iso,
                                uint32_t k) {
    if (n_iso > BATCH_MAX_ISO) return cudaErrorInvalidValue;
    if (nw == 1) return blp1<1>(L, iso, read_base, n_iso, k);
    if (nw == 2) return blp1<2>(L, iso, read_base, n_iso, k);
    return blp1<4>(L, iso, read_base, n_iso, k);
}
cudaError_t launch_batch_count(const Launch& L, const IsoDev* iso, const unsigned long long* read_base, uint32_t n_iso, uint32_t k) {
    if (n_iso > BATCH_MAX_ISO) return cudaErrorInvalidValue;
    k_batch_count<<<grid_of(k_batch_count, L, 0), L.block, 0, L.stream>>>(iso, read_base, n_iso, k);
    return cudaGetLastError();
}

template <int NW>
static cudaError_t bemit(const Launch& L, const IsoDev* iso, const unsigned long long* rb, uint32_t n, uint32_t k, uint32_t S) {
    const size_t smem = (size_t)(L.block / 32) * EMIT_WARP_WORDS(NW) * 8;
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(k_batch_emit<NW>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
    }
    k_batch_emit<NW><<<grid_of(k_batch_emit<NW>, L, smem), L.block, smem, L.stream>>>(iso, rb, n, k, S);
    return cudaGetLastError();
}
cudaError_t launch_batch_emit(int nw, const Launch& L, const IsoDev* iso, const unsigned long long* read_base, uint32_t n_iso,
                              uint32_t k, uint32_t stripes) {
    if (n_iso > BATCH_MAX_ISO || stripes == 0 || stripes > 256) return cudaErrorInvalidValue;
    if (nw == 1) return bemit<1>(L, iso, read_base, n_iso, k, stripes);
    if (nw == 2) return bemit<2>(L, iso, read_base, n_iso, k, stripes);
    return bemit<4>(L, iso, read_base, n_iso, k, stripes);
}

}  // namespace fbk
