// fbk_k_pass.cu — build front-end kernels: pass 1 (CMS update), pass 2 (CMS-gated
// transitions into the open-addressing solid table) and the SolidKmerNode
// conversion (src/graph/build.rs:84-328).
//
// Work split: one warp per read (reads are ~150-300 bases), lane j handles the
// k-mer windows j, j+32, ... of the read, each computed directly from the packed
// bank (no rolling dependency).  The grid is persistent (a multiple of the SM
// count) and warps stride over the read range.
#include <cuda/atomic>

#include "fbk_device.cuh"
#include "fbk_kernels.cuh"

namespace fbk {

static constexpr uint64_t TABLE_SALT = 0x6a09e667f3bcc908ULL;
static constexpr uint64_t FP_SALT = 0xbb67ae8584caa73bULL;
static constexpr uint64_t TAG_READY = 1ULL << 63;
static constexpr uint64_t KEY_EMPTY = ~0ULL;

// ---------------------------------------------------------------------------
// Pass 1 — build.rs:90-116 (mult = 1) and the prior-contig weighting x10
// (build.rs:118-138, mult = 10: ten saturating increments == one add of 10).
// ---------------------------------------------------------------------------
template <int NW, int CB>
__global__ void __launch_bounds__(256) k_pass1(BankDev b, uint32_t k, uint32_t* __restrict__ cms, uint32_t log2w,
                                               uint32_t mult, uint32_t* __restrict__ hll12) {
    __shared__ uint32_t s_hll[4096];
    const bool do_hll = hll12 != nullptr;
    if (do_hll) {
        for (int i = threadIdx.x; i < 4096; i += blockDim.x) s_hll[i] = 0;
        __syncthreads();
    }
    const uint32_t lane = threadIdx.x & 31;
    const uint64_t gw = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    for (uint64_t r = b.r_begin + gw; r < b.r_end; r += nwarps) {
        const uint32_t len = b.len[r];
        if (len < k || !bank_keep(b, r)) continue;
        const uint64_t off = b.off[r];
        const uint32_t nk = len - k + 1;
        for (uint32_t i = lane; i < nk; i += 32) {
            Key<NW> can;
            bool rc;
            window_canonical<NW>(b.data, off + i, k, can, rc);
            const uint64_t key = key_fold<NW>(can);
            uint64_t c[4];
#pragma unroll
            for (int rr = 0; rr < 4; ++rr) c[rr] = cms_index(key, rr, log2w);
#pragma unroll
            for (int rr = 0; rr < 4; ++rr) cms_sat_add<CB>(cms, c[rr], mult);
            if (do_hll) {
                // Any bijective hash of the key serves the distinct count.
                uint32_t idx, rho;
                hll_idx_rho(smix(key ^ cms_seed(0)), 12, idx, rho);
                if (s_hll[idx] < rho) atomicMax(&s_hll[idx], rho);
            }
        }
    }
    if (do_hll) {
        __syncthreads();
        for (int i = threadIdx.x; i < 4096; i += blockDim.x) {
            const uint32_t v = s_hll[i];
            if (v) atomicMax(&hll12[i], v);
        }
    }
}

// ---------------------------------------------------------------------------
// Solid table probing
// ---------------------------------------------------------------------------
__device__ __forceinline__ int64_t table_slot1(const TableDev& t, uint64_t key, uint32_t* status) {
    uint64_t s = smix(key ^ TABLE_SALT) & t.mask;
    for (uint32_t probe = 0; probe < t.max_probe; ++probe) {
        const uint64_t cur = __ldcg(&t.keys[s]);
        if (cur == key) return (int64_t)s;
        if (cur == KEY_EMPTY) {
            const uint64_t old = atomicCAS((unsigned long long*)&t.keys[s], KEY_EMPTY, key);
            if (old == KEY_EMPTY || old == key) return (int64_t)s;
        }
        s = (s + 1) & t.mask;
    }
    atomicOr(status, ST_TABLE_FULL);
    return -1;
}

template <int NW>
__device__ __forceinline__ int64_t table_slotw(const TableDev& t, const Key<NW>& key, uint32_t* status) {
    const uint64_t f = key_fold<NW>(key);
    uint64_t s = smix(f ^ TABLE_SALT) & t.mask;
    const uint64_t fp = (smix(f ^ FP_SALT) | 1ULL) & ~TAG_READY;
    for (uint32_t probe = 0; probe < t.max_probe; ++probe) {
        cuda::atomic_ref<unsigned long long, cuda::thread_scope_device> tag_ref(*(unsigned long long*)&t.tags[s]);
        uint64_t tag = tag_ref.load(cuda::memory_order_acquire);
        if (tag == 0) {
            const uint64_t old = atomicCAS((unsigned long long*)&t.tags[s], 0ULL, fp);
            if (old == 0) {
#pragma unroll
                for (int i = 0; i < NW; ++i) __stcg(&t.keys[s * NW + i], key.w[i]);
                tag_ref.fetch_or(TAG_READY, cuda::memory_order_release);
                return (int64_t)s;
            }
            tag = old;
        }
        if ((tag & ~TAG_READY) == fp) {
            // Same fingerprint: wait (bounded) until the claiming thread has published
            // the key words, then compare them.
            uint32_t spins = 0;
            while (!(tag & TAG_READY)) {
                if (++spins > t.spin_limit) {
                    atomicOr(status, ST_SPIN_TIMEOUT);
                    return -1;
                }
                __nanosleep(64);
                tag = tag_ref.load(cuda::memory_order_acquire);
            }
            bool eq = true;
#pragma unroll
            for (int i = 0; i < NW; ++i) eq &= (__ldcg(&t.keys[s * NW + i]) == key.w[i]);
            if (eq) return (int64_t)s;
        }
        s = (s + 1) & t.mask;
    }
    atomicOr(status, ST_TABLE_FULL);
    return -1;
}

template <int NW>
__device__ __forceinline__ int64_t table_slot(const TableDev& t, const Key<NW>& key, uint32_t* status) {
    if constexpr (NW == 1) return table_slot1(t, key.w[0], status);
    else return table_slotw<NW>(t, key, status);
}

// ---------------------------------------------------------------------------
// Pass 2 — build.rs:242-289 (gate = 1, w_edge = 1, w_cov = 1) and the prior-contig
// backbone (build.rs:202-240: gate = 0, w_edge = 1000, w_cov = 100).
//
// For the transition (u, v) between windows q and q+1 the reference pushes
// (u_can, base(q+k) + 4*u_rc) and (v_can, (3 - base(q)) + 4*!v_rc), each push adding
// to cov and to one edge counter.  Here the owner lane of window q performs both
// pushes that concern its own key: as u of (q, q+1) and as v of (q-1, q).  The
// solidity of the neighbours comes from warp ballots; a window's pushes are issued
// one iteration later, once the ballot of the next 32 windows is known.
// ---------------------------------------------------------------------------
template <int NW, int CB>
__global__ void __launch_bounds__(256) k_pass2(BankDev b, uint32_t k, const uint32_t* __restrict__ cms, uint32_t log2w,
                                               uint32_t t_solid, int gate, uint32_t w_edge, uint32_t w_cov, TableDev t,
                                               uint32_t* status) {
    const uint32_t lane = threadIdx.x & 31;
    const uint64_t gw = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    for (uint64_t r = b.r_begin + gw; r < b.r_end; r += nwarps) {
        const uint32_t len = b.len[r];
        if (len < k + 1 || !bank_keep(b, r)) continue;
        const uint64_t off = b.off[r];
        const uint32_t nk = len - k + 1;
        const uint32_t n_it = (nk + 31) >> 5;
        uint32_t m_prev2 = 0, m_prev = 0;
        Key<NW> pkey;
#pragma unroll
        for (int i = 0; i < NW; ++i) pkey.w[i] = 0;
        bool prc = false;
        for (uint32_t it = 0; it <= n_it; ++it) {
            uint32_t m_cur = 0;
            Key<NW> ckey;
#pragma unroll
            for (int i = 0; i < NW; ++i) ckey.w[i] = 0;
            bool crc = false;
            if (it < n_it) {
                const uint32_t p = (it << 5) + lane;
                bool solid = false;
                if (p < nk) {
                    window_canonical<NW>(b.data, off + p, k, ckey, crc);
                    solid = !gate || cms_estimate<CB>(cms, key_fold<NW>(ckey), log2w) >= t_solid;
                }
                m_cur = __ballot_sync(0xffffffffu, solid);
            }
            if (it > 0 && ((m_prev >> lane) & 1u)) {
                const uint32_t q = ((it - 1) << 5) + lane;
                const bool sl = lane > 0 ? ((m_prev >> (lane - 1)) & 1u) : ((m_prev2 >> 31) & 1u);
                const bool sr = lane < 31 ? ((m_prev >> (lane + 1)) & 1u) : (m_cur & 1u);
                if (sl || sr) {
                    const int64_t s = table_slot<NW>(t, pkey, status);
                    if (s >= 0) {
                        uint32_t* c = t.cnt + (uint64_t)s * 8;
                        if (sr) atomicAdd(&c[base_at(b.data, off + q + k) + (prc ? 4u : 0u)], w_edge);
                        if (sl) atomicAdd(&c[(3u - base_at(b.data, off + q - 1)) + (prc ? 0u : 4u)], w_edge);
                        if (t.cov) atomicAdd(&t.cov[s], w_cov * ((sl ? 1u : 0u) + (sr ? 1u : 0u)));
                    }
                }
            }
            m_prev2 = m_prev;
            m_prev = m_cur;
            pkey = ckey;
            prc = crc;
        }
    }
}

// ---------------------------------------------------------------------------
// SolidKmerNode conversion — build.rs:302-328.  Edge counters are exact u32 sums
// (clamped to 65535 between chunks when a bank is large), so the reference's
// saturating u16 values are min(65535, count).  cov is the saturating sum of all
// pushes: min(65535, sum of edges) — the clamp commutes because the increments
// are positive — or the separate cov counter when prior contigs were added.
// ---------------------------------------------------------------------------
// Each block handles tiles of 256 threads x 8 consecutive slots; output rows are
// reserved with one atomic per tile (block-wide prefix sums in shared memory), and
// the key count, digest and raw edge total are accumulated per thread and added
// once per warp at the end.
constexpr int CONV_SLOTS = 8;

__device__ __forceinline__ uint32_t block_excl_scan(uint32_t v, uint32_t* s_warp, uint32_t& total) {
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= (uint32_t)o) x += y;
    }
    if (lane == 31) s_warp[warp] = x;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = lane < nwarp ? s_warp[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= (uint32_t)o) w += y;
        }
        if (lane < nwarp) s_warp[lane] = w;  // inclusive prefix of warp totals
    }
    __syncthreads();
    total = s_warp[nwarp - 1];
    const uint32_t before = warp ? s_warp[warp - 1] : 0;
    __syncthreads();
    return before + x - v;
}

template <int NW>
__global__ void __launch_bounds__(256) k_convert(TableDev t, uint32_t min_trans_cov, ConvOut o) {
    __shared__ uint32_t s_warp[32];
    __shared__ unsigned long long s_base[2];
    const uint64_t cap = t.mask + 1;
    const uint64_t tile = (uint64_t)blockDim.x * CONV_SLOTS;
    unsigned long long n_keys = 0, digest = 0, raw_total = 0;
    for (uint64_t base = (uint64_t)blockIdx.x * tile; base < cap; base += (uint64_t)gridDim.x * tile) {
        const uint64_t s0 = base + (uint64_t)threadIdx.x * CONV_SLOTS;
        uint32_t occ_bits = 0, keep_bits = 0;
#pragma unroll
        for (int j = 0; j < CONV_SLOTS; ++j) {
            const uint64_t s = s0 + j;
            if (s >= cap) break;
            const bool occ = NW == 1 ? (t.keys[s] != KEY_EMPTY) : (t.tags[s] != 0);
            occ_bits |= (uint32_t)occ << j;
        }
        // mask per occupied slot (needs the counters)
        uint8_t masks[CONV_SLOTS];
        uint16_t covs[CONV_SLOTS];
#pragma unroll
        for (int j = 0; j < CONV_SLOTS; ++j) {
            masks[j] = 0;
            covs[j] = 0;
            if (!((occ_bits >> j) & 1u)) continue;
            const uint64_t s = s0 + j;
            const uint4* c4 = reinterpret_cast<const uint4*>(t.cnt + s * 8);
            const uint4 a = c4[0], bq = c4[1];
            const uint32_t e[8] = {a.x, a.y, a.z, a.w, bq.x, bq.y, bq.z, bq.w};
            uint32_t sum = 0, m = 0;
#pragma unroll
            for (int i = 0; i < 8; ++i) {
                raw_total += e[i];
                const uint32_t ec = e[i] > 0xFFFFu ? 0xFFFFu : e[i];
                sum += ec;
                if (ec >= min_trans_cov) m |= 1u << i;
            }
            if (t.cov) sum = t.cov[s];
            covs[j] = (uint16_t)(sum > 0xFFFFu ? 0xFFFFu : sum);
            masks[j] = (uint8_t)m;
            keep_bits |= (uint32_t)(m != 0) << j;
        }
        n_keys += __popc(occ_bits);
        uint32_t tot_keep = 0, tot_acc = 0;
        const uint32_t my_keep = __popc(keep_bits);
        const uint32_t off_keep = block_excl_scan(my_keep, s_warp, tot_keep);
        uint32_t off_acc = 0;
        if (o.acc_keys) off_acc = block_excl_scan(__popc(occ_bits), s_warp, tot_acc);
        if (threadIdx.x == 0) {
            s_base[0] = tot_keep ? atomicAdd(&o.counts[1], (unsigned long long)tot_keep) : 0;
            s_base[1] = (o.acc_keys && tot_acc) ? atomicAdd(&o.counts[4], (unsigned long long)tot_acc) : 0;
        }
        __syncthreads();
        uint64_t wk = s_base[0] + off_keep, wa = s_base[1] + off_acc;
        __syncthreads();
        if (!occ_bits) continue;
#pragma unroll
        for (int j = 0; j < CONV_SLOTS; ++j) {
            if (!((occ_bits >> j) & 1u)) continue;
            const uint64_t s = s0 + j;
            Key<NW> key;
#pragma unroll
            for (int i = 0; i < NW; ++i) key.w[i] = t.keys[s * NW + i];
            if (o.acc_keys) {
                if (wa < o.cap_acc) {
#pragma unroll
                    for (int i = 0; i < NW; ++i) o.acc_keys[wa * NW + i] = key.w[i];
                    o.acc_cov[wa] = covs[j];
                    const uint4* c4 = reinterpret_cast<const uint4*>(t.cnt + s * 8);
                    const uint4 a = c4[0], bq = c4[1];
                    const uint32_t e[8] = {a.x, a.y, a.z, a.w, bq.x, bq.y, bq.z, bq.w};
#pragma unroll
                    for (int i = 0; i < 8; ++i) o.acc_edges[wa * 8 + i] = (uint16_t)(e[i] > 0xFFFFu ? 0xFFFFu : e[i]);
                }
                wa++;
            }
            if ((keep_bits >> j) & 1u) {
                uint32_t cv = covs[j] / 2u;
                cv = cv < 1 ? 1 : cv;
                if (o.keys && wk < o.cap_solid) {
#pragma unroll
                    for (int i = 0; i < NW; ++i) o.keys[wk * NW + i] = key.w[i];
                    o.cov[wk] = (uint16_t)cv;
                    o.mask[wk] = masks[j];
                }
                wk++;
                uint64_t kd = 0;
#pragma unroll
                for (int i = 0; i < NW; ++i) kd = smix(kd ^ key.w[i]);
                digest += smix(kd ^ smix(((uint64_t)cv << 8) | masks[j]));
            }
        }
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        digest += __shfl_down_sync(0xffffffffu, digest, off);
        raw_total += __shfl_down_sync(0xffffffffu, raw_total, off);
        n_keys += __shfl_down_sync(0xffffffffu, n_keys, off);
    }
    if ((threadIdx.x & 31) == 0) {
        if (n_keys) atomicAdd(&o.counts[0], n_keys);
        if (digest) atomicAdd(&o.counts[2], digest);
        if (raw_total) atomicAdd(&o.counts[3], raw_total);
    }
}

__global__ void k_clamp(uint32_t* cnt, uint64_t n) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        if (cnt[i] > 0xFFFFu) cnt[i] = 0xFFFFu;
}

__global__ void k_table_init(uint64_t* keys, uint64_t n_keys_words, uint64_t fill) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n_keys_words; i += (uint64_t)gridDim.x * blockDim.x)
        keys[i] = fill;
}

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
template <int NW>
static cudaError_t pass1_nw(int cb, const Launch& L, const BankDev& b, uint32_t k, uint32_t* cms, uint32_t log2w,
                            uint32_t mult, uint32_t* hll12) {
    if (cb == 4) k_pass1<NW, 4><<<L.grid, L.block, 0, L.stream>>>(b, k, cms, log2w, mult, hll12);
    else k_pass1<NW, 16><<<L.grid, L.block, 0, L.stream>>>(b, k, cms, log2w, mult, hll12);
    return cudaGetLastError();
}
cudaError_t launch_pass1(int nw, int cb, const Launch& L, const BankDev& b, uint32_t k, uint32_t* cms, uint32_t log2w,
                         uint32_t mult, uint32_t* hll12) {
    if (nw == 1) return pass1_nw<1>(cb, L, b, k, cms, log2w, mult, hll12);
    if (nw == 2) return pass1_nw<2>(cb, L, b, k, cms, log2w, mult, hll12);
    return pass1_nw<4>(cb, L, b, k, cms, log2w, mult, hll12);
}

template <int NW>
static cudaError_t pass2_nw(int cb, const Launch& L, const BankDev& b, uint32_t k, const uint32_t* cms, uint32_t log2w,
                            uint32_t t_solid, int gate, uint32_t we, uint32_t wc, const TableDev& t, uint32_t* status) {
    if (cb == 4) k_pass2<NW, 4><<<L.grid, L.block, 0, L.stream>>>(b, k, cms, log2w, t_solid, gate, we, wc, t, status);
    else k_pass2<NW, 16><<<L.grid, L.block, 0, L.stream>>>(b, k, cms, log2w, t_solid, gate, we, wc, t, status);
    return cudaGetLastError();
}
cudaError_t launch_pass2(int nw, int cb, const Launch& L, const BankDev& b, uint32_t k, const uint32_t* cms, uint32_t log2w,
                         uint32_t t_solid, int gate, uint32_t w_edge, uint32_t w_cov, const TableDev& t, uint32_t* status) {
    if (nw == 1) return pass2_nw<1>(cb, L, b, k, cms, log2w, t_solid, gate, w_edge, w_cov, t, status);
    if (nw == 2) return pass2_nw<2>(cb, L, b, k, cms, log2w, t_solid, gate, w_edge, w_cov, t, status);
    return pass2_nw<4>(cb, L, b, k, cms, log2w, t_solid, gate, w_edge, w_cov, t, status);
}

cudaError_t launch_convert(int nw, const Launch& L, const TableDev& t, uint32_t min_trans_cov, const ConvOut& o) {
    if (nw == 1) k_convert<1><<<L.grid, L.block, 0, L.stream>>>(t, min_trans_cov, o);
    else if (nw == 2) k_convert<2><<<L.grid, L.block, 0, L.stream>>>(t, min_trans_cov, o);
    else k_convert<4><<<L.grid, L.block, 0, L.stream>>>(t, min_trans_cov, o);
    return cudaGetLastError();
}

cudaError_t launch_clamp_counters(const Launch& L, uint32_t* cnt, uint64_t n) {
    k_clamp<<<L.grid, L.block, 0, L.stream>>>(cnt, n);
    return cudaGetLastError();
}

cudaError_t launch_table_init(int nw, const Launch& L, const TableDev& t) {
    const uint64_t cap = t.mask + 1;
    if (nw == 1) {
        k_table_init<<<L.grid, L.block, 0, L.stream>>>(t.keys, cap, KEY_EMPTY);
        return cudaGetLastError();
    }
    return cudaMemsetAsync(t.tags, 0, cap * sizeof(uint64_t), L.stream);
}

}  // namespace fbk
