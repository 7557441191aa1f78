// fbk_k_pass.cu — build front-end kernels: pass 1 (CMS update), the CMS gate as a
// solidity bitmap, pass 2 (gated transitions into the open-addressing solid table)
// and the SolidKmerNode conversion (src/graph/build.rs:84-328).
//
// Work split: one warp per read (reads are ~150-300 bases), lane j handles the
// k-mer windows j, j+32, ... of the read, each computed directly from the packed
// bank (no rolling dependency).  The grid is persistent (a multiple of the SM
// count) and warps stride over the read range.
#include <cuda/atomic>

#include "fbk_device.cuh"
#include "fbk_kernels.cuh"
#include "fbk_table.cuh"

namespace fbk {


// ---------------------------------------------------------------------------
// Count-Min Sketch on the device.  The sketch keeps an exact u32 count per
// (row, column) — count_r(col) — and every reader applies the reference's cap:
// the nibble value is min(15, count), the u16 value min(65535, count).  This is
// the same as the reference's saturating increments (sketch.rs:199-221) because
// increments are positive: min(cap, min(cap, a) + b) = min(cap, a + b).  Counts are
// clamped to 65535 between launches, and a launch adds less than 2^32 - 2^17 in
// total, so no u32 wraps.  The gain: an increment is one fire-and-forget RED.ADD
// instead of a load + CAS round trip.
//
// Pass 1 — build.rs:90-116 (mult = 1) and the prior-contig weighting x10
// (build.rs:118-138, mult = 10).  One launch is one sweep over the bank that adds
// only the k-mers whose column in row `row` falls in [c0, c1): the host sizes the
// column range so the sweep's slice of the sketch (~64 MB) stays resident in L2,
// and runs the sweeps for all rows and ranges back to back.
// ---------------------------------------------------------------------------
template <int NW>
__global__ void __launch_bounds__(256) k_pass1_sweep(BankDev b, uint32_t k, uint32_t* __restrict__ cnt, uint32_t log2w,
                                                     uint32_t r0, uint32_t r1, uint64_t c0, uint64_t c1, uint32_t mult,
                                                     uint32_t* __restrict__ hll12) {
    __shared__ uint32_t s_hll[4096];
    const bool do_hll = hll12 != nullptr;
    if (do_hll) {
        for (int i = threadIdx.x; i < 4096; i += blockDim.x) s_hll[i] = 0;
        __syncthreads();
    }
    const uint64_t wmask = (1ULL << log2w) - 1, span = c1 - c0, seed0 = cms_seed((int)r0);
    uint32_t* row0 = cnt + ((uint64_t)r0 << log2w);
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
            if (r1 == r0 + 1) {
                const uint64_t col = smix(key ^ seed0) & wmask;
                if (col - c0 < span) atomicAdd(row0 + col, mult);
            } else {
                for (uint32_t row = r0; row < r1; ++row) {
                    const uint64_t col = smix(key ^ cms_seed((int)row)) & wmask;
                    if (col - c0 < span) atomicAdd(cnt + ((uint64_t)row << log2w) + col, mult);
                }
            }
            if (do_hll) {
                // any bijective hash of the key serves the distinct count; the keys
                // whose hash has its low 4 bits zero (1 in 16) are counted
                const uint64_t h = smix(key ^ cms_seed(0));
                if ((h & (PASS1_HLL_SAMPLE - 1)) == 0) {
                    uint32_t idx, rho;
                    hll_idx_rho(h, 12, idx, rho);
                    if (s_hll[idx] < rho) atomicMax(&s_hll[idx], rho);
                }
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
// Solidity bitmap — the CMS gate of pass 2 (build.rs:259-267): window q of a read
// is solid iff min_r min(cap, count_r) >= t_solid, i.e. iff every row's capped count
// is >= t_solid.  Bit (off + q) of the bitmap (indexed by the window's first base in
// the bank) starts at 1; each sweep clears the bits of windows whose column in its
// row slice fails the test.  A warp's 32 windows are 32 consecutive bits, so one
// ballot becomes at most two atomicAnd.
// ---------------------------------------------------------------------------
template <int NW>
__global__ void __launch_bounds__(256) k_solid_sweep(BankDev b, uint32_t k, const uint32_t* __restrict__ cnt, uint32_t log2w,
                                                     uint32_t r0, uint32_t r1, uint64_t c0, uint64_t c1, uint32_t t_solid,
                                                     uint32_t cap, uint32_t* __restrict__ bm) {
    const uint64_t wmask = (1ULL << log2w) - 1, span = c1 - c0, seed0 = cms_seed((int)r0);
    const uint32_t* row0 = cnt + ((uint64_t)r0 << log2w);
    const uint32_t lane = threadIdx.x & 31;
    const uint64_t gw = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    for (uint64_t r = b.r_begin + gw; r < b.r_end; r += nwarps) {
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
                if (r1 == r0 + 1) {
                    const uint64_t col = smix(key ^ seed0) & wmask;
                    if (col - c0 < span) {
                        uint32_t c = __ldg(row0 + col);
                        c = c < cap ? c : cap;
                        clr = c < t_solid;
                    }
                } else {
                    for (uint32_t row = r0; row < r1; ++row) {
                        const uint64_t col = smix(key ^ cms_seed((int)row)) & wmask;
                        if (col - c0 < span) {
                            uint32_t c = __ldg(cnt + ((uint64_t)row << log2w) + col);
                            c = c < cap ? c : cap;
                            clr |= c < t_solid;
                        }
                    }
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

// ---------------------------------------------------------------------------
// Pass 2 — build.rs:242-289 (gate = 1, w_edge = 1, w_cov = 1) and the prior-contig
// backbone (build.rs:202-240: gate = 0, w_edge = 1000, w_cov = 100).
//
// For the transition (u, v) between windows q and q+1 the reference pushes
// (u_can, base(q+k) + 4*u_rc) and (v_can, (3 - base(q)) + 4*!v_rc), each push adding
// to cov and to one edge counter.  Here the lane of window q makes both pushes that
// concern its own key — as u of (q, q+1) and as v of (q-1, q) — with one probe.
// Solidity comes from the bitmap.  One launch handles the keys whose home slot lies
// in [s0, s1): the host splits the table into slot ranges whose hot part fits L2 and
// sweeps the bank once per range; every occurrence of a key lands in the same sweep.
// ---------------------------------------------------------------------------

template <int NW>
__global__ void __launch_bounds__(256) k_pass2_sweep(BankDev b, uint32_t k, const uint32_t* __restrict__ bm, int gate,
                                                     uint64_t s0, uint64_t s1, uint32_t w_edge, uint32_t w_cov, TableDev t,
                                                     uint32_t* status) {
    const uint64_t span = s1 - s0;
    const uint32_t lane = threadIdx.x & 31;
    const uint64_t gw = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    for (uint64_t r = b.r_begin + gw; r < b.r_end; r += nwarps) {
        const uint32_t len = b.len[r];
        if (len < k + 1 || !bank_keep(b, r)) continue;
        const uint64_t off = b.off[r];
        const uint32_t nk = len - k + 1;
        for (uint32_t q = lane; q < nk; q += 32) {
            const uint64_t g = off + q;
            bool sq = true, sl = q > 0, sr = q + 1 < nk;
            if (gate) {
                sq = bm_bit(bm, g);
                sl = sl && bm_bit(bm, g - 1);
                sr = sr && bm_bit(bm, g + 1);
            }
            if (!sq || !(sl || sr)) continue;
            Key<NW> key;
            bool rc;
            window_canonical<NW>(b.data, g, k, key, rc);
            const uint64_t f = key_fold<NW>(key);
            const uint64_t home = home_slot(f, t.cap);
            if (home - s0 >= span) continue;
            int64_t s;
            if constexpr (NW == 1) s = table_slot1(t, key.w[0], home, status);
            else if constexpr (NW == 2) s = table_slot2(t, key, home, status);
            else s = table_slotw<NW>(t, key, f, home, status);
            if (s < 0) continue;
            uint32_t* c = t.cnt + (uint64_t)s * 8;
            if (sr) atomicAdd(&c[base_at(b.data, g + k) + (rc ? 4u : 0u)], w_edge);
            if (sl) atomicAdd(&c[(3u - base_at(b.data, g - 1)) + (rc ? 0u : 4u)], w_edge);
            if (t.cov) atomicAdd(&t.cov[s], w_cov * ((sl ? 1u : 0u) + (sr ? 1u : 0u)));
        }
    }
}

// ---------------------------------------------------------------------------
// Pass 2, record form.  k_emit scans the bank once: every window that is solid and
// has a solid neighbour inside its read yields one record (its canonical key and the
// one or two pushes it makes, same rules as k_pass2_sweep) appended to the bucket of
// its home slot.  k_upsert then processes one bucket per launch: every lane owns a
// record, probes from the home slot and adds the pushes.
// ---------------------------------------------------------------------------
template <int NW>
__global__ void __launch_bounds__(256) k_emit(BankDev b, uint32_t k, const uint32_t* __restrict__ bm, int gate, TableDev t,
                                              BucketDev bk) {
    extern __shared__ uint64_t emit_smem[];
    const uint32_t lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    uint64_t* buf = emit_smem + (uint64_t)wib * EMIT_WARP_WORDS(NW);
    uint8_t* bbuf = reinterpret_cast<uint8_t*>(buf + emit_buf(NW) * (NW + 1));      // emit_buf(NW) bytes
    uint16_t* rank = reinterpret_cast<uint16_t*>(bbuf + emit_buf(NW));              // emit_buf(NW) u16
    uint32_t* hist = reinterpret_cast<uint32_t*>(rank + emit_buf(NW));              // EMIT_MAX_BUCKETS u32
    unsigned long long* gbase = reinterpret_cast<unsigned long long*>(hist + EMIT_MAX_BUCKETS);
    uint16_t* perm = reinterpret_cast<uint16_t*>(gbase + EMIT_MAX_BUCKETS);
    const uint64_t gw = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    const uint32_t stripe = (uint32_t)(gw % bk.stripes);
    uint32_t n_buf = 0;  // warp-uniform
    for (uint64_t r = b.r_begin + gw; r < b.r_end; r += nwarps) {
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
                bool sq = true, sl = q > 0, sr = q + 1 < nk;
                if (gate) {
                    sq = bm_bit(bm, g);
                    sl = sl && bm_bit(bm, g - 1);
                    sr = sr && bm_bit(bm, g + 1);
                }
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

// Record emit with the gate read inline from a threshold ladder (fbk_k_ladder.cu):
// every lane decides its own window's solidity (the top ladder level set in all
// four rows), and a warp walks its read one chunk of 32 windows ahead, so the
// solidity of both neighbours of every window comes from the ballots of the
// previous, current and next chunks.  No solidity bitmap is built or read.
template <int NW>
__device__ __forceinline__ bool ladder_gate(const uint32_t* __restrict__ top, uint32_t log2w, uint64_t key) {
    const uint64_t wmask = (1ULL << log2w) - 1;
    bool ok = true;
#pragma unroll
    for (int row = 0; row < 4; ++row) {
        const uint64_t bit = ((uint64_t)row << log2w) + (smix(key ^ cms_seed(row)) & wmask);
        ok &= (__ldg(top + (bit >> 5)) >> (bit & 31)) & 1u;
    }
    return ok;
}

template <int NW>
__global__ void __launch_bounds__(256) k_emit_ladder(BankDev b, uint32_t k, const uint32_t* __restrict__ lad, uint32_t log2w,
                                                     uint32_t t_solid, TableDev t, BucketDev bk) {
    extern __shared__ uint64_t emit_smem[];
    const uint32_t lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    uint64_t* buf = emit_smem + (uint64_t)wib * EMIT_WARP_WORDS(NW);
    uint8_t* bbuf = reinterpret_cast<uint8_t*>(buf + emit_buf(NW) * (NW + 1));
    uint16_t* rank = reinterpret_cast<uint16_t*>(bbuf + emit_buf(NW));
    uint32_t* hist = reinterpret_cast<uint32_t*>(rank + emit_buf(NW));
    unsigned long long* gbase = reinterpret_cast<unsigned long long*>(hist + EMIT_MAX_BUCKETS);
    uint16_t* perm = reinterpret_cast<uint16_t*>(gbase + EMIT_MAX_BUCKETS);
    const uint32_t* top = lad + (uint64_t)(t_solid - 1) * ((4ULL << log2w) >> 5);
    const uint64_t gw = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    const uint32_t stripe = (uint32_t)(gw % bk.stripes);
    uint32_t n_buf = 0;  // warp-uniform
    for (uint64_t r = b.r_begin + gw; r < b.r_end; r += nwarps) {
        const uint32_t len = b.len[r];
        if (len < k + 1 || !bank_keep(b, r)) continue;
        const uint64_t off = b.off[r];
        const uint32_t nk = len - k + 1;
        const uint32_t n_it = (nk + 31) >> 5;
        Key<NW> kc;
        bool rcc = false, sc = false;
        if (lane < nk) {
            window_canonical<NW>(b.data, off + lane, k, kc, rcc);
            sc = ladder_gate<NW>(top, log2w, key_fold<NW>(kc));
        }
        uint32_t mprev = 0, mcur = __ballot_sync(0xffffffffu, sc);
        for (uint32_t it = 0; it < n_it; ++it) {
            Key<NW> kn;
            bool rcn = false, sn = false;
            const uint32_t qn = ((it + 1) << 5) + lane;
            if (qn < nk) {
                window_canonical<NW>(b.data, off + qn, k, kn, rcn);
                sn = ladder_gate<NW>(top, log2w, key_fold<NW>(kn));
            }
            const uint32_t mnext = __ballot_sync(0xffffffffu, sn);
            const uint32_t q = (it << 5) + lane;
            bool emit = false;
            uint32_t info = 0, bucket = 0;
            if (q < nk) {
                const bool sq = (mcur >> lane) & 1u;
                const bool sl = q > 0 && (lane ? ((mcur >> (lane - 1)) & 1u) : (mprev >> 31));
                const bool sr = q + 1 < nk && (lane < 31 ? ((mcur >> (lane + 1)) & 1u) : (mnext & 1u));
                emit = sq && (sl || sr);
                if (emit) {
                    const uint64_t g = off + q;
                    if (sr) info |= 8u | (base_at(b.data, g + k) + (rcc ? 4u : 0u));
                    if (sl) info |= (8u | ((3u - base_at(b.data, g - 1)) + (rcc ? 0u : 4u))) << 4;
                    bucket = bucket_of(key_fold<NW>(kc), bk.n_buckets);
                }
            }
            const uint32_t active = __ballot_sync(0xffffffffu, emit);
            if (emit) {
                const uint32_t pos = n_buf + __popc(active & ((1u << lane) - 1));
                rec_put<NW>(buf + pos * (NW + 1), kc, info, bk);
                bbuf[pos] = (uint8_t)bucket;
            }
            n_buf += __popc(active);
            if (n_buf > emit_buf(NW) - 32) {
                __syncwarp();
                emit_flush<NW>(bk, stripe, lane, buf, bbuf, n_buf, hist, gbase, rank, perm);
                n_buf = 0;
            }
            mprev = mcur;
            mcur = mnext;
            kc = kn;
            rcc = rcn;
        }
    }
    __syncwarp();
    if (n_buf) emit_flush<NW>(bk, stripe, lane, buf, bbuf, n_buf, hist, gbase, rank, perm);
}

// The same emit with the gate loads of chunk it + 2 in flight while chunk it is
// emitted: a lane holds three keys (chunks it, it + 1, it + 2), the loads of the
// farthest one are issued before the emit work and resolved after it (GateLoads,
// fbk_table.cuh).
// WS = (64*NW - 2k) / 64 is a template parameter: key words below WS are constant
// zeros, which saves their registers and instructions (k = 77 in 256-bit keys: one
// word of four).
template <int NW, int WS>
__global__ void __launch_bounds__(256, 3) k_emit_ladder2(BankDev b, uint32_t k, const uint32_t* __restrict__ lad, uint32_t log2w,
                                                         uint32_t t_solid, TableDev t, BucketDev bk) {
    extern __shared__ uint64_t emit_smem[];
    const uint32_t lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    uint64_t* buf = emit_smem + (uint64_t)wib * EMIT_WARP_WORDS(NW);
    uint8_t* bbuf = reinterpret_cast<uint8_t*>(buf + emit_buf(NW) * (NW + 1));
    uint16_t* rank = reinterpret_cast<uint16_t*>(bbuf + emit_buf(NW));
    uint32_t* hist = reinterpret_cast<uint32_t*>(rank + emit_buf(NW));
    unsigned long long* gbase = reinterpret_cast<unsigned long long*>(hist + EMIT_MAX_BUCKETS);
    uint16_t* perm = reinterpret_cast<uint16_t*>(gbase + EMIT_MAX_BUCKETS);
    const uint32_t* top = lad + (uint64_t)(t_solid - 1) * ((4ULL << log2w) >> 5);
    const uint64_t gw = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    const uint32_t stripe = (uint32_t)(gw % bk.stripes);
    uint32_t n_buf = 0;  // warp-uniform
    for (uint64_t r = b.r_begin + gw; r < b.r_end; r += nwarps) {
        const uint32_t len = b.len[r];
        if (len < k + 1 || !bank_keep(b, r)) continue;
        const uint64_t off = b.off[r];
        const uint32_t nk = len - k + 1;
        const uint32_t n_it = (nk + 31) >> 5;
        // chunks 0 and 1 resolved up front
        Key<NW> k0{}, k1{};
        bool rc0 = false, rc1 = false;
        const bool l0 = lane < nk, l1 = 32 + lane < nk;
        if (l0) canonical_ws<NW, WS>(b.data, off + lane, k, k0, rc0);
        if (l1) canonical_ws<NW, WS>(b.data, off + 32 + lane, k, k1, rc1);
        GateLoads g0, g1;
        gate_issue(top, log2w, l0 ? key_fold<NW>(k0) : 0, l0, g0);
        gate_issue(top, log2w, l1 ? key_fold<NW>(k1) : 0, l1, g1);
        uint32_t mprev = 0, mcur = __ballot_sync(0xffffffffu, gate_resolve(g0, l0));
        uint32_t mnext = __ballot_sync(0xffffffffu, gate_resolve(g1, l1));
        Key<NW> kc = k0, kn = k1;
        bool rcc = rc0, rcn = rc1;
        uint64_t hc = g0.h0, hn = g1.h0;
        for (uint32_t it = 0; it < n_it; ++it) {
            // issue chunk it + 2
            Key<NW> kf{};
            bool rcf = false;
            const uint32_t qf = ((it + 2) << 5) + lane;
            const bool lf = qf < nk;
            if (lf) canonical_ws<NW, WS>(b.data, off + qf, k, kf, rcf);
            GateLoads gf;
            gate_issue(top, log2w, lf ? key_fold<NW>(kf) : 0, lf, gf);
            // emit chunk it
            const uint32_t q = (it << 5) + lane;
            bool emit = false;
            uint32_t info = 0, bucket = 0;
            if (q < nk) {
                const bool sq = (mcur >> lane) & 1u;
                const bool sl = q > 0 && (lane ? ((mcur >> (lane - 1)) & 1u) : (mprev >> 31));
                const bool sr = q + 1 < nk && (lane < 31 ? ((mcur >> (lane + 1)) & 1u) : (mnext & 1u));
                emit = sq && (sl || sr);
                if (emit) {
                    const uint64_t g = off + q;
                    if (sr) info |= 8u | (base_at(b.data, g + k) + (rcc ? 4u : 0u));
                    if (sl) info |= (8u | ((3u - base_at(b.data, g - 1)) + (rcc ? 0u : 4u))) << 4;
                    bucket = bucket_of_h(hc, bk.n_buckets);
                }
            }
            const uint32_t active = __ballot_sync(0xffffffffu, emit);
            if (emit) {
                const uint32_t pos = n_buf + __popc(active & ((1u << lane) - 1));
                rec_put<NW>(buf + pos * (NW + 1), kc, info, bk);
                bbuf[pos] = (uint8_t)bucket;
            }
            n_buf += __popc(active);
            if (n_buf > emit_buf(NW) - 32) {
                __syncwarp();
                emit_flush<NW>(bk, stripe, lane, buf, bbuf, n_buf, hist, gbase, rank, perm);
                n_buf = 0;
            }
            // resolve chunk it + 2 and rotate
            const uint32_t mfar = __ballot_sync(0xffffffffu, gate_resolve(gf, lf));
            mprev = mcur;
            mcur = mnext;
            mnext = mfar;
            kc = kn;
            rcc = rcn;
            hc = hn;
            kn = kf;
            rcn = rcf;
            hn = gf.h0;
        }
    }
    __syncwarp();
    if (n_buf) emit_flush<NW>(bk, stripe, lane, buf, bbuf, n_buf, hist, gbase, rank, perm);
}

// The same emit over a flattened window stream: a warp takes a run of EMIT_RUN
// consecutive reads and walks the concatenation of their windows 32 at a time, so a
// chunk may hold the end of one read and the start of the next and no lane idles at
// the end of each read (a 146-base read has 70 windows of 77 bases: three chunks of
// 32 per read, 27% of the lanes idle, when walked read by read).  Window q of a read
// has its left neighbour at the previous stream position iff q > 0 and its right
// neighbour at the next iff q + 1 < nk, so the ballot logic is unchanged.  Gate
// loads run two chunks ahead as in k_emit_ladder2.
constexpr uint32_t EMIT_RUN = 32;

struct StreamCursor {
    uint64_t r, r_end;  // current read, end of the run
    uint64_t off;       // first base of read r
    uint32_t q, nk;     // window within read r, windows of read r (0 if skipped)
};

__device__ __forceinline__ uint32_t stream_nk(const BankDev& b, uint64_t r, uint32_t k) {
    const uint32_t len = b.len[r];
    return len >= k + 1 && bank_keep(b, r) ? len - k + 1 : 0u;
}
// Moves the cursor `step` windows forward; r == r_end afterwards means past the run.
__device__ __forceinline__ void stream_advance(const BankDev& b, uint32_t k, StreamCursor& c, uint32_t step) {
    c.q += step;
    while (c.r < c.r_end && c.q >= c.nk) {
        c.q -= c.nk;
        if (++c.r < c.r_end) {
            c.nk = stream_nk(b, c.r, k);
            c.off = b.off[c.r];
        }
    }
}

template <int NW>
struct StreamWindow {
    Key<NW> key;
    uint64_t g;     // first base
    bool live, rc;
    bool has_l, has_r;  // neighbours inside the read
};
template <int NW, int WS>
__device__ __forceinline__ void stream_window(const BankDev& b, uint32_t k, const StreamCursor& c, StreamWindow<NW>& w) {
    w.live = c.r < c.r_end;
    w.rc = false;
    w.g = c.off + c.q;
    w.has_l = c.q > 0;
    w.has_r = c.q + 1 < c.nk;
    if (w.live) canonical_ws<NW, WS>(b.data, w.g, k, w.key, w.rc);
}

// WS = (64*NW - 2k) / 64 as in k_emit_ladder2; the record's bucket comes from the
// row-0 hash the gate computed for the window (GateLoads::h0).
template <int NW, int WS>
__global__ void __launch_bounds__(256, 3) k_emit_flat(BankDev b, uint32_t k, const uint32_t* __restrict__ lad, uint32_t log2w,
                                                      uint32_t t_solid, TableDev t, BucketDev bk) {
    extern __shared__ uint64_t emit_smem[];
    const uint32_t lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    uint64_t* buf = emit_smem + (uint64_t)wib * EMIT_WARP_WORDS(NW);
    uint8_t* bbuf = reinterpret_cast<uint8_t*>(buf + emit_buf(NW) * (NW + 1));
    uint16_t* rank = reinterpret_cast<uint16_t*>(bbuf + emit_buf(NW));
    uint32_t* hist = reinterpret_cast<uint32_t*>(rank + emit_buf(NW));
    unsigned long long* gbase = reinterpret_cast<unsigned long long*>(hist + EMIT_MAX_BUCKETS);
    uint16_t* perm = reinterpret_cast<uint16_t*>(gbase + EMIT_MAX_BUCKETS);
    const uint32_t* top = lad + (uint64_t)(t_solid - 1) * ((4ULL << log2w) >> 5);
    const uint64_t gw = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    const uint32_t stripe = (uint32_t)(gw % bk.stripes);
    uint32_t n_buf = 0;  // warp-uniform
    for (uint64_t r0 = b.r_begin + gw * EMIT_RUN; r0 < b.r_end; r0 += nwarps * EMIT_RUN) {
        StreamCursor cur;
        cur.r = r0;
        cur.r_end = r0 + EMIT_RUN < b.r_end ? r0 + EMIT_RUN : b.r_end;
        cur.nk = stream_nk(b, r0, k);
        cur.off = b.off[r0];
        cur.q = 0;
        stream_advance(b, k, cur, lane);
        // chunks 0 and 1 resolved up front
        StreamWindow<NW> wc, wn;
        stream_window<NW, WS>(b, k, cur, wc);
        stream_advance(b, k, cur, 32);
        stream_window<NW, WS>(b, k, cur, wn);
        stream_advance(b, k, cur, 32);
        GateLoads g0, g1;
        gate_issue(top, log2w, wc.live ? key_fold<NW>(wc.key) : 0, wc.live, g0);
        gate_issue(top, log2w, wn.live ? key_fold<NW>(wn.key) : 0, wn.live, g1);
        uint32_t mprev = 0, mcur = __ballot_sync(0xffffffffu, gate_resolve(g0, wc.live));
        uint32_t mnext = __ballot_sync(0xffffffffu, gate_resolve(g1, wn.live));
        uint64_t hc = g0.h0, hn = g1.h0;
        // the stream of a run is contiguous: once a chunk has no live lane, none has
        while (__any_sync(0xffffffffu, wc.live)) {
            StreamWindow<NW> wf;
            stream_window<NW, WS>(b, k, cur, wf);
            stream_advance(b, k, cur, 32);
            GateLoads gf;
            gate_issue(top, log2w, wf.live ? key_fold<NW>(wf.key) : 0, wf.live, gf);
            bool emit = false;
            uint32_t info = 0, bucket = 0;
            if (wc.live) {
                const bool sq = (mcur >> lane) & 1u;
                const bool sl = wc.has_l && (lane ? ((mcur >> (lane - 1)) & 1u) : (mprev >> 31));
                const bool sr = wc.has_r && (lane < 31 ? ((mcur >> (lane + 1)) & 1u) : (mnext & 1u));
                emit = sq && (sl || sr);
                if (emit) {
                    if (sr) info |= 8u | (base_at(b.data, wc.g + k) + (wc.rc ? 4u : 0u));
                    if (sl) info |= (8u | ((3u - base_at(b.data, wc.g - 1)) + (wc.rc ? 0u : 4u))) << 4;
                    bucket = bucket_of_h(hc, bk.n_buckets);
                }
            }
            const uint32_t active = __ballot_sync(0xffffffffu, emit);
            if (emit) {
                const uint32_t pos = n_buf + __popc(active & ((1u << lane) - 1));
                rec_put<NW, WS>(buf + pos * (NW + 1), wc.key, info, bk);
                bbuf[pos] = (uint8_t)bucket;
            }
            n_buf += __popc(active);
            if (n_buf > emit_buf(NW) - 32) {
                __syncwarp();
                emit_flush<NW>(bk, stripe, lane, buf, bbuf, n_buf, hist, gbase, rank, perm);
                n_buf = 0;
            }
            const uint32_t mfar = __ballot_sync(0xffffffffu, gate_resolve(gf, wf.live));
            mprev = mcur;
            mcur = mnext;
            mnext = mfar;
            wc = wn;
            wn = wf;
            hc = hn;
            hn = gf.h0;
        }
    }
    __syncwarp();
    if (n_buf) emit_flush<NW>(bk, stripe, lane, buf, bbuf, n_buf, hist, gbase, rank, perm);
}

// Upsert of one bucket's records: every thread resolves its record's key from its
// home slot and adds the pushes.  (Taking two records per thread and issuing both
// home-slot loads first measured 18% slower: register pressure cost more occupancy
// than the overlap gained.)
// Bucket upserts and record counts run on a 2D grid: blockIdx.y is the stripe, and the
// blocks of a stripe stride over its records (the stripes of a bucket hold about the
// same number).  A block reads its stripe's fill counter once; there is no prefix over
// the stripes and no search for a record's stripe.
__device__ __forceinline__ uint64_t stripe_records(const BucketDev& bk, uint32_t bucket, const uint64_t*& base, int rw) {
    const uint32_t s = blockIdx.y;
    const unsigned long long f = bk.fill[(uint64_t)bucket * bk.stripes + s];
    base = bk.recs + ((uint64_t)bucket * bk.stripes + s) * bk.stripe_cap * (uint64_t)rw;
    return f < bk.stripe_cap ? f : bk.stripe_cap;
}

// Keys that cannot become SolidKmerNodes can stay out of the table when the caller
// does not need the whole accumulator: edge counter e of a key grows by at most one
// per record of the key (a record pushes two different edges), so a key with fewer
// than min_trans_cov records has an empty mask (build.rs:306-314).  Before a bucket's
// upserts, k_count_records adds 1 per record to a counter chosen by the key's hash;
// every record of a key lies in the same bucket and hits the same counter, so the
// counter bounds the key's records from above, and the upsert skips the records whose
// bound is below min_trans_cov.  Exact when the bucket holds every record of the pass (one
// read chunk, no prior contigs, whose pushes weigh more than 1).
constexpr uint64_t FILTER_SALT = 0x3c6ef372fe94f82bULL;
__device__ __forceinline__ uint32_t filter_col(uint64_t fold, uint32_t log2m) {
    return (uint32_t)(smix(fold ^ FILTER_SALT) >> (64 - log2m));
}

// Number of counters at or above `min` (the filter's survivors of one bucket).
__global__ void __launch_bounds__(256) k_count_at_least(const uint32_t* __restrict__ cnt, uint64_t n, uint32_t min,
                                                        unsigned long long* out) {
    unsigned long long c = 0;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        c += __ldcg(cnt + i) >= min;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) c += __shfl_down_sync(0xffffffffu, c, off);
    if ((threadIdx.x & 31) == 0 && c) atomicAdd(out, c);
}

template <int NW>
__global__ void __launch_bounds__(256) k_count_records(BucketDev bk, uint32_t bucket, RecordFilter flt) {
    const uint64_t* base;
    const uint64_t n = stripe_records(bk, bucket, base, bk.rw);
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        Key<NW> key;
        rec_key<NW>(base + i * bk.rw, key, bk);
        atomicAdd(flt.cnt + filter_col(key_fold<NW>(key), flt.log2m), 1u);
    }
}

// Resolve a key's slot from its home slot and add the record's pushes (info byte).
template <int NW>
__device__ __forceinline__ void upsert_key(const Key<NW>& key, uint32_t info, uint64_t f, uint64_t home, uint32_t w_edge,
                                           uint32_t w_cov, const TableDev& t, uint32_t* status) {
    int64_t s;
    if constexpr (NW == 1) s = table_slot1(t, key.w[0], home, status);
    else if constexpr (NW == 2) s = table_slot2(t, key, home, status);
    else s = table_slotw<NW>(t, key, f, home, status);
    if (s < 0) return;
    uint32_t* c = t.cnt + (uint64_t)s * 8;
    const uint32_t nu = (info >> 3) & 1u, nv = (info >> 7) & 1u;
    if (nu) atomicAdd(&c[info & 7u], w_edge);
    if (nv) atomicAdd(&c[(info >> 4) & 7u], w_edge);
    if (t.cov) atomicAdd(&t.cov[s], w_cov * (nu + nv));
}

// One record's upsert: resolve the key's slot from its home slot and add its pushes.
template <int NW>
__device__ __forceinline__ void upsert_record(const uint64_t* rec, const BucketDev& bk, uint32_t w_edge, uint32_t w_cov,
                                              const TableDev& t, uint32_t* status, const RecordFilter& flt,
                                              unsigned long long& skipped) {
    Key<NW> key;
    const uint32_t info = rec_get<NW>(rec, key, bk);
    const uint64_t f = key_fold<NW>(key);
    const uint64_t home = home_slot(f, t.cap);
    // The filter counter is read before any probe: records the filter drops (about 40% at
    // k = 77, keys seen once or twice) then touch no table slot.  (Loading the home slot
    // together with the counter made the filtered upserts slower: k = 55 7.38 -> 8.60 ms,
    // k = 77 10.8 -> 12.5 ms per 100x pass.)
    if (flt.cnt) {
        if (__ldcg(flt.cnt + filter_col(f, flt.log2m)) < flt.min_records) {
            skipped += ((info >> 3) & 1u) + ((info >> 7) & 1u);
            return;
        }
    }
    upsert_key<NW>(key, info, f, home, w_edge, w_cov, t, status);
}

template <int NW>
__global__ void __launch_bounds__(256, 8) k_upsert(BucketDev bk, uint32_t bucket, uint32_t w_edge, uint32_t w_cov, TableDev t,
                                                uint32_t* status, RecordFilter flt) {
    const uint64_t* base;
    const uint64_t n = stripe_records(bk, bucket, base, bk.rw);
    unsigned long long skipped = 0;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        upsert_record<NW>(base + i * bk.rw, bk, w_edge, w_cov, t, status, flt, skipped);
    if (flt.cnt) {
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) skipped += __shfl_down_sync(0xffffffffu, skipped, off);
        if ((threadIdx.x & 31) == 0 && skipped) atomicAdd(flt.skipped, skipped);
    }
}

// The filtered upsert with the filter's survivors queued per warp.  A warp reads 32
// records at a time (one per lane, coalesced) and tests their filter counters; the
// indices of the records that pass go to the warp's queue in shared memory, and the
// warp probes the table 32 queued records at a time, re-reading each record (an L1
// hit), so every lane of the probe phase has a record.  With the test inline, the
// lanes whose record the filter drops (about 40% at k = 77) wait for the others'
// probes: 12 of 32 lanes were active per instruction.
constexpr int UPQ_WARPS = 8;
template <int NW, int MINB>
__global__ void __launch_bounds__(256, MINB) k_upsert_q(BucketDev bk, uint32_t bucket, uint32_t w_edge, uint32_t w_cov, TableDev t,
                                                  uint32_t* status, RecordFilter flt) {
    __shared__ uint32_t s_q[UPQ_WARPS][64];
    const uint64_t* base;
    const uint64_t n = stripe_records(bk, bucket, base, bk.rw);
    const uint32_t lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    uint32_t* q = s_q[wib];
    uint32_t qn = 0;  // queued records (warp-uniform), below 32 between batches
    unsigned long long skipped = 0;
    const uint64_t gwarp = (((uint64_t)blockIdx.x * blockDim.x) >> 5) + wib;
    const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    for (uint64_t r0 = gwarp * 32; r0 < n; r0 += nwarps * 32) {
        const uint64_t i = r0 + lane;
        bool keep = false;
        if (i < n) {
            Key<NW> key;
            const uint32_t info = rec_get<NW, true>(base + i * bk.rw, key, bk);
            keep = __ldcg(flt.cnt + filter_col(key_fold<NW>(key), flt.log2m)) >= flt.min_records;
            if (!keep) skipped += ((info >> 3) & 1u) + ((info >> 7) & 1u);
        }
        const uint32_t m = __ballot_sync(0xffffffffu, keep);
        if (keep) q[qn + __popc(m & ((1u << lane) - 1u))] = (uint32_t)i;
        qn += __popc(m);
        __syncwarp();
        if (qn >= 32) {
            qn -= 32;
            const uint64_t j = q[qn + lane];
            __syncwarp();
            Key<NW> key;
            const uint32_t info = rec_get<NW, true>(base + j * bk.rw, key, bk);
            const uint64_t f = key_fold<NW>(key);
            upsert_key<NW>(key, info, f, home_slot(f, t.cap), w_edge, w_cov, t, status);
        }
    }
    if (lane < qn) {
        const uint64_t j = q[lane];
        Key<NW> key;
        const uint32_t info = rec_get<NW, true>(base + j * bk.rw, key, bk);
        const uint64_t f = key_fold<NW>(key);
        upsert_key<NW>(key, info, f, home_slot(f, t.cap), w_edge, w_cov, t, status);
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) skipped += __shfl_down_sync(0xffffffffu, skipped, off);
    if (lane == 0 && skipped) atomicAdd(flt.skipped, skipped);
}

// Every bucket of a pass in one persistent launch: blocks take work items (bucket,
// stripe, run of UPSERT_ITEM records) from a counter in bucket order, so at any time
// the blocks work on one or two buckets' table ranges, without a launch and its tail
// per bucket.  Measured per step at 100x: items of 2048 records 31.9 ms, 4096 32.3,
// 16384 37.0 (the blocks then spread over more buckets at once); items taken per warp
// instead, which removes the block barriers, 35.9 (every warp waits on the shared
// counter's atomic).  No record filter (its counts must be complete before a bucket's
// upserts start).
constexpr uint32_t UPSERT_ITEM = 2048;
template <int NW>
__global__ void __launch_bounds__(256, NW == 4 ? 6 : 8) k_upsert_all(BucketDev bk, uint32_t w_edge, uint32_t w_cov, TableDev t,
                                                    uint32_t* status, unsigned long long* work) {
    __shared__ unsigned long long s_item;
    const uint64_t per_stripe = (bk.stripe_cap + UPSERT_ITEM - 1) / UPSERT_ITEM;
    const uint64_t n_items = (uint64_t)bk.n_buckets * bk.stripes * per_stripe;
    const RecordFilter none{};
    unsigned long long skipped = 0;
    for (;;) {
        if (threadIdx.x == 0) s_item = atomicAdd(work, 1ULL);
        __syncthreads();
        const uint64_t item = s_item;
        __syncthreads();
        if (item >= n_items) break;
        const uint64_t bs = item / per_stripe;  // bucket * stripes + stripe
        const uint64_t first = (item - bs * per_stripe) * UPSERT_ITEM;
        const unsigned long long f = bk.fill[bs];
        const uint64_t n = f < bk.stripe_cap ? f : bk.stripe_cap;
        if (first >= n) continue;
        const uint64_t last = first + UPSERT_ITEM < n ? first + UPSERT_ITEM : n;
        const uint64_t* base = bk.recs + bs * bk.stripe_cap * bk.rw;
        for (uint64_t i = first + threadIdx.x; i < last; i += blockDim.x)
            upsert_record<NW>(base + i * bk.rw, bk, w_edge, w_cov, t, status, none, skipped);
    }
}

// The persistent upsert with every lane's probe sequence advanced one slot per step:
// a lane whose record is placed takes its next record at once instead of waiting at
// the loop's reconvergence for the lanes with longer probe runs, so each step of a
// warp issues one table load per busy lane.  A warp works through its own records of
// the block's work item (lane j: records first + 32 w + j, + blockDim, ...).
// 64- and 128-bit keys (slots claimed by one CAS, no publication wait).
template <int NW>
__device__ __forceinline__ int probe_step(const TableDev& t, const Key<NW>& key, uint64_t s) {
    // 1: the key's slot is s; 0: go on with the next slot
    if constexpr (NW == 1) {
        const uint64_t cur = __ldcg(&t.keys[s]);
        if (cur == key.w[0]) return 1;
        if (cur == KEY_EMPTY) {
            const uint64_t old = atomicCAS((unsigned long long*)&t.keys[s], KEY_EMPTY, key.w[0]);
            if (old == KEY_EMPTY || old == key.w[0]) return 1;
        }
        return 0;
    } else {
        uint64_t* a = t.keys + s * 2;
        const ulonglong2 c = __ldcg(reinterpret_cast<const ulonglong2*>(a));
        const bool other = (c.x != KEY_EMPTY && c.x != key.w[0]) || (c.y != KEY_EMPTY && c.y != key.w[1]);
        if (other) return 0;
        if (c.x == key.w[0] && c.y == key.w[1] && key.w[1] != KEY_EMPTY) return 1;
        uint64_t o0, o1;
        cas128(a, KEY_EMPTY, KEY_EMPTY, key.w[0], key.w[1], o0, o1);
        return ((o0 == KEY_EMPTY && o1 == KEY_EMPTY) || (o0 == key.w[0] && o1 == key.w[1])) ? 1 : 0;
    }
}

template <int NW>
__global__ void __launch_bounds__(256, 8) k_upsert_all_step(BucketDev bk, uint32_t w_edge, uint32_t w_cov, TableDev t,
                                                         uint32_t* status, unsigned long long* work) {
    static_assert(NW <= 2, "one-CAS slots only");
    __shared__ unsigned long long s_item;
    const uint64_t per_stripe = (bk.stripe_cap + UPSERT_ITEM - 1) / UPSERT_ITEM;
    const uint64_t n_items = (uint64_t)bk.n_buckets * bk.stripes * per_stripe;
    const uint32_t lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    for (;;) {
        if (threadIdx.x == 0) s_item = atomicAdd(work, 1ULL);
        __syncthreads();
        const uint64_t item = s_item;
        __syncthreads();
        if (item >= n_items) break;
        const uint64_t bs = item / per_stripe;  // bucket * stripes + stripe
        const uint64_t first = (item - bs * per_stripe) * UPSERT_ITEM;
        const unsigned long long fl = bk.fill[bs];
        const uint64_t n = fl < bk.stripe_cap ? fl : bk.stripe_cap;
        if (first >= n) continue;
        const uint64_t last = first + UPSERT_ITEM < n ? first + UPSERT_ITEM : n;
        const uint64_t* base = bk.recs + bs * bk.stripe_cap * bk.rw;
        uint64_t i = first + 32 * wib + lane;
        bool have = false;
        Key<NW> key;
        uint32_t info = 0, probe = 0;
        uint64_t s = 0;
        for (;;) {
            if (!have && i < last) {
                info = rec_get<NW>(base + i * bk.rw, key, bk);
                s = home_slot(key_fold<NW>(key), t.cap);
                probe = 0;
                have = true;
                i += blockDim.x;
            }
            if (!__any_sync(0xffffffffu, have)) break;
            if (!have) continue;
            if (probe_step<NW>(t, key, s)) {
                uint32_t* c = t.cnt + s * 8;
                const uint32_t nu = (info >> 3) & 1u, nv = (info >> 7) & 1u;
                if (nu) atomicAdd(&c[info & 7u], w_edge);
                if (nv) atomicAdd(&c[(info >> 4) & 7u], w_edge);
                if (t.cov) atomicAdd(&t.cov[s], w_cov * (nu + nv));
                have = false;
            } else {
                s = s + 1 == t.cap ? 0 : s + 1;
                if (++probe >= t.max_probe) {
                    atomicOr(status, ST_TABLE_FULL);
                    have = false;
                }
            }
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

// Order-free digest term of one accumulated key (KmerAcc, build.rs:145-149): the key's
// words (big-endian order) folded through splitmix64, then cov and the 8 capped edge
// counts packed as u16 fields.  Summed over keys mod 2^64, it compares a whole
// accumulator without exporting it (the oracle computes the same sum).
template <int NW>
__device__ __forceinline__ uint64_t acc_row_digest(const Key<NW>& key, uint16_t cov, const uint32_t* cnt) {
    uint64_t kd = 0;
#pragma unroll
    for (int i = 0; i < NW; ++i) kd = smix(kd ^ key.w[i]);
    uint64_t e[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) e[i] = cnt[i] > 0xFFFFu ? 0xFFFFu : cnt[i];
    const uint64_t v0 = (uint64_t)cov | (e[0] << 16) | (e[1] << 32) | (e[2] << 48);
    const uint64_t v1 = e[3] | (e[4] << 16) | (e[5] << 32) | (e[6] << 48);
    return smix(kd ^ smix(v0 ^ smix(v1 ^ smix(e[7]))));
}

template <int NW>
__global__ void __launch_bounds__(256) k_convert(TableDev t, uint32_t min_trans_cov, ConvOut o) {
    __shared__ uint32_t s_warp[32];
    __shared__ unsigned long long s_base[2];
    const uint64_t cap = t.cap;
    const uint64_t tile = (uint64_t)blockDim.x * CONV_SLOTS;
    unsigned long long n_keys = 0, digest = 0, raw_total = 0, acc_digest = 0;
    for (uint64_t base = (uint64_t)blockIdx.x * tile; base < cap; base += (uint64_t)gridDim.x * tile) {
        const uint64_t s0 = base + (uint64_t)threadIdx.x * CONV_SLOTS;
        uint32_t occ_bits = 0, keep_bits = 0;
#pragma unroll
        for (int j = 0; j < CONV_SLOTS; ++j) {
            const uint64_t s = s0 + j;
            if (s >= cap) break;
            const bool occ = NW <= 2 ? (t.keys[s * NW] != KEY_EMPTY) : (t.tags[s * t.tag_stride] != 0);
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
            if (NW == 4 && t.tag_stride == NW) key.w[0] = 0;  // word 0 holds the tag
            if (o.acc_digest) acc_digest += acc_row_digest<NW>(key, covs[j], t.cnt + s * 8);
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
        acc_digest += __shfl_down_sync(0xffffffffu, acc_digest, off);
    }
    if ((threadIdx.x & 31) == 0) {
        if (acc_digest) atomicAdd(&o.counts[5], acc_digest);
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
// Persistent grid: resident blocks per SM for this kernel and block size, times SMs.
template <class K>
static int grid_for(K kernel, const Launch& L) {
    if (L.grid > 0) return L.grid;
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, L.block, 0) != cudaSuccess || per_sm < 1) per_sm = 1;
    return per_sm * (L.sms > 0 ? L.sms : 1);
}

template <int NW>
static cudaError_t pass1_nw(const Launch& L, const BankDev& b, uint32_t k, uint32_t* cnt, uint32_t log2w, uint32_t r0,
                            uint32_t r1, uint64_t c0, uint64_t c1, uint32_t mult, uint32_t* hll12) {
    k_pass1_sweep<NW><<<grid_for(k_pass1_sweep<NW>, L), L.block, 0, L.stream>>>(b, k, cnt, log2w, r0, r1, c0, c1, mult, hll12);
    return cudaGetLastError();
}
cudaError_t launch_pass1_sweep(int nw, const Launch& L, const BankDev& b, uint32_t k, uint32_t* cnt, uint32_t log2w,
                               uint32_t r0, uint32_t r1, uint64_t c0, uint64_t c1, uint32_t mult, uint32_t* hll12) {
    if (nw == 1) return pass1_nw<1>(L, b, k, cnt, log2w, r0, r1, c0, c1, mult, hll12);
    if (nw == 2) return pass1_nw<2>(L, b, k, cnt, log2w, r0, r1, c0, c1, mult, hll12);
    return pass1_nw<4>(L, b, k, cnt, log2w, r0, r1, c0, c1, mult, hll12);
}

template <int NW>
static cudaError_t solid_nw(const Launch& L, const BankDev& b, uint32_t k, const uint32_t* cnt, uint32_t log2w, uint32_t r0,
                            uint32_t r1, uint64_t c0, uint64_t c1, uint32_t t_solid, uint32_t cap, uint32_t* bm) {
    k_solid_sweep<NW><<<grid_for(k_solid_sweep<NW>, L), L.block, 0, L.stream>>>(b, k, cnt, log2w, r0, r1, c0, c1, t_solid, cap, bm);
    return cudaGetLastError();
}
cudaError_t launch_solid_sweep(int nw, const Launch& L, const BankDev& b, uint32_t k, const uint32_t* cnt, uint32_t log2w,
                               uint32_t r0, uint32_t r1, uint64_t c0, uint64_t c1, uint32_t t_solid, uint32_t cap, uint32_t* bm) {
    if (nw == 1) return solid_nw<1>(L, b, k, cnt, log2w, r0, r1, c0, c1, t_solid, cap, bm);
    if (nw == 2) return solid_nw<2>(L, b, k, cnt, log2w, r0, r1, c0, c1, t_solid, cap, bm);
    return solid_nw<4>(L, b, k, cnt, log2w, r0, r1, c0, c1, t_solid, cap, bm);
}

template <int NW>
static cudaError_t pass2_nw(const Launch& L, const BankDev& b, uint32_t k, const uint32_t* bm, int gate, uint64_t s0,
                            uint64_t s1, uint32_t we, uint32_t wc, const TableDev& t, uint32_t* status) {
    k_pass2_sweep<NW><<<grid_for(k_pass2_sweep<NW>, L), L.block, 0, L.stream>>>(b, k, bm, gate, s0, s1, we, wc, t, status);
    return cudaGetLastError();
}
cudaError_t launch_pass2_sweep(int nw, const Launch& L, const BankDev& b, uint32_t k, const uint32_t* bm, int gate,
                               uint64_t s0, uint64_t s1, uint32_t w_edge, uint32_t w_cov, const TableDev& t,
                               uint32_t* status) {
    if (nw == 1) return pass2_nw<1>(L, b, k, bm, gate, s0, s1, w_edge, w_cov, t, status);
    if (nw == 2) return pass2_nw<2>(L, b, k, bm, gate, s0, s1, w_edge, w_cov, t, status);
    return pass2_nw<4>(L, b, k, bm, gate, s0, s1, w_edge, w_cov, t, status);
}

template <int NW>
static cudaError_t emit_nw(const Launch& L, const BankDev& b, uint32_t k, const uint32_t* bm, int gate, const TableDev& t,
                           const BucketDev& bk) {
    const size_t smem = (size_t)(L.block / 32) * EMIT_WARP_WORDS(NW) * 8;
    if (smem > 48 * 1024) cudaFuncSetAttribute(k_emit<NW>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    int grid = L.grid;
    if (grid <= 0) {
        int per_sm = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_emit<NW>, L.block, smem) != cudaSuccess || per_sm < 1)
            per_sm = 1;
        grid = per_sm * (L.sms > 0 ? L.sms : 1);
    }
    k_emit<NW><<<grid, L.block, smem, L.stream>>>(b, k, bm, gate, t, bk);
    return cudaGetLastError();
}
template <class Kern>
static cudaError_t emit_launch(Kern kern, const Launch& L, const BankDev& b, uint32_t k, const uint32_t* lad, uint32_t log2w,
                               uint32_t ts, const TableDev& t, const BucketDev& bk, size_t smem) {
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
    }
    int grid = L.grid;
    if (grid <= 0) {
        int per_sm = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, L.block, smem) != cudaSuccess || per_sm < 1) per_sm = 1;
        grid = per_sm * (L.sms > 0 ? L.sms : 1);
    }
    kern<<<grid, L.block, smem, L.stream>>>(b, k, lad, log2w, ts, t, bk);
    return cudaGetLastError();
}
template <int NW>
static cudaError_t emitl_nw(const Launch& L, const BankDev& b, uint32_t k, const uint32_t* lad, uint32_t log2w, uint32_t ts,
                            const TableDev& t, const BucketDev& bk, int lookahead) {
    const size_t smem = (size_t)(L.block / 32) * EMIT_WARP_WORDS(NW) * 8;
    const uint32_t ws = (64u * NW - 2u * k) >> 6;
    if (lookahead == 4 || lookahead == 5) {  // one lane per read, rolled (fbk_k_roll.cu); 5: two blocks per SM
        Launch L2 = L;
        L2.block = 256;
        return launch_emit_roll(NW, L2, b, k, lad, log2w, ts, t, bk, lookahead == 5);
    }
    if (lookahead == 3) {
        if constexpr (NW == 1) {
            return emit_launch(k_emit_flat<1, 0>, L, b, k, lad, log2w, ts, t, bk, smem);
        } else if constexpr (NW == 2) {
            if (ws == 0) return emit_launch(k_emit_flat<2, 0>, L, b, k, lad, log2w, ts, t, bk, smem);
            return emit_launch(k_emit_flat<2, 1>, L, b, k, lad, log2w, ts, t, bk, smem);
        } else {
            if (ws == 0) return emit_launch(k_emit_flat<4, 0>, L, b, k, lad, log2w, ts, t, bk, smem);
            if (ws == 1) return emit_launch(k_emit_flat<4, 1>, L, b, k, lad, log2w, ts, t, bk, smem);
            if (ws == 2) return emit_launch(k_emit_flat<4, 2>, L, b, k, lad, log2w, ts, t, bk, smem);
            return emit_launch(k_emit_flat<4, 3>, L, b, k, lad, log2w, ts, t, bk, smem);
        }
    }
    if (lookahead == 2) {
        if constexpr (NW == 1) {
            return emit_launch(k_emit_ladder2<1, 0>, L, b, k, lad, log2w, ts, t, bk, smem);
        } else if constexpr (NW == 2) {
            if (ws == 0) return emit_launch(k_emit_ladder2<2, 0>, L, b, k, lad, log2w, ts, t, bk, smem);
            return emit_launch(k_emit_ladder2<2, 1>, L, b, k, lad, log2w, ts, t, bk, smem);
        } else {
            if (ws == 0) return emit_launch(k_emit_ladder2<4, 0>, L, b, k, lad, log2w, ts, t, bk, smem);
            if (ws == 1) return emit_launch(k_emit_ladder2<4, 1>, L, b, k, lad, log2w, ts, t, bk, smem);
            if (ws == 2) return emit_launch(k_emit_ladder2<4, 2>, L, b, k, lad, log2w, ts, t, bk, smem);
            return emit_launch(k_emit_ladder2<4, 3>, L, b, k, lad, log2w, ts, t, bk, smem);
        }
    }
    return emit_launch(k_emit_ladder<NW>, L, b, k, lad, log2w, ts, t, bk, smem);
}
cudaError_t launch_emit_ladder(int nw, const Launch& L, const BankDev& b, uint32_t k, const uint32_t* lad, uint32_t log2w,
                               uint32_t t_solid, const TableDev& t, const BucketDev& bk, int lookahead) {
    if (t_solid < 1 || t_solid > LADDER_MAX_LEVELS || log2w > 29) return cudaErrorInvalidValue;
    if (nw == 1) return emitl_nw<1>(L, b, k, lad, log2w, t_solid, t, bk, lookahead);
    if (nw == 2) return emitl_nw<2>(L, b, k, lad, log2w, t_solid, t, bk, lookahead);
    return emitl_nw<4>(L, b, k, lad, log2w, t_solid, t, bk, lookahead);
}

cudaError_t launch_emit(int nw, const Launch& L, const BankDev& b, uint32_t k, const uint32_t* bm, int gate, const TableDev& t,
                        const BucketDev& bk) {
    if (nw == 1) return emit_nw<1>(L, b, k, bm, gate, t, bk);
    if (nw == 2) return emit_nw<2>(L, b, k, bm, gate, t, bk);
    return emit_nw<4>(L, b, k, bm, gate, t, bk);
}

// blocks per stripe: the occupancy-sized grid spread over the stripes
static dim3 stripe_grid(int blocks, uint32_t stripes) {
    const uint32_t s = stripes ? stripes : 1;
    return dim3((unsigned)std::max<int>(1, (blocks + (int)s - 1) / (int)s), s);
}
template <int NW>
static cudaError_t upsert_nw(const Launch& L, const BucketDev& bk, uint32_t bucket, uint32_t we, uint32_t wc, const TableDev& t,
                             uint32_t* status, const RecordFilter& flt, int queued) {
    if (queued == 1)
        k_upsert_q<NW, 8><<<stripe_grid(grid_for(k_upsert_q<NW, 8>, L), bk.stripes), L.block, 0, L.stream>>>(bk, bucket, we, wc, t,
                                                                                                             status, flt);
    else if (queued == 2)
        k_upsert_q<NW, 6><<<stripe_grid(grid_for(k_upsert_q<NW, 6>, L), bk.stripes), L.block, 0, L.stream>>>(bk, bucket, we, wc, t,
                                                                                                             status, flt);
    else
        k_upsert<NW><<<stripe_grid(grid_for(k_upsert<NW>, L), bk.stripes), L.block, 0, L.stream>>>(bk, bucket, we, wc, t, status, flt);
    return cudaGetLastError();
}
cudaError_t launch_upsert(int nw, const Launch& L, const BucketDev& bk, uint32_t bucket, uint32_t w_edge, uint32_t w_cov,
                          const TableDev& t, uint32_t* status, const RecordFilter& flt, int queue) {
    if (flt.cnt && (flt.log2m < 8 || flt.log2m > 30)) return cudaErrorInvalidValue;
    // the queue holds 32-bit record indices of at most UPQ_WARPS warps
    const int queued = flt.cnt && L.block % 32 == 0 && L.block <= 32 * UPQ_WARPS && bk.stripe_cap <= 0xFFFFFFFFull ? queue : 0;
    if (nw == 1) return upsert_nw<1>(L, bk, bucket, w_edge, w_cov, t, status, flt, queued);
    if (nw == 2) return upsert_nw<2>(L, bk, bucket, w_edge, w_cov, t, status, flt, queued);
    return upsert_nw<4>(L, bk, bucket, w_edge, w_cov, t, status, flt, queued);
}
template <int NW>
static cudaError_t upsert_all_nw(const Launch& L, const BucketDev& bk, uint32_t we, uint32_t wc, const TableDev& t,
                                 uint32_t* status, unsigned long long* work, bool stepped) {
    if constexpr (NW <= 2) {
        if (stepped) {
            k_upsert_all_step<NW><<<grid_for(k_upsert_all_step<NW>, L), L.block, 0, L.stream>>>(bk, we, wc, t, status, work);
            return cudaGetLastError();
        }
    }
    k_upsert_all<NW><<<grid_for(k_upsert_all<NW>, L), L.block, 0, L.stream>>>(bk, we, wc, t, status, work);
    return cudaGetLastError();
}
cudaError_t launch_upsert_all(int nw, const Launch& L, const BucketDev& bk, uint32_t w_edge, uint32_t w_cov, const TableDev& t,
                              uint32_t* status, unsigned long long* work, int form) {
    if (!work) return cudaErrorInvalidValue;
    // the stepped form gives each warp 32-record runs of a work item
    const bool stepped = form == 2 && L.block % 32 == 0;
    if (nw == 1) return upsert_all_nw<1>(L, bk, w_edge, w_cov, t, status, work, stepped);
    if (nw == 2) return upsert_all_nw<2>(L, bk, w_edge, w_cov, t, status, work, stepped);
    return upsert_all_nw<4>(L, bk, w_edge, w_cov, t, status, work, false);
}
template <int NW>
static cudaError_t count_nw(const Launch& L, const BucketDev& bk, uint32_t bucket, const RecordFilter& flt) {
    k_count_records<NW><<<stripe_grid(grid_for(k_count_records<NW>, L), bk.stripes), L.block, 0, L.stream>>>(bk, bucket, flt);
    return cudaGetLastError();
}
cudaError_t launch_count_at_least(const Launch& L, const uint32_t* cnt, uint64_t n, uint32_t min, unsigned long long* out) {
    k_count_at_least<<<L.grid, L.block, 0, L.stream>>>(cnt, n, min, out);
    return cudaGetLastError();
}
cudaError_t launch_count_records(int nw, const Launch& L, const BucketDev& bk, uint32_t bucket, const RecordFilter& flt) {
    if (!flt.cnt || flt.log2m < 8 || flt.log2m > 30) return cudaErrorInvalidValue;
    if (nw == 1) return count_nw<1>(L, bk, bucket, flt);
    if (nw == 2) return count_nw<2>(L, bk, bucket, flt);
    return count_nw<4>(L, bk, bucket, flt);
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
    const uint64_t cap = t.cap;
    if (nw <= 2) {
        k_table_init<<<L.grid, L.block, 0, L.stream>>>(t.keys, cap * nw, KEY_EMPTY);
        return cudaGetLastError();
    }
    // tags: their own array, or word 0 of every key (the other words are written
    // when the slot is claimed)
    return cudaMemsetAsync(t.tags, 0, cap * sizeof(uint64_t) * t.tag_stride, L.stream);
}

}  // namespace fbk
