// fbk_k_roll.cu — pass 1 (threshold-ladder gate) and the pass-2 record emit with
// one lane per read and the k-mer rolled base by base (src/graph/build.rs:93-116 and
// :243-289, rolled like RollingKmer::roll_next, kmer.rs:104-112, 181-189, 307-329).
//
// A warp takes a run of 32 consecutive reads; lane j walks read j of the run window by
// window.  The run's packed words are first staged in shared memory with 128-bit
// loads (one coalesced copy per run), and every lane then reads its bases from there:
// the first window of its read is cut from the packed words (its forward and reverse
// complement integers), every later one is rolled from the previous by one base —
//   fwd' = ((fwd << 2) | c) & mask(2k),   rc' = (rc >> 2) | ((3 - c) << (2k - 2))
// — a few word operations instead of re-extracting and bit-reversing k bases.  Reads of
// a run have about the same length (the bank keeps merged reads and each mate arena
// apart), so the lanes stay busy until the run's longest read ends.  A run whose packed
// span does not fit the staging buffer reads its bases from global memory instead.
//
// The results are those of the per-window kernels (fbk_k_ladder.cu, fbk_k_pass.cu):
// the same canonical keys, the same ladder updates, the same records.
#include "fbk_device.cuh"
#include "fbk_kernels.cuh"
#include "fbk_table.cuh"

namespace fbk {

constexpr uint32_t ROLL_RUN = 32;           // reads per warp run (one per lane)
constexpr uint32_t ROLL_STAGE_WORDS = 320;  // staged packed words per warp in the emit (2.5 KB)
constexpr uint32_t P1_STAGE_WORDS = 160;    // in pass 1 (1.25 KB: six blocks of 256 fit an SM);
                                            // a run of 32 mate reads of ~146 bases spans ~150

// The run's packed words in shared memory: words [lo, lo + n) of the bank.
struct RunStage {
    const uint64_t* s;
    uint64_t lo;
    uint32_t n;
};

// Loads the bank words of reads [r0, r0 + nr) into the warp's staging buffer with
// 16-byte loads (an aligned pair of words per lane per step).  Every lane passes its
// read's first base and length (len 0 for lanes without a read).  NK + 1 words past the
// last base are included (a window cut from the packed words reads that far).  Returns
// a stage with n = 0 when the span does not fit: the caller then reads global memory.
__device__ __forceinline__ RunStage stage_run(const uint64_t* __restrict__ d, uint64_t* s, uint32_t cap_words, uint32_t lane,
                                              uint64_t my_off, uint32_t my_len, uint32_t nk_words) {
    const bool has = my_len > 0;
    // first and last word of the run: reads are stored in increasing order
    const unsigned long long lo_c = has ? (my_off >> 5) : ~0ULL;
    const unsigned long long hi_c = has ? ((my_off + my_len - 1) >> 5) : 0ULL;
    unsigned long long lo = lo_c, hi = hi_c;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long a = __shfl_xor_sync(0xffffffffu, lo, o), b = __shfl_xor_sync(0xffffffffu, hi, o);
        lo = a < lo ? a : lo;
        hi = b > hi ? b : hi;
    }
    RunStage st{s, 0, 0};
    if (lo == ~0ULL) return st;  // no read with bases
    const uint64_t lo2 = lo & ~1ULL;  // 16-byte aligned start
    const uint64_t end = hi + 1 + nk_words + 1;
    const uint64_t n = (end - lo2 + 1) & ~1ULL;
    if (n > cap_words) return st;
    const ulonglong2* src = reinterpret_cast<const ulonglong2*>(d + lo2);
    ulonglong2* dst = reinterpret_cast<ulonglong2*>(s);
    for (uint32_t i = lane; i < n / 2; i += 32) dst[i] = __ldg(src + i);
    __syncwarp();
    st.lo = lo2;
    st.n = (uint32_t)n;
    return st;
}

__device__ __forceinline__ uint64_t run_word(const RunStage& st, const uint64_t* __restrict__ d, uint64_t wi) {
    const uint64_t i = wi - st.lo;
    return i < st.n ? st.s[i] : __ldg(d + wi);
}

// Forward and reverse-complement integers (NK significant words, big-endian) of the
// window of k bases at base g, cut from the packed words (the same arithmetic as
// canonical_ws, keeping both strands).
template <int NW, int WS>
__device__ __forceinline__ void window_strands(const RunStage& st, const uint64_t* __restrict__ d, uint64_t g, uint32_t k,
                                               uint64_t (&F)[NW - WS], uint64_t (&R)[NW - WS]) {
    constexpr int NK = NW - WS;
    const uint64_t wi = g >> 5;
    const uint32_t sh = (uint32_t)(g & 31) << 1;
    uint64_t D[NK + 1], W[NK], Rv[NK];
#pragma unroll
    for (int i = 0; i <= NK; ++i) D[i] = run_word(st, d, wi + i);
#pragma unroll
    for (int i = 0; i < NK; ++i) {
        W[i] = (D[i] >> sh) | ((D[i + 1] << (63 - sh)) << 1);
        Rv[i] = rev2(W[i]);
    }
    const uint32_t bs = (64u * NW - 2u * k) & 63;
    // fwd word j (significant index) = big-endian word WS + j of the full key
#pragma unroll
    for (int j = 0; j < NK; ++j) {
        const uint64_t hi = Rv[j];
        const uint64_t lo = j >= 1 ? Rv[j >= 1 ? j - 1 : 0] : 0ULL;
        F[j] = (hi >> bs) | (bs ? (lo << (64 - bs)) : 0ULL);
    }
    // rc: ~W masked to 2k bits; LSB-first word i is significant word NK - 1 - i
#pragma unroll
    for (int i = 0; i < NK; ++i) R[NK - 1 - i] = (~W[i]) & field_mask(k, i);
}

// Rolls both strands by one base c entering at the right end.  topb = 2k - 2 - 64 (NK - 1)
// is the bit of the first base in the most significant word; tmask masks that word.
template <int NK>
__device__ __forceinline__ void roll_strands(uint64_t (&F)[NK], uint64_t (&R)[NK], uint32_t c, uint32_t topb, uint64_t tmask) {
#pragma unroll
    for (int i = 0; i < NK - 1; ++i) F[i] = (F[i] << 2) | (F[i + 1] >> 62);
    F[NK - 1] = (F[NK - 1] << 2) | c;
    F[0] &= tmask;
#pragma unroll
    for (int i = NK - 1; i > 0; --i) R[i] = (R[i] >> 2) | (R[i - 1] << 62);
    R[0] = (R[0] >> 2) | ((uint64_t)(3u - c) << topb);
}

// Canonical key (NW words, the leading WS zero) and strand of the rolled window:
// rc is taken iff rc < fwd (build.rs:102,258).
template <int NW, int WS>
__device__ __forceinline__ void strands_canonical(const uint64_t (&F)[NW - WS], const uint64_t (&R)[NW - WS], Key<NW>& can,
                                                  bool& is_rc) {
    constexpr int NK = NW - WS;
    bool lt = false, eq = true;
#pragma unroll
    for (int i = 0; i < NK; ++i) {
        lt = lt || (eq && R[i] < F[i]);
        eq = eq && R[i] == F[i];
    }
    is_rc = lt;
#pragma unroll
    for (int i = 0; i < NW; ++i) can.w[i] = i < WS ? 0ULL : (lt ? R[i >= WS ? i - WS : 0] : F[i >= WS ? i - WS : 0]);
}

// Lane state for one read: the packed word holding the next base to enter, and where.
struct BaseCursor {
    uint64_t word;
    uint64_t wi;  // index of `word`
    uint32_t sh;  // bit of the next base in `word`
};
__device__ __forceinline__ void cursor_at(BaseCursor& c, const RunStage& st, const uint64_t* __restrict__ d, uint64_t g) {
    c.wi = g >> 5;
    c.sh = (uint32_t)(g & 31) << 1;
    c.word = run_word(st, d, c.wi);
}
__device__ __forceinline__ uint32_t cursor_next(BaseCursor& c, const RunStage& st, const uint64_t* __restrict__ d) {
    const uint32_t b = (uint32_t)(c.word >> c.sh) & 3u;
    c.sh += 2;
    if (c.sh == 64) {
        c.sh = 0;
        c.word = run_word(st, d, ++c.wi);
    }
    return b;
}

// ---------------------------------------------------------------------------
// Pass 1 with the threshold-ladder gate (fbk_k_ladder.cu), rolled.
// ---------------------------------------------------------------------------
// P windows per lane per step (1 or 2): with P = 2 a lane rolls two consecutive windows
// and issues their eight gate loads together before climbing both (two increments of
// the same counter climb correctly: every level is still claimed by one atomicOr).
template <int NW, int WS, int P>
__global__ void __launch_bounds__(256, P == 1 ? 6 : 4) k_ladder_pass1_roll(BankDev b, uint32_t k, uint32_t* __restrict__ lad,
                                                                          uint32_t log2w, uint32_t t, uint32_t* __restrict__ hll12) {
    constexpr int NK = NW - WS;
    __shared__ uint32_t s_hll[4096];
    __shared__ __align__(16) uint64_t s_stage[8][P1_STAGE_WORDS];
    const bool do_hll = hll12 != nullptr;
    if (do_hll) {
        for (int i = threadIdx.x; i < 4096; i += blockDim.x) s_hll[i] = 0;
        __syncthreads();
    }
    const uint64_t wmask = (1ULL << log2w) - 1;
    const uint64_t level_words = (4ULL << log2w) >> 5;
    uint32_t* top = lad + (uint64_t)(t - 1) * level_words;
    const uint32_t lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const uint32_t topb = 2u * k - 2u - 64u * (NK - 1);
    const uint64_t tmask = (topb + 2 >= 64) ? ~0ULL : ((1ULL << (topb + 2)) - 1);
    const uint64_t gw = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    for (uint64_t r0 = b.r_begin + gw * ROLL_RUN; r0 < b.r_end; r0 += nwarps * ROLL_RUN) {
        const uint64_t r = r0 + lane;
        uint32_t len = 0;
        uint64_t off = 0;
        if (r < b.r_end) {
            len = b.len[r];
            off = b.off[r];
            if (len < k || !bank_keep(b, r)) len = 0;
        }
        const uint32_t nk = len ? len - k + 1 : 0;
        __syncwarp();
        const RunStage st = stage_run(b.data, s_stage[wib], P1_STAGE_WORDS, lane, off, len, NK);
        const uint32_t steps = __reduce_max_sync(0xffffffffu, nk);
        uint64_t F[NK], R[NK];
        BaseCursor cur;
        if (nk) {
            window_strands<NW, WS>(st, b.data, off, k, F, R);
            cursor_at(cur, st, b.data, off + k);
        }
        for (uint32_t q = 0; q < steps; q += P) {
            uint32_t wd[4 * P], mk[4 * P];
            uint64_t h0[P];
            bool live[P], climb[4 * P];
#pragma unroll
            for (int p = 0; p < P; ++p) {
                const uint32_t qq = q + (uint32_t)p;
                live[p] = qq < nk;
                h0[p] = 0;
#pragma unroll
                for (int row = 0; row < 4; ++row) wd[4 * p + row] = mk[4 * p + row] = 0;
                if (!live[p]) continue;
                if (qq > 0) roll_strands<NK>(F, R, cursor_next(cur, st, b.data), topb, tmask);
                Key<NW> can;
                bool rc;
                strands_canonical<NW, WS>(F, R, can, rc);
                uint64_t hr[4];
                cms_row_hashes(key_fold<NW>(can), hr);
                h0[p] = hr[0];
#pragma unroll
                for (int row = 0; row < 4; ++row) {
                    const uint32_t bit = ((uint32_t)row << log2w) + (uint32_t)(hr[row] & wmask);
                    wd[4 * p + row] = bit >> 5;
                    mk[4 * p + row] = 1u << (bit & 31);
                }
            }
#pragma unroll
            for (int i = 0; i < 4 * P; ++i) climb[i] = live[i / 4] && !(__ldcg(top + wd[i]) & mk[i]);
            ladder_climb<4 * P>(lad, level_words, t, wd, mk, climb);
            if (do_hll) {
#pragma unroll
                for (int p = 0; p < P; ++p)
                    if (live[p] && (h0[p] & (PASS1_HLL_SAMPLE - 1)) == 0) {  // 1 key in 16 by hash
                        uint32_t idx, rho;
                        hll_idx_rho(h0[p], 12, idx, rho);
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
// Pass-2 record emit with the ladder gate, rolled.  Lane j walks read j of the run:
// at step q it rolls window q + 2 and issues its four gate loads, resolves the gate of
// window q + 1 (issued a step earlier) and emits window q, whose neighbours' gates it
// holds (build.rs:250-286: a window is emitted when it is solid and has a solid
// neighbour in its read; the right push carries the base after the window, the left
// push the complement of the base before it).
// ---------------------------------------------------------------------------
template <int NW, int WS, int MINB>
__global__ void __launch_bounds__(256, MINB) k_emit_roll(BankDev b, uint32_t k, const uint32_t* __restrict__ lad, uint32_t log2w,
                                                      uint32_t t_solid, TableDev t, BucketDev bk) {
    constexpr int NK = NW - WS;
    extern __shared__ __align__(16) uint64_t emit_smem[];
    const uint32_t lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    uint64_t* buf = emit_smem + (uint64_t)wib * (EMIT_WARP_WORDS(NW) + ROLL_STAGE_WORDS);
    uint8_t* bbuf = reinterpret_cast<uint8_t*>(buf + emit_buf(NW) * (NW + 1));
    uint16_t* rank = reinterpret_cast<uint16_t*>(bbuf + emit_buf(NW));
    uint32_t* hist = reinterpret_cast<uint32_t*>(rank + emit_buf(NW));
    unsigned long long* gbase = reinterpret_cast<unsigned long long*>(hist + EMIT_MAX_BUCKETS);
    uint16_t* perm = reinterpret_cast<uint16_t*>(gbase + EMIT_MAX_BUCKETS);
    uint64_t* stage = buf + EMIT_WARP_WORDS(NW);
    const uint32_t* top = lad + (uint64_t)(t_solid - 1) * ((4ULL << log2w) >> 5);
    const uint32_t topb = 2u * k - 2u - 64u * (NK - 1);
    const uint64_t tmask = (topb + 2 >= 64) ? ~0ULL : ((1ULL << (topb + 2)) - 1);
    const uint64_t gw = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    const uint32_t stripe = (uint32_t)(gw % bk.stripes);
    uint32_t n_buf = 0;  // warp-uniform
    for (uint64_t r0 = b.r_begin + gw * ROLL_RUN; r0 < b.r_end; r0 += nwarps * ROLL_RUN) {
        const uint64_t r = r0 + lane;
        uint32_t len = 0;
        uint64_t off = 0;
        if (r < b.r_end) {
            len = b.len[r];
            off = b.off[r];
            if (len < k + 1 || !bank_keep(b, r)) len = 0;
        }
        const uint32_t nk = len ? len - k + 1 : 0;
        __syncwarp();
        const RunStage st = stage_run(b.data, stage, ROLL_STAGE_WORDS, lane, off, len, NK);
        const uint32_t steps = __reduce_max_sync(0xffffffffu, nk);
        uint64_t F[NK], R[NK];
        BaseCursor cur;
        // pipeline: window q (emitted), q + 1 (gate resolved), q + 2 (gate loads in flight)
        Key<NW> kq{}, kq1{}, kq2{};
        bool rq = false, rq1 = false, rq2 = false;
        uint64_t hq = 0, hq1 = 0, hq2 = 0;
        bool gprev = false, gq = false, gq1 = false;
        uint32_t cq1 = 0, cq2 = 0;  // base entering when rolling to window q + 1 / q + 2
        uint32_t lq = 0, lq1 = 0, lq2 = 0;  // base leaving when rolling to window q / q + 1 / q + 2
        GateLoads g2;
        if (nk) {
            window_strands<NW, WS>(st, b.data, off, k, F, R);
            cursor_at(cur, st, b.data, off + k);
            strands_canonical<NW, WS>(F, R, kq, rq);
        }
        // window 0: gate now; window 1: gate loads issued
        GateLoads g0;
        gate_issue(top, log2w, nk ? key_fold<NW>(kq) : 0, nk > 0, g0);
        hq = g0.h0;
        if (nk > 1) {
            lq1 = (uint32_t)(F[0] >> topb) & 3u;
            cq1 = cursor_next(cur, st, b.data);
            roll_strands<NK>(F, R, cq1, topb, tmask);
            strands_canonical<NW, WS>(F, R, kq1, rq1);
        }
        GateLoads g1;
        gate_issue(top, log2w, nk > 1 ? key_fold<NW>(kq1) : 0, nk > 1, g1);
        hq1 = g1.h0;
        gq = gate_resolve(g0, nk > 0);
        for (uint32_t q = 0; q < steps; ++q) {
            // roll window q + 2 and issue its gate loads
            const bool l2 = q + 2 < nk;
            if (l2) {
                lq2 = (uint32_t)(F[0] >> topb) & 3u;
                cq2 = cursor_next(cur, st, b.data);
                roll_strands<NK>(F, R, cq2, topb, tmask);
                strands_canonical<NW, WS>(F, R, kq2, rq2);
            }
            gate_issue(top, log2w, l2 ? key_fold<NW>(kq2) : 0, l2, g2);
            hq2 = g2.h0;
            // gate of window q + 1, issued one step ago
            gq1 = gate_resolve(g1, q + 1 < nk);
            // emit window q
            bool emit = false;
            uint32_t info = 0, bucket = 0;
            if (q < nk) {
                const bool sl = q > 0 && gprev;
                const bool sr = q + 1 < nk && gq1;
                emit = gq && (sl || sr);
                if (emit) {
                    if (sr) info |= 8u | (cq1 + (rq ? 4u : 0u));
                    if (sl) info |= (8u | ((3u - lq) + (rq ? 0u : 4u))) << 4;
                    bucket = bucket_of_h(hq, bk.n_buckets);
                }
            }
            const uint32_t active = __ballot_sync(0xffffffffu, emit);
            if (emit) {
                const uint32_t pos = n_buf + __popc(active & ((1u << lane) - 1));
                rec_put<NW, WS>(buf + pos * (NW + 1), kq, info, bk);
                bbuf[pos] = (uint8_t)bucket;
            }
            n_buf += __popc(active);
            if (n_buf > emit_buf(NW) - 32) {
                __syncwarp();
                emit_flush<NW>(bk, stripe, lane, buf, bbuf, n_buf, hist, gbase, rank, perm);
                n_buf = 0;
            }
            // rotate
            gprev = gq;
            gq = gq1;
            kq = kq1;
            kq1 = kq2;
            rq = rq1;
            rq1 = rq2;
            hq = hq1;
            hq1 = hq2;
            lq = lq1;
            lq1 = lq2;
            cq1 = cq2;
            g1 = g2;
        }
    }
    __syncwarp();
    if (n_buf) emit_flush<NW>(bk, stripe, lane, buf, bbuf, n_buf, hist, gbase, rank, perm);
}

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
template <class Kern>
static int roll_grid(Kern kern, const Launch& L, size_t smem) {
    if (L.grid > 0) return L.grid;
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, L.block, smem) != cudaSuccess || per_sm < 1) per_sm = 1;
    return per_sm * (L.sms > 0 ? L.sms : 1);
}

template <int NW, int WS, int P>
static cudaError_t lp1r(const Launch& L, const BankDev& b, uint32_t k, uint32_t* lad, uint32_t log2w, uint32_t t, uint32_t* hll) {
    if (L.block != 256) return cudaErrorInvalidValue;  // the staging buffers are sized for 8 warps
    k_ladder_pass1_roll<NW, WS, P><<<roll_grid(k_ladder_pass1_roll<NW, WS, P>, L, 0), L.block, 0, L.stream>>>(b, k, lad, log2w, t,
                                                                                                             hll);
    return cudaGetLastError();
}
template <int P>
static cudaError_t lp1r_p(int nw, const Launch& L, const BankDev& b, uint32_t k, uint32_t* lad, uint32_t log2w, uint32_t t,
                          uint32_t* hll12) {
    const uint32_t ws = (64u * (uint32_t)nw - 2u * k) >> 6;
    if (nw == 1) return lp1r<1, 0, P>(L, b, k, lad, log2w, t, hll12);
    if (nw == 2) return ws == 0 ? lp1r<2, 0, P>(L, b, k, lad, log2w, t, hll12) : lp1r<2, 1, P>(L, b, k, lad, log2w, t, hll12);
    if (ws == 0) return lp1r<4, 0, P>(L, b, k, lad, log2w, t, hll12);
    if (ws == 1) return lp1r<4, 1, P>(L, b, k, lad, log2w, t, hll12);
    if (ws == 2) return lp1r<4, 2, P>(L, b, k, lad, log2w, t, hll12);
    return lp1r<4, 3, P>(L, b, k, lad, log2w, t, hll12);
}
cudaError_t launch_ladder_pass1_roll(int nw, const Launch& L, const BankDev& b, uint32_t k, uint32_t* lad, uint32_t log2w,
                                     uint32_t t, uint32_t* hll12, int windows_per_step) {
    if (t < 1 || t > LADDER_MAX_LEVELS || log2w > 29) return cudaErrorInvalidValue;
    return windows_per_step == 2 ? lp1r_p<2>(nw, L, b, k, lad, log2w, t, hll12) : lp1r_p<1>(nw, L, b, k, lad, log2w, t, hll12);
}

template <int NW, int WS, int MINB>
static cudaError_t emr_b(const Launch& L, const BankDev& b, uint32_t k, const uint32_t* lad, uint32_t log2w, uint32_t ts,
                         const TableDev& t, const BucketDev& bk) {
    const size_t smem = (size_t)(L.block / 32) * (EMIT_WARP_WORDS(NW) + ROLL_STAGE_WORDS) * 8;
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(k_emit_roll<NW, WS, MINB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
    }
    k_emit_roll<NW, WS, MINB><<<roll_grid(k_emit_roll<NW, WS, MINB>, L, smem), L.block, smem, L.stream>>>(b, k, lad, log2w, ts,
                                                                                                          t, bk);
    return cudaGetLastError();
}
// Register budget: two blocks per SM for 256-bit keys (three windows of three key
// words in flight spill at three blocks: k = 77 8.88 ms per 100x pass at three blocks,
// 5.74 at two), three for narrower keys; two_blocks = two for every width.
template <int NW, int WS>
static cudaError_t emr(const Launch& L, const BankDev& b, uint32_t k, const uint32_t* lad, uint32_t log2w, uint32_t ts,
                       const TableDev& t, const BucketDev& bk, bool two_blocks) {
    if constexpr (NW == 4) {
        return emr_b<NW, WS, 2>(L, b, k, lad, log2w, ts, t, bk);
    } else {
        if (two_blocks) return emr_b<NW, WS, 2>(L, b, k, lad, log2w, ts, t, bk);
        return emr_b<NW, WS, 3>(L, b, k, lad, log2w, ts, t, bk);
    }
}
cudaError_t launch_emit_roll(int nw, const Launch& L, const BankDev& b, uint32_t k, const uint32_t* lad, uint32_t log2w,
                             uint32_t t_solid, const TableDev& t, const BucketDev& bk, bool two_blocks) {
    if (t_solid < 1 || t_solid > LADDER_MAX_LEVELS || log2w > 29) return cudaErrorInvalidValue;
    const uint32_t ws = (64u * (uint32_t)nw - 2u * k) >> 6;
    if (nw == 1) return emr<1, 0>(L, b, k, lad, log2w, t_solid, t, bk, two_blocks);
    if (nw == 2)
        return ws == 0 ? emr<2, 0>(L, b, k, lad, log2w, t_solid, t, bk, two_blocks)
                       : emr<2, 1>(L, b, k, lad, log2w, t_solid, t, bk, two_blocks);
    if (ws == 0) return emr<4, 0>(L, b, k, lad, log2w, t_solid, t, bk, two_blocks);
    if (ws == 1) return emr<4, 1>(L, b, k, lad, log2w, t_solid, t, bk, two_blocks);
    if (ws == 2) return emr<4, 2>(L, b, k, lad, log2w, t_solid, t, bk, two_blocks);
    return emr<4, 3>(L, b, k, lad, log2w, t_solid, t, bk, two_blocks);
}

}  // namespace fbk
