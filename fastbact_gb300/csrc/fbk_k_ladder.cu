// fbk_k_ladder.cu — the CMS gate of the build front end as threshold ladders.
//
// Pass 2 reads the pass-1 sketch only through one predicate (build.rs:259-267):
//   solid(x)  <=>  min over rows r of min(cap, count_r(col_r(x))) >= t_solid.
// With 1 <= t_solid <= cap that is "every row's count reached t_solid".  A ladder
// keeps t_solid bits per (row, column); level j (0-based) is set by the (j+1)-th
// increment.  An increment climbs: atomicOr on level 0; if that bit was already set,
// level 1; and so on.  Each level is claimed by exactly one increment, and a level is
// tried only when the one below it is already set, so the claimed levels are always
// {0 .. m-1} with m = min(t_solid, increments): the top level is set iff the count
// reached t_solid.  The top level is read first, so a saturated counter costs one L2
// load and no atomic.
//
// Size: t_solid x 4 x 2^log2w bits — 16 MB for t = 2 and 2^24 columns — so the whole
// gate stays in L2 and one sweep serves all four rows (the exact u32 sketch needs one
// 64 MB sweep per row).  Layout: bit ((level * 4 + row) << log2w) + col.
#include "fbk_device.cuh"
#include "fbk_kernels.cuh"

namespace fbk {

// WS = (64*NW - 2k) / 64 is a template parameter (key words below it are constant
// zeros).
template <int NW, int ILP, int WS>
__global__ void __launch_bounds__(256, ILP == 1 ? 6 : 2) k_ladder_pass1(BankDev b, uint32_t k, uint32_t* __restrict__ lad,
                                                                        uint32_t log2w, uint32_t t, uint32_t* __restrict__ hll12) {
    __shared__ uint32_t s_hll[4096];
    const bool do_hll = hll12 != nullptr;
    if (do_hll) {
        for (int i = threadIdx.x; i < 4096; i += blockDim.x) s_hll[i] = 0;
        __syncthreads();
    }
    const uint64_t wmask = (1ULL << log2w) - 1;
    const uint64_t level_words = (4ULL << log2w) >> 5;
    uint32_t* top = lad + (uint64_t)(t - 1) * level_words;
    const uint32_t lane = threadIdx.x & 31;
    const uint64_t gw = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    for (uint64_t r = b.r_begin + gw; r < b.r_end; r += nwarps) {
        const uint32_t len = b.len[r];
        if (len < k || !bank_keep(b, r)) continue;
        const uint64_t off = b.off[r];
        const uint32_t nk = len - k + 1;
        // Warp-uniform trip counts throughout (ILP chunks of 32 windows at a time, all t
        // levels): the climb is a predicated atomic per level, so the warp never splits.
        // With ILP = 2 each lane takes two windows and issues the eight top-level loads
        // together (the kernel is bound by their L2 latency) at half the resident warps.
        // Lanes past the read's last window keep word 0 / mask 0 and never climb.
        for (uint32_t it = 0; it < ((nk + 31) >> 5); it += ILP) {
            uint32_t wd[4 * ILP], mk[4 * ILP];
            bool live[ILP], climb[4 * ILP];
            uint64_t h0[ILP];
#pragma unroll
            for (int p = 0; p < ILP; ++p) {
                const uint32_t q = ((it + p) << 5) + lane;
                live[p] = q < nk;
                h0[p] = 0;
#pragma unroll
                for (int row = 0; row < 4; ++row) wd[4 * p + row] = mk[4 * p + row] = 0;
                if (!live[p]) continue;
                Key<NW> can{};
                bool rc;
                canonical_ws<NW, WS>(b.data, off + q, k, can, rc);
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
            // false once the count reached t, and for lanes past the read's last window
#pragma unroll
            for (int i = 0; i < 4 * ILP; ++i) climb[i] = live[i / 4] && !(__ldcg(top + wd[i]) & mk[i]);
            ladder_climb<4 * ILP>(lad, level_words, t, wd, mk, climb);
            if (do_hll) {
#pragma unroll
                for (int p = 0; p < ILP; ++p)
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

// The same pass 1 software-pipelined over a read's chunks of 32 windows: the top-level
// loads of chunk it + 1 are issued before chunk it climbs, so their L2 latency overlaps
// the climb's atomics and the next chunk's hashing (tuning ladder_ilp = 3).
struct LadderChunk {
    uint32_t wd[4], mk[4], top[4];
    uint64_t h0;
    bool live;
};
template <int NW, int WS>
__device__ __forceinline__ void ladder_prep(const BankDev& b, uint64_t off, uint32_t q, uint32_t nk, uint32_t k, uint32_t log2w,
                                            uint64_t wmask, const uint32_t* __restrict__ top, LadderChunk& c) {
    c.live = q < nk;
    c.h0 = 0;
#pragma unroll
    for (int row = 0; row < 4; ++row) {
        c.wd[row] = c.mk[row] = 0;
        c.top[row] = ~0u;
    }
    if (!c.live) return;
    Key<NW> can{};
    bool rc;
    canonical_ws<NW, WS>(b.data, off + q, k, can, rc);
    uint64_t hr[4];
    cms_row_hashes(key_fold<NW>(can), hr);
    c.h0 = hr[0];
#pragma unroll
    for (int row = 0; row < 4; ++row) {
        const uint32_t bit = ((uint32_t)row << log2w) + (uint32_t)(hr[row] & wmask);
        c.wd[row] = bit >> 5;
        c.mk[row] = 1u << (bit & 31);
    }
#pragma unroll
    for (int row = 0; row < 4; ++row) c.top[row] = __ldcg(top + c.wd[row]);
}

template <int NW, int WS>
__global__ void __launch_bounds__(256, 4) k_ladder_pass1p(BankDev b, uint32_t k, uint32_t* __restrict__ lad, uint32_t log2w,
                                                          uint32_t t, uint32_t* __restrict__ hll12) {
    __shared__ uint32_t s_hll[4096];
    const bool do_hll = hll12 != nullptr;
    if (do_hll) {
        for (int i = threadIdx.x; i < 4096; i += blockDim.x) s_hll[i] = 0;
        __syncthreads();
    }
    const uint64_t wmask = (1ULL << log2w) - 1;
    const uint64_t level_words = (4ULL << log2w) >> 5;
    const uint32_t* top = lad + (uint64_t)(t - 1) * level_words;
    const uint32_t lane = threadIdx.x & 31;
    const uint64_t gw = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    for (uint64_t r = b.r_begin + gw; r < b.r_end; r += nwarps) {
        const uint32_t len = b.len[r];
        if (len < k || !bank_keep(b, r)) continue;
        const uint64_t off = b.off[r];
        const uint32_t nk = len - k + 1;
        LadderChunk cur;
        ladder_prep<NW, WS>(b, off, lane, nk, k, log2w, wmask, top, cur);
        for (uint32_t it = 0; it < ((nk + 31) >> 5); ++it) {
            LadderChunk nxt;
            ladder_prep<NW, WS>(b, off, ((it + 1) << 5) + lane, nk, k, log2w, wmask, top, nxt);
            bool climb[4];
#pragma unroll
            for (int row = 0; row < 4; ++row) climb[row] = cur.live && !(cur.top[row] & cur.mk[row]);
            ladder_climb<4>(lad, level_words, t, cur.wd, cur.mk, climb);
            if (do_hll && cur.live && (cur.h0 & (PASS1_HLL_SAMPLE - 1)) == 0) {
                uint32_t idx, rho;
                hll_idx_rho(cur.h0, 12, idx, rho);
                if (s_hll[idx] < rho) atomicMax(&s_hll[idx], rho);
            }
            cur = nxt;
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

// Solidity bitmap from a ladder: a window's bit is cleared unless the top level is
// set in all four rows (one sweep).
template <int NW>
__global__ void __launch_bounds__(256) k_ladder_solid(BankDev b, uint32_t k, const uint32_t* __restrict__ lad, uint32_t log2w,
                                                      uint32_t t, uint32_t* __restrict__ bm) {
    const uint64_t wmask = (1ULL << log2w) - 1;
    const uint32_t* top = lad + (uint64_t)(t - 1) * ((4ULL << log2w) >> 5);
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
#pragma unroll
                for (int row = 0; row < 4; ++row) {
                    const uint64_t bit = ((uint64_t)row << log2w) + (smix(key ^ cms_seed(row)) & wmask);
                    clr |= !((__ldg(top + (bit >> 5)) >> (bit & 31)) & 1u);
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

template <class K>
static int grid_l(K kernel, const Launch& L) {
    if (L.grid > 0) return L.grid;
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, L.block, 0) != cudaSuccess || per_sm < 1) per_sm = 1;
    return per_sm * (L.sms > 0 ? L.sms : 1);
}

template <int NW, int ILP, int WS>
static cudaError_t lp1(const Launch& L, const BankDev& b, uint32_t k, uint32_t* lad, uint32_t log2w, uint32_t t, uint32_t* hll) {
    if constexpr (ILP == 3)
        k_ladder_pass1p<NW, WS><<<grid_l(k_ladder_pass1p<NW, WS>, L), L.block, 0, L.stream>>>(b, k, lad, log2w, t, hll);
    else
        k_ladder_pass1<NW, ILP, WS><<<grid_l(k_ladder_pass1<NW, ILP, WS>, L), L.block, 0, L.stream>>>(b, k, lad, log2w, t, hll);
    return cudaGetLastError();
}
template <int NW, int ILP>
static cudaError_t lp1_ws(const Launch& L, const BankDev& b, uint32_t k, uint32_t* lad, uint32_t log2w, uint32_t t, uint32_t* hll) {
    const uint32_t ws = (64u * NW - 2u * k) >> 6;
    if constexpr (NW == 1) {
        return lp1<1, ILP, 0>(L, b, k, lad, log2w, t, hll);
    } else if constexpr (NW == 2) {
        return ws == 0 ? lp1<2, ILP, 0>(L, b, k, lad, log2w, t, hll) : lp1<2, ILP, 1>(L, b, k, lad, log2w, t, hll);
    } else {
        if (ws == 0) return lp1<4, ILP, 0>(L, b, k, lad, log2w, t, hll);
        if (ws == 1) return lp1<4, ILP, 1>(L, b, k, lad, log2w, t, hll);
        if (ws == 2) return lp1<4, ILP, 2>(L, b, k, lad, log2w, t, hll);
        return lp1<4, ILP, 3>(L, b, k, lad, log2w, t, hll);
    }
}
cudaError_t launch_ladder_pass1(int nw, const Launch& L, const BankDev& b, uint32_t k, uint32_t* lad, uint32_t log2w, uint32_t t,
                                uint32_t* hll12, int ilp) {
    if (t < 1 || t > LADDER_MAX_LEVELS || log2w > 29) return cudaErrorInvalidValue;  // bit indices fit 32 bits
    if (ilp == 4 || ilp == 5) {  // one lane per read, rolled (fbk_k_roll.cu); 5: two windows per step
        Launch L2 = L;
        L2.block = 256;
        return launch_ladder_pass1_roll(nw, L2, b, k, lad, log2w, t, hll12, ilp == 5 ? 2 : 1);
    }
    if (ilp == 2) {
        if (nw == 1) return lp1_ws<1, 2>(L, b, k, lad, log2w, t, hll12);
        if (nw == 2) return lp1_ws<2, 2>(L, b, k, lad, log2w, t, hll12);
        return lp1_ws<4, 2>(L, b, k, lad, log2w, t, hll12);
    }
    if (ilp == 3) {
        if (nw == 1) return lp1_ws<1, 3>(L, b, k, lad, log2w, t, hll12);
        if (nw == 2) return lp1_ws<2, 3>(L, b, k, lad, log2w, t, hll12);
        return lp1_ws<4, 3>(L, b, k, lad, log2w, t, hll12);
    }
    if (nw == 1) return lp1_ws<1, 1>(L, b, k, lad, log2w, t, hll12);
    if (nw == 2) return lp1_ws<2, 1>(L, b, k, lad, log2w, t, hll12);
    return lp1_ws<4, 1>(L, b, k, lad, log2w, t, hll12);
}

template <int NW>
static cudaError_t lsol(const Launch& L, const BankDev& b, uint32_t k, const uint32_t* lad, uint32_t log2w, uint32_t t, uint32_t* bm) {
    k_ladder_solid<NW><<<grid_l(k_ladder_solid<NW>, L), L.block, 0, L.stream>>>(b, k, lad, log2w, t, bm);
    return cudaGetLastError();
}
cudaError_t launch_ladder_solid(int nw, const Launch& L, const BankDev& b, uint32_t k, const uint32_t* lad, uint32_t log2w,
                                uint32_t t, uint32_t* bm) {
    if (t < 1 || t > LADDER_MAX_LEVELS) return cudaErrorInvalidValue;
    if (nw == 1) return lsol<1>(L, b, k, lad, log2w, t, bm);
    if (nw == 2) return lsol<2>(L, b, k, lad, log2w, t, bm);
    return lsol<4>(L, b, k, lad, log2w, t, bm);
}

}  // namespace fbk
