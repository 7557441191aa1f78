// fbk_shard.cu — device side of one isolate counted across ranks: the accumulated
// KmerAcc rows of a rank's table grouped by the owner rank of their key, and an
// owner's table rebuilt from the rows it received (src/graph/build.rs:141-196: the
// 64 mutex-sharded maps whose entries add up saturating u16 counts; here the
// partition is by rank, and the sum is exact in u32 and capped when read).
//
// A row is NW key words (big-endian, as exported) and two words of edge counts:
// e0 | e1 << 16 | e2 << 32 | e3 << 48, then e4 .. e7 the same way.  The owner of a
// key is splitmix64(fold(key)) mod world, fold = KmerInt::to_u64 (kmer.rs:115-117,
// 192-194, 332-334).
#include "fbk_device.cuh"
#include "fbk_kernels.cuh"
#include "fbk_table.cuh"

namespace fbk {

template <int NW>
__device__ __forceinline__ uint32_t row_owner(const uint64_t* row, uint32_t world) {
    uint64_t f = 0;
#pragma unroll
    for (int i = 0; i < NW; ++i) f ^= row[i];
    return (uint32_t)(smix(f) % world);
}

// counts[o] += rows of owner o
template <int NW>
__global__ void __launch_bounds__(256) k_owner_hist(const uint64_t* __restrict__ keys, uint64_t n, uint32_t world,
                                                    unsigned long long* __restrict__ counts) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        atomicAdd(&counts[row_owner<NW>(keys + i * NW, world)], 1ull);
}

// Rows in owner order: cursor[o] starts at owner o's first position (exclusive scan of
// the counts); the order within an owner is arbitrary (the owner sums equal keys).
template <int NW>
__global__ void __launch_bounds__(256) k_owner_scatter(const uint64_t* __restrict__ keys, const uint16_t* __restrict__ edges,
                                                       uint64_t n, uint32_t world, unsigned long long* __restrict__ cursor,
                                                       uint64_t* __restrict__ rows) {
    constexpr int RW = NW + 2;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t* key = keys + i * NW;
        const unsigned long long pos = atomicAdd(&cursor[row_owner<NW>(key, world)], 1ull);
        uint64_t* dst = rows + pos * RW;
#pragma unroll
        for (int j = 0; j < NW; ++j) dst[j] = key[j];
        const uint16_t* e = edges + i * 8;
        dst[NW] = (uint64_t)e[0] | ((uint64_t)e[1] << 16) | ((uint64_t)e[2] << 32) | ((uint64_t)e[3] << 48);
        dst[NW + 1] = (uint64_t)e[4] | ((uint64_t)e[5] << 16) | ((uint64_t)e[6] << 32) | ((uint64_t)e[7] << 48);
    }
}

// Adds every row's edge counts to its key's slot (claimed from the key's home slot).
template <int NW>
__global__ void __launch_bounds__(256) k_rows_upsert(const uint64_t* __restrict__ rows, uint64_t n, TableDev t,
                                                     uint32_t* __restrict__ status) {
    constexpr int RW = NW + 2;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t* row = rows + i * RW;
        Key<NW> key;
#pragma unroll
        for (int j = 0; j < NW; ++j) key.w[j] = row[j];
        const uint64_t f = key_fold<NW>(key);
        const uint64_t home = home_slot(f, t.cap);
        int64_t s;
        if constexpr (NW == 1) s = table_slot1(t, key.w[0], home, status);
        else if constexpr (NW == 2) s = table_slot2(t, key, home, status);
        else s = table_slotw<NW>(t, key, f, home, status);
        if (s < 0) continue;
        uint32_t* c = t.cnt + (uint64_t)s * 8;
#pragma unroll
        for (int e = 0; e < 8; ++e) {
            const uint32_t v = (uint32_t)(row[NW + (e >> 2)] >> ((e & 3) * 16)) & 0xFFFFu;
            if (v) atomicAdd(&c[e], v);
        }
    }
}

static int grid_of(const Launch& L, uint64_t n) {
    const uint64_t want = (n + L.block - 1) / L.block;
    const uint64_t cap = (uint64_t)(L.sms > 0 ? L.sms : 152) * 8;
    return (int)(want < 1 ? 1 : want < cap ? want : cap);
}

cudaError_t launch_owner_hist(int nw, const Launch& L, const uint64_t* keys, uint64_t n, uint32_t world,
                              unsigned long long* counts) {
    if (!n) return cudaSuccess;
    const int g = grid_of(L, n);
    if (nw == 1) k_owner_hist<1><<<g, L.block, 0, L.stream>>>(keys, n, world, counts);
    else if (nw == 2) k_owner_hist<2><<<g, L.block, 0, L.stream>>>(keys, n, world, counts);
    else k_owner_hist<4><<<g, L.block, 0, L.stream>>>(keys, n, world, counts);
    return cudaGetLastError();
}

cudaError_t launch_owner_scatter(int nw, const Launch& L, const uint64_t* keys, const uint16_t* edges, uint64_t n, uint32_t world,
                                 unsigned long long* cursor, uint64_t* rows) {
    if (!n) return cudaSuccess;
    const int g = grid_of(L, n);
    if (nw == 1) k_owner_scatter<1><<<g, L.block, 0, L.stream>>>(keys, edges, n, world, cursor, rows);
    else if (nw == 2) k_owner_scatter<2><<<g, L.block, 0, L.stream>>>(keys, edges, n, world, cursor, rows);
    else k_owner_scatter<4><<<g, L.block, 0, L.stream>>>(keys, edges, n, world, cursor, rows);
    return cudaGetLastError();
}

cudaError_t launch_rows_upsert(int nw, const Launch& L, const uint64_t* rows, uint64_t n, const TableDev& t, uint32_t* status) {
    if (!n) return cudaSuccess;
    const int g = grid_of(L, n);
    if (nw == 1) k_rows_upsert<1><<<g, L.block, 0, L.stream>>>(rows, n, t, status);
    else if (nw == 2) k_rows_upsert<2><<<g, L.block, 0, L.stream>>>(rows, n, t, status);
    else k_rows_upsert<4><<<g, L.block, 0, L.stream>>>(rows, n, t, status);
    return cudaGetLastError();
}

}  // namespace fbk
