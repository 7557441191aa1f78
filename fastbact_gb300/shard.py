"""One isolate counted across ranks (one process per GPU, torch.distributed).

Reads are partitioned between ranks; each rank counts its share with its own
engine and three exchange steps make the result equal to one process counting
every read (src/graph/build.rs:84-328):

* pass 1: the rank sketches (counts capped at 15 or 65535) are summed and capped
  again with one all-reduce.  Exact, because the increments are positive:
  min(cap, min(cap, a) + min(cap, b)) = min(cap, a + b).
* pass 2: every rank gates its own reads with the merged sketch and accumulates a
  local table; each accumulated row (canonical key, 8 edge counts capped at 65535)
  goes to the owner rank of its key, splitmix64(fold(key)) mod world, in one
  all-to-all.  The owner sums the rows of a key (the same capped-sum identity) and
  converts them to SolidKmerNodes (build.rs:295-328): mask bit e iff
  edges[e] >= min_trans_cov, cov = min(65535, sum of edges), node cov =
  max(1, cov / 2), rows with an empty mask dropped.
* the table digest is a sum over rows, so the owners' digests add up (mod 2^64)
  to the single-process digest.

The genome-size estimator's sample loop (estimator.rs:296-379) shards by pair range
with two exchanges (sharded_estimate): the first occurrence touching each sketch
counter (all-reduce MIN; occurrence t's estimate is >= 2 iff every row's counter was
touched before t), then the HLL register maxima per checkpoint segment (all-reduce
MAX); the checkpoints and the post-math run on the merged registers.

The engine is what counts one rank's reads.  With DeviceEngine (this library's
kernels) the data plane stays on the GPU: the rank sketches are reduced in place on
the device counters (fbk_cms_counts_device), the accumulated rows leave the table
already grouped by owner (fbk_table_export_acc_owned) and the owner rebuilds and
converts its table from the received rows on the device (fbk_table_from_acc_rows).
The collectives move CUDA tensors when the process group is NCCL and host tensors
otherwise (gloo).  Any other object with the three host methods (pass1, load,
pass2) can stand in for the engine, which is how the exchange logic is tested on
hosts without a GPU.
"""
from __future__ import annotations

import numpy as np

M64 = np.uint64(0xFFFFFFFFFFFFFFFF)


def splitmix64_np(z: np.ndarray) -> np.ndarray:
    """splitmix64 finaliser (src/common/sketch.rs:13-18) on a uint64 array."""
    z = z.astype(np.uint64, copy=True)
    with np.errstate(over="ignore"):
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
    return z ^ (z >> np.uint64(31))


def fold(keys: np.ndarray) -> np.ndarray:
    """KmerInt::to_u64 (kmer.rs:115-117, 192-194, 332-334): XOR of the key words."""
    f = np.zeros(len(keys), np.uint64)
    for j in range(keys.shape[1]):
        f ^= keys[:, j]
    return f


def owner(keys: np.ndarray, world: int) -> np.ndarray:
    return (splitmix64_np(fold(keys)) % np.uint64(world)).astype(np.int64)


def shard_bank(bank, rank: int, world: int):
    """The reads of `bank` that rank `rank` of `world` counts (every world-th read
    of each arena); the packed words are shared, not copied."""
    from . import api

    arenas = []
    for a in bank.arenas:
        sel = np.arange(rank, len(a), world)
        arenas.append(api.BitSeqArena(a.data, np.ascontiguousarray(a.offsets[sel]), np.ascontiguousarray(a.lengths[sel]),
                                      np.ascontiguousarray(a.pair_idx[sel]) if a.pair_idx is not None else None))
    return api.ReadBank(*arenas)


def sketch_values(raw: np.ndarray, counter_bits: int) -> np.ndarray:
    """Counter values of an exported sketch (reference layout)."""
    if counter_bits == 16:
        return raw.view(np.uint16).astype(np.int64)
    v = np.empty(raw.size * 2, np.int64)
    v[0::2] = raw & 15
    v[1::2] = raw >> 4
    return v


def sketch_bytes(values: np.ndarray, counter_bits: int) -> np.ndarray:
    if counter_bits == 16:
        return values.astype(np.uint16).view(np.uint8)
    v = values.astype(np.uint8)
    return (v[0::2] | (v[1::2] << 4)).astype(np.uint8)


def merge_sketch(raw: np.ndarray, counter_bits: int, group=None) -> np.ndarray:
    """All-reduce of the rank sketches: sum, then cap."""
    import torch
    import torch.distributed as dist

    cap = 15 if counter_bits == 4 else 0xFFFF
    t = torch.from_numpy(sketch_values(raw, counter_bits))
    dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
    return sketch_bytes(np.minimum(t.numpy(), cap), counter_bits)


def exchange_rows(keys: np.ndarray, edges: np.ndarray, world: int, group=None):
    """Sends every accumulated row to the owner of its key (one all-to-all);
    returns the rows this rank owns."""
    import torch
    import torch.distributed as dist

    nw = keys.shape[1]
    dest = owner(keys, world) if len(keys) else np.zeros(0, np.int64)
    order = np.argsort(dest, kind="stable")
    rows = np.concatenate([keys.view(np.int64), edges.astype(np.int64)], axis=1)[order] if len(keys) else \
        np.zeros((0, nw + 8), np.int64)
    send = np.bincount(dest, minlength=world).astype(np.int64)
    recv = torch.zeros(world, dtype=torch.int64)
    dist.all_to_all_single(recv, torch.from_numpy(send), group=group)
    recv = recv.numpy()
    out = torch.zeros(int(recv.sum()) * (nw + 8), dtype=torch.int64)
    dist.all_to_all_single(out, torch.from_numpy(np.ascontiguousarray(rows).reshape(-1)),
                           output_split_sizes=[int(x) * (nw + 8) for x in recv],
                           input_split_sizes=[int(x) * (nw + 8) for x in send], group=group)
    got = out.numpy().reshape(-1, nw + 8)
    return np.ascontiguousarray(got[:, :nw]).view(np.uint64), got[:, nw:]


def reduce_rows(keys: np.ndarray, edges: np.ndarray):
    """Sums the edge counts of equal keys (capped at 65535); rows sorted by key."""
    nw = keys.shape[1]
    if len(keys) == 0:
        return keys.reshape(0, nw), np.zeros((0, 8), np.uint16)
    order = np.lexsort(tuple(keys[:, j] for j in reversed(range(nw))))
    k, e = keys[order], edges[order].astype(np.int64)
    new = np.ones(len(k), bool)
    new[1:] = np.any(k[1:] != k[:-1], axis=1)
    starts = np.flatnonzero(new)
    summed = np.add.reduceat(e, starts, axis=0)
    return k[starts], np.minimum(summed, 0xFFFF).astype(np.uint16)


def convert(keys: np.ndarray, edges: np.ndarray, min_trans_cov: int):
    """SolidKmerNode conversion (build.rs:295-328) of accumulated rows:
    (keys, cov u16, mask u8) of the rows with a non-empty mask."""
    e = edges.astype(np.int64)
    cov = np.minimum(e.sum(axis=1), 0xFFFF)
    mask = np.zeros(len(e), np.int64)
    for b in range(8):
        mask |= (e[:, b] >= min_trans_cov).astype(np.int64) << b
    keep = mask != 0
    node_cov = np.maximum(1, cov[keep] // 2).astype(np.uint16)
    return keys[keep], node_cov, mask[keep].astype(np.uint8)


def digest(keys: np.ndarray, cov: np.ndarray, mask: np.ndarray) -> int:
    """Order-free digest of SolidKmerNode rows: sum over rows of
    smix(kd ^ smix(cov << 8 | mask)), kd = smix chained over the key words."""
    kd = np.zeros(len(keys), np.uint64)
    for j in range(keys.shape[1]):
        kd = splitmix64_np(kd ^ keys[:, j])
    v = splitmix64_np(kd ^ splitmix64_np((cov.astype(np.uint64) << np.uint64(8)) | mask.astype(np.uint64)))
    with np.errstate(over="ignore"):
        return int(np.sum(v, dtype=np.uint64))


class DistComm:
    """The two collectives of the exchange over a torch.distributed group: CUDA
    tensors go to the collective as they are when the backend is NCCL; with any other
    backend they are staged through host memory."""

    def __init__(self, group=None):
        import torch.distributed as dist

        self.group = group
        self.on_device = dist.get_backend(group) == "nccl"

    def _dev(self, t):
        return t if self.on_device else t.cpu()

    def all_reduce_sum_(self, t):
        import torch.distributed as dist

        x = self._dev(t)
        dist.all_reduce(x, op=dist.ReduceOp.SUM, group=self.group)
        if x is not t:
            t.copy_(x)

    def all_to_all_rows(self, rows, send_counts):
        """rows: (n, w) tensor grouped by destination rank, send_counts[r] rows for rank
        r; returns (received rows on rows' device, received counts)."""
        import torch
        import torch.distributed as dist

        w = rows.shape[1]
        dev = rows.device if self.on_device else torch.device("cpu")
        send = torch.tensor([int(c) for c in send_counts], dtype=torch.int64, device=dev)
        recv = torch.zeros_like(send)
        dist.all_to_all_single(recv, send, group=self.group)
        recv_l = [int(x) for x in recv.cpu()]
        src = rows.contiguous().to(dev)
        dst = torch.empty((sum(recv_l), w), dtype=rows.dtype, device=dev)
        dist.all_to_all_single(dst.view(-1), src.view(-1), output_split_sizes=[x * w for x in recv_l],
                               input_split_sizes=[int(x) * w for x in send_counts], group=self.group)
        return dst.to(rows.device), recv_l

    def sum_u64(self, v: int) -> int:
        import torch
        import torch.distributed as dist

        t = torch.tensor([v - (1 << 64) if v >= (1 << 63) else v], dtype=torch.int64)
        t = t.cuda() if self.on_device else t
        dist.all_reduce(t, op=dist.ReduceOp.SUM, group=self.group)  # wraps: the sum mod 2^64
        return int(t.item()) & ((1 << 64) - 1)


def _sharded_build_device(engine, bank, k, key_bits, log2w, counter_bits, target_solid_cov, rank, world, comm):
    import torch

    from . import api

    min_trans_cov = 3 if target_solid_cov is None else target_solid_cov
    mine = shard_bank(bank, rank, world)
    engine.pass1_device(mine, k, key_bits, log2w, counter_bits)
    counts = engine.sketch_tensor()  # the device counters, reduced in place
    engine.ctx.sync()
    comm.all_reduce_sum_(counts)
    torch.cuda.synchronize()
    engine.clamp()
    rows, send = engine.owned_rows(mine, k, key_bits, target_solid_cov, world)
    got, _ = comm.all_to_all_rows(rows, send)
    torch.cuda.synchronize()
    table = api.table_from_acc_rows(engine.ctx, k, key_bits, min_trans_cov, got)
    merged = engine.cms.export()
    engine.release()
    d = comm.sum_u64(table.digest()[0])
    nkeys, ncov, nmask = table.export(sort=True)
    table.release()
    return (nkeys, ncov, nmask), merged, d


def sharded_build(engine, bank, k: int, key_bits: int, log2w: int, counter_bits: int, target_solid_cov: int | None,
                  rank: int, world: int, group=None, comm=None):
    """Counts this rank's share of `bank` and runs the exchange steps.  Returns the
    SolidKmerNode rows this rank owns (sorted by key), the merged sketch bytes and
    the global digest.  target_solid_cov as in build_cdbg (None: gate 2, mask 3).
    A DeviceEngine keeps the data plane on the GPU; `comm` (default: DistComm over
    `group`) carries its collectives."""
    import torch
    import torch.distributed as dist

    if isinstance(engine, DeviceEngine):
        return _sharded_build_device(engine, bank, k, key_bits, log2w, counter_bits, target_solid_cov, rank, world,
                                     comm or DistComm(group))
    min_trans_cov = 3 if target_solid_cov is None else target_solid_cov
    mine = shard_bank(bank, rank, world)
    raw = engine.pass1(mine, k, key_bits, log2w, counter_bits)
    merged = merge_sketch(raw, counter_bits, group)
    engine.load(merged)
    keys, edges = engine.pass2(mine, k, key_bits, target_solid_cov)
    okeys, oedges = exchange_rows(keys, edges, world, group)
    rkeys, redges = reduce_rows(okeys, oedges)
    nkeys, ncov, nmask = convert(rkeys, redges, min_trans_cov)
    d = digest(nkeys, ncov, nmask)
    t = torch.tensor([d - (1 << 64) if d >= (1 << 63) else d], dtype=torch.int64)
    dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)  # wraps: the sum mod 2^64
    return (nkeys, ncov, nmask), merged, int(t.item()) & ((1 << 64) - 1)


def pair_range(n_use: int, rank: int, world: int) -> tuple[int, int]:
    """The contiguous pairs of the estimator sample that rank `rank` of `world` runs."""
    return n_use * rank // world, n_use * (rank + 1) // world


def sharded_estimate(engine, lengths: np.ndarray, n_pairs: int, stats, rank: int, world: int, group=None, **params):
    """estimate_genome's sample loop over this rank's pairs and the two exchange steps.
    Every rank holds the whole sample (R1,R2 interleaved; `lengths` are its read
    lengths) and gets the same (GenomeEstimate, regs_total, regs_solid) as one process
    running every pair.  `engine` runs the two stages on the rank's pairs:
    firstpos(n_use, pair_begin, pair_end) and segments(n_use, pair_begin, pair_end, first)."""
    import torch
    import torch.distributed as dist

    from . import api

    n_use, _ = api.est_shard_plan(lengths, n_pairs, stats, **params)
    lo, hi = pair_range(n_use, rank, world)
    first = torch.from_numpy(engine.firstpos(n_use, lo, hi).astype(np.int64))
    dist.all_reduce(first, op=dist.ReduceOp.MIN, group=group)
    merged_first = first.numpy().astype(np.uint32)
    regs = torch.from_numpy(engine.segments(n_use, lo, hi, merged_first).astype(np.int32))
    dist.all_reduce(regs, op=dist.ReduceOp.MAX, group=group)
    return api.est_shard_finish(lengths, n_use, stats, regs.numpy().astype(np.uint8), **params)


class DeviceEstimatorEngine:
    """Runs a rank's estimator stages on its GPU; the sample is uploaded once."""

    def __init__(self, ctx, sample, lengths: np.ndarray, **params):
        from . import api

        self.ctx, self.params = ctx, params
        self.lengths = np.ascontiguousarray(lengths, np.uint32)
        self.bank = api.DeviceBank(ctx, sample)

    def firstpos(self, n_use, lo, hi):
        from . import api

        return api.est_shard_firstpos(self.ctx, self.bank, self.lengths, n_use, lo, hi, **self.params)

    def segments(self, n_use, lo, hi, first):
        from . import api

        return api.est_shard_segments(self.ctx, self.bank, self.lengths, n_use, lo, hi, first, **self.params)

    def release(self):
        self.bank.release()


class DeviceEngine:
    """Counts one rank's reads on its GPU with this library's kernels.  The host
    methods (pass1, load, pass2) export to numpy; the device methods keep the sketch
    and the accumulated rows on the GPU for the collectives."""

    def __init__(self, ctx):
        self.ctx = ctx
        self.cms = None
        self.dbank = None

    # ---- device data plane -------------------------------------------------------
    def pass1_device(self, bank, k, key_bits, log2w, counter_bits):
        from . import api

        self.dbank = api.DeviceBank(self.ctx, bank)
        self.cms = api.CountMinSketch(1 << log2w, self.ctx, counter_bits)
        self.cms.add_bank(self.dbank, k, key_bits)

    def sketch_tensor(self):
        """The sketch's u32 device counters as an int32 CUDA tensor (no copy)."""
        return self.cms.counts_tensor()

    def clamp(self):
        self.cms.clamp_counts()

    def owned_rows(self, bank, k, key_bits, target_solid_cov, world):
        """Pass 2 against the merged sketch; every accumulated row, grouped by owner
        rank, as a (n, key_bits/64 + 2) int64 CUDA tensor, and the rows per owner."""
        from . import api

        prev = self.ctx.get_tuning("acc_filter")
        self.ctx.set_tuning(acc_filter=0)  # the owners need every accumulated key
        try:
            t = api.solid_build(self.ctx, self.dbank, self.cms, k, target_solid_cov, key_bits=key_bits)
        finally:
            self.ctx.set_tuning(acc_filter=prev)
        rows, counts = t.export_acc_owned(world)
        t.release()
        return rows, counts

    def release(self):
        if self.cms is not None:
            self.cms.release()
            self.cms = None
        if self.dbank is not None:
            self.dbank.release()
            self.dbank = None

    # ---- host data plane (gloo tests; the oracle engine has the same three) --------

    def pass1(self, bank, k, key_bits, log2w, counter_bits):
        from . import api

        self.dbank = api.DeviceBank(self.ctx, bank)
        self.cms = api.CountMinSketch(1 << log2w, self.ctx, counter_bits)
        self.cms.add_bank(self.dbank, k, key_bits)
        return self.cms.export()

    def load(self, raw):
        self.cms.load(raw)

    def pass2(self, bank, k, key_bits, target_solid_cov):
        from . import api

        # the owners sum the ranks' accumulators: every accumulated key is needed, not
        # only those that may become solid in this rank's share
        prev = self.ctx.get_tuning("acc_filter")
        self.ctx.set_tuning(acc_filter=0)
        try:
            t = api.solid_build(self.ctx, self.dbank, self.cms, k, target_solid_cov, key_bits=key_bits)
        finally:
            self.ctx.set_tuning(acc_filter=prev)
        keys, cov, edges = t.export_acc(sort=False)
        t.release()
        self.cms.release()
        self.dbank.release()
        return keys, edges
