"""Counting one isolate across ranks (fastbact_gb300.shard) gives the single-process
result: world-size-2 process groups over gloo on the CPU, with the oracle as each
rank's counting engine (the device engine runs the same exchange code).  Checked:
the merged pass-1 sketch bytes, the SolidKmerNode rows (union of the owners' rows)
and the table digest, against the oracle counting every read in one process; and the
sharded genome-size estimator against the oracle's sequential sample loop
(estimator.rs:296-439)."""
import os
import socket

import numpy as np
import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

from fastbact_gb300 import api, shard
from oracle import orc


class OracleEngine:
    """The oracle as a rank's counting engine (build.rs:84-289 restated on the CPU)."""

    def pass1(self, bank, k, key_bits, log2w, counter_bits):
        self.cms = orc.Cms(1 << log2w, counter_bits)
        ar = orc.arenas3(bank)
        assert orc.lib().orc_build_pass1(ar, k, key_bits, self.cms.h, 2, None, None) == 0
        return self.cms.export()

    def load(self, raw):
        self.cms.load(raw)

    def pass2(self, bank, k, key_bits, target_solid_cov):
        ar = orc.arenas3(bank)
        t_solid = 2 if target_solid_cov is None else target_solid_cov
        h = orc.lib().orc_build_pass2(ar, k, key_bits, self.cms.h, t_solid, 2, None, None, None, None, 0)
        assert h
        keys, cov, edges = orc.Table(h, key_bits).export_acc()
        return keys, edges


CASES = [(31, 64, 16, 16, None), (21, 64, 4, 14, None), (45, 128, 16, 15, 4), (77, 256, 4, 14, None)]


def isolate():
    p = api.synth_params(seed=77, genome_len=20_000, coverage=25.0, gc=0.55, n_repeats=2, repeat_len=1000)
    return api.synth_isolate(p, threads=1, sample_pairs=0)[0]


def _rank_main(rank, world, port, q):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        bank = isolate()
        out = []
        for k, kb, cb, log2w, tsc in CASES:
            rows, merged, d = shard.sharded_build(OracleEngine(), bank, k, kb, log2w, cb, tsc, rank, world)
            gathered = [None] * world
            dist.all_gather_object(gathered, rows)
            out.append((gathered, merged, d))
        if rank == 0:
            q.put(out)
    finally:
        dist.destroy_process_group()


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


@pytest.mark.parametrize("world", [2])
def test_sharded_count_equals_single_process(world):
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    try:
        out = q.get(timeout=300)  # read before joining: a child cannot exit while its result fills the pipe
    finally:
        for p in procs:
            if p.is_alive():
                p.join(timeout=60)
    for p in procs:
        p.join(timeout=300)
        assert p.exitcode == 0
    bank = isolate()
    for (k, kb, cb, log2w, tsc), (gathered, merged, d) in zip(CASES, out):
        o_cms, o_tab, _, mtc = orc.build_front(bank, k, kb, log2w, cb, tsc, threads=2)
        assert np.array_equal(merged, o_cms.export()), (k, "merged sketch differs")
        keys = np.concatenate([g[0] for g in gathered])
        cov = np.concatenate([g[1] for g in gathered])
        mask = np.concatenate([g[2] for g in gathered])
        sk, sc, sm = api.sort_rows(keys, cov, mask)
        ok, oc, om = api.sort_rows(*o_tab.export_solid(mtc))
        assert len(sk) > 100
        assert np.array_equal(sk, ok) and np.array_equal(sc, oc) and np.array_equal(sm, om), k
        # every key has exactly one owner
        assert len(np.unique(sk, axis=0)) == len(sk)
        assert d == o_tab.digest(mtc)[0]



def _comm_rank_main(rank, world, port, q):
    """DistComm over gloo: the collectives the device data plane uses, on host tensors."""
    import torch

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        comm = shard.DistComm()
        assert not comm.on_device
        t = torch.arange(10, dtype=torch.int32) * (rank + 1)
        comm.all_reduce_sum_(t)
        # rank r sends r + 1 + d rows to rank d, each row (r, d, i)
        rows, counts = [], []
        for d in range(world):
            n = rank + 1 + d
            rows += [[rank, d, i] for i in range(n)]
            counts.append(n)
        got, recv = comm.all_to_all_rows(torch.tensor(rows, dtype=torch.int64), counts)
        s = comm.sum_u64((1 << 64) - 5 + rank)  # wraps mod 2^64
        q.put((rank, t.tolist(), got.tolist(), recv, s))
    finally:
        dist.destroy_process_group()


def test_dist_comm_collectives_over_gloo():
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_comm_rank_main, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    try:
        res = dict((r[0], r[1:]) for r in (q.get(timeout=300) for _ in range(world)))
    finally:
        for p in procs:
            p.join(timeout=120)
    for p in procs:
        assert p.exitcode == 0
    for rank in range(world):
        t, got, recv, s = res[rank]
        assert t == [3 * i for i in range(10)]  # (1 + 2) * i
        want = [[r, rank, i] for r in range(world) for i in range(r + 1 + rank)]
        assert got == want and recv == [r + 1 + rank for r in range(world)]
        assert s == (2 * ((1 << 64) - 5) + 1) % (1 << 64)


def test_owner_partition_is_balanced():
    keys = np.arange(1, 200_001, dtype=np.uint64).reshape(-1, 1) * np.uint64(0x9E3779B97F4A7C15)
    for world in (2, 3, 8):
        counts = np.bincount(shard.owner(keys, world), minlength=world)
        assert counts.min() > 0.9 * len(keys) / world


def test_capped_sum_identity():
    # min(cap, min(cap, a) + min(cap, b)) == min(cap, a + b) for positive counts
    rng = np.random.default_rng(3)
    a, b = rng.integers(0, 70000, 10000), rng.integers(0, 70000, 10000)
    for cap in (15, 65535):
        assert np.array_equal(np.minimum(cap, np.minimum(cap, a) + np.minimum(cap, b)), np.minimum(cap, a + b))


# ---------------------------------------------------------------------------
# sharded estimator
# ---------------------------------------------------------------------------
EST_PARAMS = dict(cms_log2_width=20)


class OracleEstimatorEngine:
    """The oracle's first-touch restatement of the sample loop on a rank's pairs."""

    def __init__(self, reads, k=21, cms_log2_width=16, hll_p=14):
        self.reads, self.k, self.w, self.p = reads, k, 1 << cms_log2_width, hll_p

    def firstpos(self, n_use, lo, hi):
        return orc.est_firstpos(self.reads, lo, hi, self.k, self.w)

    def segments(self, n_use, lo, hi, first):
        return orc.est_segments(self.reads, n_use, lo, hi, self.k, self.w, self.p, first)


def estimator_sample(genome_len, coverage, seed):
    p = api.synth_params(seed=seed, genome_len=genome_len, coverage=coverage, gc=0.5, sub_rate=0.005)
    _, _, sample, n_sample, cs = api.synth_isolate(p, threads=1, sample_pairs=150_000)
    reads = [sample.extract_ascii(i) for i in range(2 * n_sample)]
    return sample, n_sample, cs, reads


EST_CASES = [  # (genome, coverage, seed, max_pairs, hll_p)
    (60_000, 60.0, 5, 250_000, 14),    # stops at the first checkpoint
    (300_000, 30.0, 6, 250_000, 14),   # several checkpoints before the stop
    (300_000, 30.0, 6, 9_000, 16),     # sample cut before the stop, p = 16
    (300_000, 30.0, 6, 5_000, 14),     # no checkpoint at all
]


def sequential(reads, cs, max_pairs, hll_p):
    return orc.estimate_from_reads(reads, orc.count_stats(**cs.__dict__), max_pairs, 110.0,
                                   cms_width=1 << EST_PARAMS["cms_log2_width"], hll_p=hll_p)


def assert_same_estimate(ge, rt, rs, oracle_out):
    rc, oe, ort, ors = oracle_out
    assert rc == 0
    for f in ("genome_size", "u_ge_1", "u_ge_2", "pairs_sampled", "m_sample", "estimated_cov", "subsample_factor",
              "sample_kmer_depth"):
        assert getattr(ge, f) == getattr(oe, f), f
    assert np.array_equal(rt, ort) and np.array_equal(rs, ors)


@pytest.mark.parametrize("world", [1, 3])
def test_estimator_stages_merge_to_the_sequential_loop(world):
    """The merge steps done in one process (MIN of first-touch arrays, MAX of segment
    registers) reproduce the reference's sequential sample loop, for uneven splits."""
    for genome, cov, seed, max_pairs, hll_p in EST_CASES:
        sample, n_sample, cs, reads = estimator_sample(genome, cov, seed)
        params = dict(EST_PARAMS, hll_p=hll_p, max_pairs=max_pairs, target_cov=110.0)
        lengths = sample.lengths[:2 * n_sample]
        n_use, n_segs = api.est_shard_plan(lengths, n_sample, cs, **params)
        eng = OracleEstimatorEngine(reads, cms_log2_width=EST_PARAMS["cms_log2_width"], hll_p=hll_p)
        ranges = [shard.pair_range(n_use, r, world) for r in range(world)]
        first = np.minimum.reduce([eng.firstpos(n_use, lo, hi) for lo, hi in ranges])
        regs = np.maximum.reduce([eng.segments(n_use, lo, hi, first) for lo, hi in ranges])
        assert regs.size == 2 * n_segs << hll_p
        ge, rt, rs = api.est_shard_finish(lengths, n_use, cs, regs, **params)
        assert_same_estimate(ge, rt, rs, sequential(reads, cs, max_pairs, hll_p))


def _est_rank_main(rank, world, port, q):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        out = []
        for genome, cov, seed, max_pairs, hll_p in EST_CASES[:2]:
            sample, n_sample, cs, reads = estimator_sample(genome, cov, seed)
            params = dict(EST_PARAMS, hll_p=hll_p, max_pairs=max_pairs, target_cov=110.0)
            eng = OracleEstimatorEngine(reads, cms_log2_width=EST_PARAMS["cms_log2_width"], hll_p=hll_p)
            ge, rt, rs = shard.sharded_estimate(eng, sample.lengths[:2 * n_sample], n_sample, cs, rank, world, **params)
            out.append((ge, rt, rs))
        gathered = [None] * world
        dist.all_gather_object(gathered, out)
        if rank == 0:
            q.put(gathered)
    finally:
        dist.destroy_process_group()


def test_sharded_estimate_equals_single_process():
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_est_rank_main, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    try:
        gathered = q.get(timeout=300)
    finally:
        for p in procs:
            if p.is_alive():
                p.join(timeout=60)
    for p in procs:
        p.join(timeout=300)
        assert p.exitcode == 0
    for i, (genome, cov, seed, max_pairs, hll_p) in enumerate(EST_CASES[:2]):
        _, n_sample, cs, reads = estimator_sample(genome, cov, seed)
        want = sequential(reads, cs, max_pairs, hll_p)
        for r in range(world):  # every rank holds the same estimate
            assert_same_estimate(*gathered[r][i], want)
