"""One isolate counted across ranks with the device data plane (fastbact_gb300.shard,
DeviceEngine), on one GPU: the ranks are threads of this process, each with its own
library context and stream, and the collectives are carried out on the same CUDA
tensors NCCL would receive — the sketch counters reduced in place (all-reduce SUM),
the owner-grouped accumulator rows exchanged (all-to-all), the digests summed.  No
kernel waits on another rank's kernel: the ranks meet only at host barriers between
launches.  The result must equal the oracle counting every read in one process
(build.rs:84-328): the merged sketch bytes, the union of the owners' SolidKmerNode
rows and the digest."""
import threading

import numpy as np
import pytest

from fastbact_gb300 import api, shard
from oracle import orc

pytestmark = pytest.mark.gpu


class ThreadComm:
    """The exchange's collectives among `world` threads (one rank each)."""

    def __init__(self, world):
        self.world = world
        self.barrier = threading.Barrier(world, timeout=120)
        self.slots = [None] * world
        self.result = None

    def rank(self, r):
        return _RankComm(self, r)


class _RankComm:
    def __init__(self, shared, rank):
        self.s, self.rank = shared, rank

    def all_reduce_sum_(self, t):
        import torch

        s = self.s
        s.slots[self.rank] = t
        s.barrier.wait()
        if self.rank == 0:
            s.result = torch.stack([x.to(torch.int64) for x in s.slots]).sum(0)
        s.barrier.wait()
        t.copy_(s.result.to(t.dtype))
        torch.cuda.synchronize()
        s.barrier.wait()

    def all_to_all_rows(self, rows, send_counts):
        import torch

        s = self.s
        off = np.concatenate([[0], np.cumsum(send_counts)]).astype(np.int64)
        s.slots[self.rank] = (rows, off)
        s.barrier.wait()
        parts = [s.slots[r][0][int(s.slots[r][1][self.rank]):int(s.slots[r][1][self.rank + 1])] for r in range(s.world)]
        got = torch.cat(parts) if parts else rows[:0]
        counts = [len(p_) for p_ in parts]
        torch.cuda.synchronize()
        s.barrier.wait()
        return got, counts

    def sum_u64(self, v):
        s = self.s
        s.slots[self.rank] = v
        s.barrier.wait()
        total = sum(s.slots) & ((1 << 64) - 1)
        s.barrier.wait()
        return total


@pytest.fixture(scope="module")
def isolate():
    p = api.synth_params(seed=78, genome_len=40_000, coverage=30.0, gc=0.55, n_repeats=2, repeat_len=1000,
                         sub_rate=0.01)
    return api.synth_isolate(p, threads=0, sample_pairs=0)[0]


@pytest.mark.parametrize("world", [2, 3])
@pytest.mark.parametrize("k,kb,cb,log2w,tsc", [(31, 64, 16, 14, None), (21, 64, 4, 13, None), (45, 128, 16, 14, 4),
                                               (77, 256, 4, 14, None), (101, 256, 16, 14, None)])
def test_device_sharded_build_equals_single_process(isolate, world, k, kb, cb, log2w, tsc):
    bank = isolate
    comm = ThreadComm(world)
    out, errors = [None] * world, []

    def run(rank):
        ctx = api.Context(0)
        try:
            out[rank] = shard.sharded_build(shard.DeviceEngine(ctx), bank, k, kb, log2w, cb, tsc, rank, world,
                                            comm=comm.rank(rank))
        except BaseException as e:  # noqa: BLE001 - reported below
            errors.append(e)
            comm.barrier.abort()
        finally:
            ctx.close()

    threads = [threading.Thread(target=run, args=(r,)) for r in range(world)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    assert not errors, errors
    o_cms, o_tab, _, mtc = orc.build_front(bank, k, kb, log2w, cb, tsc, threads=4)
    ref = api.sort_rows(*o_tab.export_solid(mtc))
    keys = np.concatenate([o[0][0] for o in out])
    cov = np.concatenate([o[0][1] for o in out])
    mask = np.concatenate([o[0][2] for o in out])
    got = api.sort_rows(keys, cov, mask)
    assert all(np.array_equal(a, b) for a, b in zip(got, ref))
    for o in out:
        assert np.array_equal(o[1], o_cms.export()), "merged sketch differs"
        assert o[2] == o_tab.digest(mtc)[0]
    # every owner holds only its own keys
    for r, o in enumerate(out):
        if len(o[0][0]):
            assert (shard.owner(o[0][0], world) == r).all()
