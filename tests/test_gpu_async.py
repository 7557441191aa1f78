"""Asynchronous upload and export (fbk_bank_upload_async, fbk_table_export_async): a
bank copied from page-locked arrays on the copy stream while other work is queued, and
rows copied out while the next build runs, give exactly the results of the synchronous
calls; pageable arrays fall back to the synchronous copy; a table released with its
export in flight waits for it."""
import numpy as np
import pytest

from fastbact_gb300 import _native as N
from fastbact_gb300 import api

pytestmark = pytest.mark.gpu


def pinned(a: np.ndarray, keep: list) -> np.ndarray:
    import torch

    t = torch.empty(max(a.nbytes, 8), dtype=torch.uint8, pin_memory=True)
    keep.append(t)
    out = t.numpy().view(a.dtype)[: a.size].reshape(a.shape)
    out[...] = a
    return out


def pinned_bank(bank: api.ReadBank, keep: list) -> api.ReadBank:
    arenas = []
    for a in bank.arenas:
        arenas.append(api.BitSeqArena(pinned(a.data, keep), pinned(a.offsets, keep), pinned(a.lengths, keep),
                                      pinned(a.pair_idx, keep) if a.pair_idx is not None else None))
    return api.ReadBank(*arenas)


@pytest.fixture(scope="module")
def isolate():
    p = api.synth_params(seed=515, genome_len=80_000, coverage=40.0, gc=0.45, n_repeats=2, repeat_len=1500,
                         sub_rate=0.01)
    return api.synth_isolate(p, threads=0, sample_pairs=0)[0]


@pytest.mark.parametrize("k", [21, 33, 77])
def test_async_upload_and_export_match_sync(ctx, isolate, k):
    keep = []
    ref_bank = api.DeviceBank(ctx, isolate)
    ref = api.build_cdbg_ext(ref_bank, k, None, ctx=ctx, cms_log2_width=16)
    ref_rows = ref.export(sort=True)
    ref_digest = ref.digest()
    ref.release()
    ref_bank.release()

    pb = pinned_bank(isolate, keep)
    db = api.DeviceBank(ctx, pb, async_upload=True)
    assert (db.n_reads, db.n_bases) == (isolate.total_reads(), isolate.total_bases())
    t = api.build_cdbg_ext(db, k, None, ctx=ctx, cms_log2_width=16)
    n_solid = t.info()[1]
    out = (pinned(np.zeros((n_solid, t.nw), np.uint64), keep), pinned(np.zeros(n_solid, np.uint16), keep),
           pinned(np.zeros(n_solid, np.uint8), keep))
    t.export_async(out)
    # a second build on the same bank runs while the rows are copied out
    t2 = api.build_cdbg_ext(db, k, None, ctx=ctx, cms_log2_width=16)
    rows = api.sort_rows(*t.export_wait())
    assert all(np.array_equal(a, b) for a, b in zip(rows, ref_rows))
    assert t.digest() == ref_digest and t2.digest() == ref_digest
    t.release()
    t2.release()
    db.release()


def test_async_export_released_in_flight(ctx, isolate):
    keep = []
    db = api.DeviceBank(ctx, isolate)
    t = api.build_cdbg_ext(db, 31, None, ctx=ctx, cms_log2_width=16)
    n_solid = t.info()[1]
    ref = t.export(sort=True)
    out = (pinned(np.zeros((n_solid, t.nw), np.uint64), keep), pinned(np.zeros(n_solid, np.uint16), keep),
           pinned(np.zeros(n_solid, np.uint8), keep))
    t.export_async(out)
    t.release()  # waits for the copies before the rows' device memory goes back to the pool
    got = api.sort_rows(out[0][:n_solid], out[1][:n_solid], out[2][:n_solid])
    assert all(np.array_equal(a, b) for a, b in zip(got, ref))
    db.release()


def test_async_upload_of_pageable_arrays_copies_synchronously(ctx, isolate):
    db = api.DeviceBank(ctx, isolate, async_upload=True)  # numpy arrays: pageable
    ref = api.DeviceBank(ctx, isolate)
    a, b = db.export(), ref.export()
    assert all(np.array_equal(x, y) for x, y in zip(a[:4], b[:4])) and a[4] == b[4]
    db.release()
    ref.release()


def test_async_export_needs_page_locked_buffers(ctx, isolate):
    db = api.DeviceBank(ctx, isolate)
    t = api.build_cdbg_ext(db, 31, None, ctx=ctx, cms_log2_width=16)
    n_solid = t.info()[1]
    out = (np.zeros((n_solid, t.nw), np.uint64), np.zeros(n_solid, np.uint16), np.zeros(n_solid, np.uint8))
    with pytest.raises(N.FbkError, match="page-locked"):
        t.export_async(out)
    t.release()
    db.release()
