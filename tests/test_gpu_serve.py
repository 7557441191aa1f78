"""Serving: requests that arrive while others are on the device are admitted as the
memory budget allows, share waves with them, and every result is the same alone and
in the mix (integer results: tolerance exact, 0), and the same as the single-isolate
path (estimate, src/main.rs subsampling policy, build front end)."""
import threading
import time

import numpy as np
import pytest

from fastbact_gb300 import api

pytestmark = pytest.mark.gpu

SPECS = [  # seed, genome length, depth, GC
    (2000, 30_000, 40.0, 0.40),
    (2001, 60_000, 190.0, 0.60),   # subsampled to 110x
    (2002, 20_000, 80.0, 0.50),
    (2003, 45_000, 120.0, 0.33),
    (2004, 25_000, 160.0, 0.66),   # subsampled to 110x
    (2005, 35_000, 60.0, 0.45),
]
POLICY = dict(enable_auto_subsample=True, depth=110.0, threshold_ratio=150.0 / 110.0)
K, LOG2W = 31, 18


@pytest.fixture(scope="module")
def isolates():
    return [api.synth_isolate(api.synth_params(seed=s, genome_len=g, coverage=c, gc=gc), threads=0, sample_pairs=150_000)
            for s, g, c, gc in SPECS]


@pytest.fixture(scope="module")
def pctx():
    c = api.Context(0, pool_bytes=6 << 30)
    yield c
    c.close()


def single(ctx, iso):
    bank, _, sample, n_sample, cs = iso
    est, _, _ = api.estimate_sample(ctx, sample, n_sample, cs, max_pairs=250_000, target_cov=110.0)
    f, _ = api.subsample_decide(api.subsample_policy(**POLICY), est)
    t = api.build_cdbg_ext(bank, K, None, ctx=ctx, key_bits=64, counter_bits=16, cms_log2_width=LOG2W, subsample=(f, 0))
    out = (t.digest(), t.export(sort=True))
    t.release()
    return out


@pytest.fixture(scope="module")
def expected(pctx, isolates):
    return [single(pctx, iso) for iso in isolates]


def server(ctx, **kw):
    return api.Server(ctx, api.server_params(policy=api.subsample_policy(**POLICY), k=K, cms_log2_width=LOG2W, **kw))


def drain(srv, i):
    info = srv.wait(i)
    assert info.state == 4, info.state
    t = srv.take_table(i)
    out = (t.digest(), t.export(sort=True))
    t.release()
    return info, out


def same(a, b):
    assert a[0] == b[0]
    for x, y in zip(a[1], b[1]):
        assert np.array_equal(x, y)


def test_alone_and_in_the_mix_are_identical(pctx, isolates, expected):
    srv = server(pctx, workers=2)
    # alone
    alone = {}
    for j in (1, 3):
        bank, _, sample, n, cs = isolates[j]
        _, alone[j] = drain(srv, srv.submit(bank, sample, n, cs))
        same(alone[j], expected[j])
    # in the mix: arrivals from another thread at short random gaps, so that some
    # come while earlier ones are on the device
    ids = {}
    rng = np.random.default_rng(7)

    def arrivals():
        for j in rng.permutation(len(isolates)):
            bank, _, sample, n, cs = isolates[j]
            ids[int(j)] = srv.submit(bank, sample, n, cs)
            time.sleep(float(rng.exponential(0.01)))

    th = threading.Thread(target=arrivals)
    th.start()
    th.join()
    got = {j: drain(srv, i) for j, i in ids.items()}
    for j in (1, 3):
        same(got[j][1], alone[j])
    for j, (info, out) in got.items():
        same(out, expected[j])
        assert info.t_done_ms >= info.t_admit_ms >= info.t_submit_ms
    st = srv.stats()
    assert st.done == 2 + len(isolates) and st.failed == 0
    assert st.reserved_bytes == 0
    srv.release()


def test_burst_shares_waves(pctx, isolates, expected):
    srv = server(pctx, workers=2)
    ids = [srv.submit(bank, sample, n, cs) for bank, _, sample, n, cs in isolates]
    outs = [drain(srv, i)[1] for i in ids]
    for o, e in zip(outs, expected):
        same(o, e)
    st = srv.stats()
    # continuous batching: queued requests were admitted together, not one by one
    assert st.waves_a < len(isolates) and st.isolates_a == len(isolates)
    assert st.peak_in_flight >= 2
    srv.release()


def test_tight_budget_admits_one_at_a_time(pctx, isolates, expected):
    # a budget below any single request: each runs alone, in arrival order
    srv = server(pctx, workers=2, budget_bytes=1 << 20)
    ids = [srv.submit(bank, sample, n, cs) for bank, _, sample, n, cs in isolates[:4]]
    infos = []
    for i, e in zip(ids, expected[:4]):
        info, out = drain(srv, i)
        same(out, e)
        infos.append(info)
    st = srv.stats()
    assert st.peak_in_flight == 1 and st.waves_a == 4
    admits = [x.t_admit_ms for x in infos]
    assert admits == sorted(admits)
    srv.release()


def test_tables_stay_resident_until_taken(pctx, isolates):
    srv = server(pctx, workers=1)
    bank, _, sample, n, cs = isolates[2]
    i = srv.submit(bank, sample, n, cs)
    info = srv.wait(i)
    assert info.state == 4 and info.reserved_bytes > 0
    assert srv.stats().reserved_bytes == info.reserved_bytes
    srv.release_request(i)
    assert srv.stats().reserved_bytes == 0
    with pytest.raises(Exception):
        srv.take_table(i)
    srv.release()
