"""Synthetic isolate cohorts for batches and serving.

A cohort member i is drawn from a splitmix64 stream seeded with first_seed + i:
genome size uniform in [2, 7] Mbp, GC uniform in [0.30, 0.68], depth uniform in
[30, 200]x; reads as in the single-isolate workload (PE150, fragments N(350, 30),
0.5% substitutions, Phred 30-40 decaying to 15 over the last 20 bases).  Isolates
above 150x are subsampled to 110x by the pipeline driver's policy
(src/main.rs:84-180 with --enable-auto-subsample --depth 110 and a trigger ratio of
150/110)."""
from __future__ import annotations

import time
from dataclasses import dataclass

from . import api

M64 = (1 << 64) - 1
GOLDEN = 0x9E3779B97F4A7C15


def _stream(seed: int):
    x = seed & M64
    while True:
        x = (x + GOLDEN) & M64
        yield api.splitmix64(x) >> 11


def draw(seed: int, scale: float = 1.0) -> dict:
    """Genome length, GC and depth of the cohort member with this seed; `scale`
    multiplies the genome length (smaller cohorts for quick runs)."""
    s = _stream(seed)
    u = [next(s) * (1.0 / (1 << 53)) for _ in range(3)]
    genome = int((2_000_000 + u[0] * 5_000_000) * scale)
    gc = 0.30 + u[1] * 0.38
    depth = 30.0 + u[2] * 170.0
    return dict(seed=seed, genome_len=max(genome, 20_000), gc=gc, coverage=depth)


POLICY = dict(enable_auto_subsample=True, depth=110.0, threshold_ratio=150.0 / 110.0)


def policy():
    return api.subsample_policy(**POLICY)


@dataclass
class Member:
    params: dict
    bank: api.ReadBank
    ingest: api.IngestStats
    sample: api.BitSeqArena
    sample_pairs: int
    stats: api.ExactCountStats
    gen_s: float


def make(n: int, first_seed: int = 1000, scale: float = 1.0, threads: int = 0, sample_pairs: int = 150_000) -> list[Member]:
    """Generates and ingests n cohort members (host side)."""
    out = []
    for i in range(n):
        d = draw(first_seed + i, scale)
        t0 = time.time()
        bank, st, sample, n_sample, cs = api.synth_isolate(api.synth_params(**d), threads=threads, sample_pairs=sample_pairs)
        out.append(Member(d, bank, st, sample, n_sample, cs, time.time() - t0))
    return out
