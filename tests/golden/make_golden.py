"""Generates tests/golden/golden.json from the oracle (the CPU restatement).

The reference publishes no hash / sketch / table vectors, so these fixtures are
the oracle's outputs on fixed inputs; the oracle itself is pinned by the
reference's own known-answer tests (tests/test_oracle_kat.py).  The fixtures let
the CPU suite detect any drift of the oracle and let the GPU suite compare the
device kernels with fixed numbers.  Inputs are small and deterministic:
LCG sequences as in the reference's tests and a seeded synthetic isolate.

Run:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import hashlib
import json
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from oracle import orc  # noqa: E402

M64 = (1 << 64) - 1
OUT = Path(__file__).resolve().parent / "golden.json"


def lcg_bases(seed: int, n: int) -> bytes:
    out, s = [], seed
    for _ in range(n):
        s = (s * 6364136223846793005 + 1442695040888963407) & M64
        out.append(b"ACGT"[s % 4])
    return bytes(out)


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def golden_sequences():
    return [lcg_bases(0xCAFEBABEDEADBEEF, 300), lcg_bases(0x123456789ABCDEF, 257),
            b"ACGTACGTACGTTTGCAACCGGTTACGT", b"A" * 64 + b"C" * 64, b"ACGTN" * 30]


def nthash_vectors(seqs, k):
    out = []
    for s in seqs:
        if len(s) < k:
            continue
        o = np.zeros(len(s) - k + 1, np.uint64)
        a = np.frombuffer(s, np.uint8).copy()
        orc.lib().orc_nthash_rolling_all(orc.p(a), len(s), k, orc.p(o))
        out.append(o)
    return np.concatenate(out)


def canon_vectors(seqs, k, kb):
    nw = kb // 64
    ks, rcs = [], []
    for s in seqs:
        if len(s) < k:
            continue
        n = len(s) - k + 1
        o = np.zeros(n * nw, np.uint64)
        r = np.zeros(n, np.uint8)
        a = np.frombuffer(s, np.uint8).copy()
        orc.lib().orc_rolling_canonicals(kb, orc.p(a), len(s), k, orc.p(o), orc.p(r))
        ks.append(o.reshape(n, nw))
        rcs.append(r)
    return np.concatenate(ks), np.concatenate(rcs)


def isolate():
    from fastbact_gb300 import api

    p = api.synth_params(seed=777, genome_len=20_000, coverage=25.0, n_repeats=2, repeat_len=800)
    return api.synth_isolate(p, threads=1, sample_pairs=150_000)


def main():
    seqs = golden_sequences()
    g = {"sequences": [s.decode() for s in seqs]}
    g["nthash_k21"] = [int(x) for x in nthash_vectors(seqs, 21)[:40]]
    g["nthash_k21_sha256"] = sha(nthash_vectors(seqs, 21))
    g["nthash_k15_sha256"] = sha(nthash_vectors(seqs, 15))
    for k, kb in [(21, 64), (31, 64), (55, 128), (99, 256), (127, 256)]:
        ks, rcs = canon_vectors(seqs, k, kb)
        g[f"canon_k{k}_sha256"] = sha(ks)
        g[f"canon_k{k}_rc_sha256"] = sha(rcs)
        g[f"canon_k{k}_first"] = [int(x) for x in ks[0]]
    keys = np.array([(i * 0x9E3779B97F4A7C15) & M64 for i in range(20000)], np.uint64)
    keys = np.concatenate([keys, np.repeat(keys[:64], 24)])
    for cb in (4, 16):
        c = orc.Cms(1 << 12, cb)
        c.add(keys)
        g[f"cms_{cb}_sha256"] = sha(c.export())
    h = orc.Hll(14)
    h.add_canonical_hash(keys)
    g["hll14_registers_sha256"] = sha(h.registers())
    g["hll14_estimate"] = h.estimate()

    bank, st, sample, n_sample, stats = isolate()
    g["isolate"] = {"reads": bank.total_reads(), "bases": bank.total_bases(), "data_sha256": [sha(a.data) for a in bank.arenas],
                    "lengths_sha256": [sha(a.lengths) for a in bank.arenas], "sample_sha256": sha(sample.data),
                    "n_sample": n_sample}
    reads = [sample.extract_ascii(i) for i in range(2 * n_sample)]
    rc, oe, rt, rs = orc.estimate_from_reads(reads, orc.count_stats(**stats.__dict__), 250_000, 110.0)
    assert rc == 0
    g["estimate"] = {"genome_size": oe.genome_size, "u_ge_1": oe.u_ge_1, "u_ge_2": oe.u_ge_2,
                     "estimated_cov": oe.estimated_cov, "subsample_factor": oe.subsample_factor,
                     "sample_kmer_depth": oe.sample_kmer_depth, "confidence": oe.confidence,
                     "pairs_sampled": oe.pairs_sampled, "m_sample": oe.m_sample,
                     "regs_total_sha256": sha(rt), "regs_solid_sha256": sha(rs)}
    builds = {}
    for k, kb, cb, tsc in [(31, 64, 4, None), (21, 64, 16, None), (33, 128, 4, None), (77, 256, 4, 4)]:
        cms, tab, ts, mtc = orc.build_front(bank, k, kb, 15, cb, tsc, threads=1)
        d, n = tab.digest(mtc)
        keys_, cov, edges = tab.export_acc()
        from fastbact_gb300.api import sort_rows

        keys_, cov, edges = sort_rows(keys_, cov, edges)
        builds[f"k{k}_b{kb}_c{cb}_t{tsc}"] = {"cms_sha256": sha(cms.export()), "n_keys": int(keys_.shape[0]),
                                              "n_solid": n, "digest": d, "acc_keys_sha256": sha(keys_),
                                              "acc_cov_sha256": sha(cov), "acc_edges_sha256": sha(edges)}
    g["builds"] = builds
    OUT.write_text(json.dumps(g, indent=1, sort_keys=True) + "\n")
    print(f"wrote {OUT} ({OUT.stat().st_size} bytes)")


if __name__ == "__main__":
    main()
