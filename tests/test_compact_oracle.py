"""The compaction oracle (build.rs:330-594 restated) against the reference's own
verification gate, build.rs:604-687: reads with 1% errors from a 10 kb circular
genome holding one 200 bp repeat twice compact, at solidity 5, into exactly three
unitigs (the repeat and the two flanks)."""
import numpy as np

from fastbact_gb300 import _native as N
from fastbact_gb300 import api
from oracle import orc

M64 = (1 << 64) - 1


def smix(z):
    z &= M64
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & M64
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & M64
    return z ^ (z >> 31)


def gate_reads():
    """The read set of build.rs:604-687, generated by the same rules."""
    alphabet = b"ACGT"

    def gen(seed, n):
        return bytes(alphabet[smix(seed + i) % 4] for i in range(n))

    rep = gen(0x1111_2222_3333_4444, 200)
    f1 = gen(0x5555_6666_7777_8888, 4800)
    f2 = gen(0x9999_AAAA_BBBB_CCCC, 4800)
    genome = rep + f1 + rep + f2
    assert len(genome) == 10_000
    reads, rng = [], 0xFEEDBEEF
    for i in range(len(genome) * 40 // 150):
        rng = smix((rng + i) & M64)
        start = rng % len(genome)
        r = bytearray()
        for j in range(150):
            base = genome[(start + j) % len(genome)]
            if smix(rng ^ j) % 100 == 0:
                alt = 1 + smix((rng + j * 31) & M64) % 3
                base = alphabet[(alphabet.index(base) + alt) % 4]
            r.append(base)
        reads.append(bytes(r))
    return reads


def gate_width(n_bases):
    # build.rs:74-84 with genome_size None: max(bases / 60, 50 kb) -> for_genome_size
    return int(N.lib().fbk_cms_width_for_genome_size(max(n_bases // 60, 50_000)))


def test_three_unitig_gate_oracle():
    reads = gate_reads()
    bank = api.ReadBank(merged_reads=api.BitSeqArena.from_seqs(reads))
    log2w = gate_width(sum(map(len, reads))).bit_length() - 1
    _, tab, _, mtc = orc.build_front(bank, 31, 64, log2w, 4, 5, threads=2)
    keys, cov, mask = tab.export_solid(mtc)
    seqs, ucov, circ, edges = orc.compact(keys, cov, mask, 31, 64)
    assert len(seqs) == 3, [len(s) for s in seqs]
    assert not circ.any()
    # the flanks (4.8 kb + the repeat's boundary k-mers) and the repeat, linked by overlaps
    lens = sorted(len(s) for s in seqs)
    assert lens[0] < 300 and lens[1] > 4000 and lens[2] > 4000
    assert len(edges) > 0
