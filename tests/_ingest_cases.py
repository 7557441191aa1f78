"""Read pairs and FASTQ files for the ingest parity tests: random reads with
lowercase, N and planted adapter prefixes, and pairs overlapping by any amount,
including reads over 512 bases."""
import numpy as np


def rc(s: bytes) -> bytes:
    return s[::-1].translate(bytes.maketrans(b"ACGT", b"TGCA"))


def rand_read(rng, n):
    alphabet = np.frombuffer(b"ACGTACGTACGTacgtN", np.uint8)
    s = alphabet[rng.integers(0, alphabet.size, n)].tobytes()
    if rng.random() < 0.3 and n > 40:  # plant an adapter prefix, sometimes with a mismatch
        ad = [b"AGATCGGAAGAGC", b"AGATGTGTATAAGAGACAG", b"CTGTCTCTTATACACATCT"][rng.integers(0, 3)]
        at = int(rng.integers(max(0, n - 100), n - 10))
        ad = bytearray(ad[: n - at])
        if rng.random() < 0.5:
            ad[int(rng.integers(0, min(10, len(ad))))] = ord("N")
        s = s[:at] + bytes(ad) + s[at + len(ad):]
    return s[:n]


def write_fastq(path, reads, quals, mate):
    with open(path, "wb") as f:
        for i, (s, q) in enumerate(zip(reads, quals)):
            f.write(b"@r%d/%d\n%s\n+\n%s\n" % (i, mate, s, q))


def odd_pairs_fastq(r1, r2, seed, n_pairs):
    """n_pairs overlapping pairs cut from random fragments (a third up to 1500 bases),
    with one N in each R2, written as two FASTQ files."""
    rng = np.random.default_rng(seed)
    reads1, reads2, q1s, q2s = [], [], [], []
    for i in range(n_pairs):
        frag_len = int(rng.integers(20, 1500 if i % 3 == 0 else 400))
        frag = rand_read(rng, frag_len)
        l1, l2 = int(rng.integers(5, frag_len + 1)), int(rng.integers(5, frag_len + 1))
        reads1.append(frag[:l1])
        reads2.append(rc(frag[frag_len - l2:].upper().replace(b"N", b"A")).replace(b"T", b"N", 1))
        q1s.append(bytes(rng.integers(33, 75, l1).astype(np.uint8)))
        q2s.append(bytes(rng.integers(33, 75, l2).astype(np.uint8)))
    write_fastq(r1, reads1, q1s, 1)
    write_fastq(r2, reads2, q2s, 2)


OPTS = [dict(), dict(subsample_factor=0.4, seed=11), dict(enable_merge=False), dict(enable_trim=False, min_len=100),
        dict(min_qual=35, min_len=60)]
