"""The seeded single-isolate workloads the benchmark measures and the full-size parity
tests check, in one place so that both run exactly the same inputs.

Each entry gives the generator parameters (fbk_synth_params fields), the k values of
its build passes, the Count-Min Sketch width (log2 columns per row, u16 counters)
and the estimator's HyperLogLog precision.  Reads are 150 bp pairs with fragments
N(350, 30) and Phred 30-40 decaying to 15 over the last 20 bases (generator
defaults); ingest trims and merges them into the read bank with min_len 30 and
min_qual 20 (src/main.rs:215-224).
"""
from __future__ import annotations

# Plain method, CPU-runnable: 1 Mbp at GC 0.50, 50x (~167k pairs), 0.5% substitutions,
# k = 31 (64-bit keys), CMS 4 x 2^22 u16, HLL p = 14, solid threshold count >= 3.
PLAIN_1MBP = dict(
    gen=dict(seed=42, genome_len=1_000_000, gc=0.50, coverage=50.0, sub_rate=0.005, indel_rate=0.0),
    ks=[31], cms_log2w=22, hll_p=14,
    text="plain 1 Mbp: GC 0.50, PE150 50x (167k pairs), N(350,30) fragments, 0.5% subs, Phred tail decay; "
         "k=31 (64-bit), CMS 4 x 2^22 u16, HLL p=14, count>=3",
)

# Plain method at isolate scale: 5 Mbp at GC 0.51 with seven inserted 5 kb repeat
# copies at >= 99% identity, 100x (1.67M pairs); multi-k pass at k = 21, 33, 55 and
# 77.  k = 33 and 55 need 128-bit keys and k = 77 256-bit keys: the reference sends
# every k above 63 to [u64; 4] (src/main.rs:350-363).
ISOLATE_5MBP = dict(
    gen=dict(seed=43, genome_len=5_000_000, gc=0.51, n_repeats=7, repeat_len=5000, repeat_identity=0.99,
             coverage=100.0, sub_rate=0.005, indel_rate=0.0),
    ks=[21, 33, 55, 77], cms_log2w=24, hll_p=14,
    text="isolate-scale plain method: 5 Mbp genome GC 0.51, 7x5 kb repeats >=99% id, PE150 100x (1.67M pairs), "
         "N(350,30) fragments, 0.5% subs, Phred tail decay; multi-k 21,33,55 (64/128-bit) + 77 (256-bit); "
         "CMS 4 x 2^24 u16; HLL p=14",
)

# Stress: 12 Mbp at GC 0.66 with ten 5 kb repeat copies and a 200 x 60 bp tandem
# array, 300x with 1% substitutions and 0.05% indels; k = 127 (256-bit keys) on the
# full input and after subsampling to 110x; CMS 4 x 2^26 u16; HLL p = 16.
STRESS_12MBP = dict(
    gen=dict(seed=46, genome_len=12_000_000, gc=0.66, n_repeats=10, repeat_len=5000, repeat_identity=0.99,
             tandem_copies=200, tandem_unit=60, coverage=300.0, sub_rate=0.01, indel_rate=0.0005),
    ks=[127], cms_log2w=26, hll_p=16,
    text="stress: 12 Mbp GC 0.66, 10 x 5 kb repeats, 200 x 60 bp tandem array, PE150 300x, 1% subs, 0.05% indels; "
         "k=127 (256-bit), CMS 4 x 2^26 u16, HLL p=16",
)

# The pipeline driver's subsampling to 110x above 150x (src/main.rs:84-180 with
# --enable-auto-subsample --depth 110 --subsample-threshold-ratio 150/110).
SUBSAMPLE_110X = dict(enable_auto_subsample=True, depth=110.0, threshold_ratio=150.0 / 110.0)

# estimate_genome's arguments in the pipeline (src/main.rs:65)
EST_MAX_PAIRS = 250_000
EST_TARGET_COV = 110.0


def generate(wl: dict, rank: int = 0, coverage_scale: float = 1.0, sample_pairs: int = 150_000):
    """Generates and ingests the workload (rank r > 0 shifts the seed by 1000 r, an
    independent isolate per rank).  Returns (params, bank, ingest stats, raw sample
    arena, sample pairs, ExactCountStats)."""
    from . import api

    g = dict(wl["gen"])
    g["seed"] += 1000 * rank
    g["coverage"] *= coverage_scale
    p = api.synth_params(**g)
    bank, st, sample, n_sample, stats = api.synth_isolate(p, threads=0, sample_pairs=sample_pairs)
    return p, bank, st, sample, n_sample, stats
