"""fastbact_gb300 — GB300 (sm_103a) k-mer counting front end for fastBact.

Device kernels behind a C ABI (include/fbk.h, fastbact_gb300/_lib/libfbk.so) with a
Python mirror of the reference's Rust interface in ``fastbact_gb300.api``.
"""
from .api import (  # noqa: F401
    BitSeqArena,
    Context,
    CountMinSketch,
    DeviceBank,
    ExactCountStats,
    GenomeEstimate,
    HyperLogLog,
    ReadBank,
    SolidTable,
    build_cdbg,
    build_cdbg_ext,
    build_cdbg_with_contigs,
    build_cdbg_with_contigs_ext,
    compute_dynamic_kmers,
    count_fastx_exact,
    estimate_genome,
    estimate_sample,
    ingest_reads_ext_with_seed,
    key_bits_for_k,
    solid_build,
    synth_isolate,
    synth_params,
)

__version__ = "0.1.0"
