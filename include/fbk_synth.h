/*
 * fbk_synth.h — seeded synthetic isolates for tests and benchmarks.
 *
 * Stands in for the reference's benchmark generator (src/bin/generate_benchmark.rs,
 * splitmix64-driven genome and reads) with the read model the benchmark
 * configurations name: GC-biased i.i.d. genome (GC draw as in
 * src/bin/experiment_a.rs:14-31), inserted near-identical repeat copies, an optional
 * tandem array, Normal(mean, sd) fragments, substitutions and indels, and Phred
 * qualities uniform in [q_lo, q_hi] with the last tail_len bases decaying to tail_q.
 * Every pair is generated from its own splitmix64 stream, so any range of pairs can
 * be produced independently and in parallel with identical results.
 */
#ifndef FBK_SYNTH_H
#define FBK_SYNTH_H

#include "fbk.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    uint64_t seed;
    uint64_t genome_len;
    double gc;
    uint32_t n_repeats;       /* inserted repeat copies */
    uint32_t repeat_len;
    double repeat_identity;   /* each copy keeps at least this identity to the unit */
    uint32_t tandem_copies;   /* tandem array copies (0 = none) */
    uint32_t tandem_unit;
    uint32_t read_len;
    uint32_t _pad;
    double coverage;          /* pairs = round(coverage * genome_len / (2 * read_len)) */
    double frag_mean, frag_sd;
    double sub_rate, indel_rate;
    uint32_t q_lo, q_hi, tail_len, tail_q;
} fbk_synth_params;

/* Defaults: 1 Mbp, GC 0.50, 150 bp pairs at 50x, fragments N(350, 30), 0.5%
 * substitutions, Phred 30-40 with the last 20 bases decaying to 15, seed 42. */
FBK_API void fbk_synth_defaults(fbk_synth_params* p);
FBK_API uint64_t fbk_synth_n_pairs(const fbk_synth_params* p);
/* ASCII genome of p->genome_len bases. */
FBK_API fbk_status fbk_synth_genome(const fbk_synth_params* p, uint8_t* out);
/* Pairs [first, first+n) as fixed-length records: r1/q1/r2/q2 each n*read_len bytes. */
FBK_API fbk_status fbk_synth_pairs(const fbk_synth_params* p, const uint8_t* genome, uint64_t first, uint64_t n, uint8_t* r1,
                                   uint8_t* q1, uint8_t* r2, uint8_t* q2);
/* Writes the isolate as two plain FASTQ files (@fbk_<i>/1, @fbk_<i>/2). */
FBK_API fbk_status fbk_synth_write_fastq(const fbk_synth_params* p, const char* r1_path, const char* r2_path);
/* Generates every pair and ingests it (trim_merge.rs ingest with the given settings,
 * subsample factor 1.0) into a host read bank, using `threads` CPU threads.  Also
 * returns count_fastx_exact's statistics of the raw reads and, when sample_pairs > 0,
 * a one-arena bank of the first sample_pairs raw pairs interleaved R1,R2 (the
 * estimator's input). */
FBK_API fbk_status fbk_synth_isolate(const fbk_synth_params* p, int threads, uint64_t min_len, uint32_t min_qual, int enable_trim,
                                     int enable_merge, fbk_hbank** bank, uint64_t sample_pairs, fbk_hbank** sample,
                                     fbk_count_stats* stats);

#ifdef __cplusplus
}
#endif
#endif /* FBK_SYNTH_H */
