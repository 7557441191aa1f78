/*
 * fbk.h — C ABI of the GB300 (sm_103a) k-mer counting front end for fastBact.
 *
 * Every entry point is `extern "C"`, takes plain pointers and sizes, and returns an
 * fbk_status (0 = FBK_OK).  fbk_last_error() gives the message of the most recent
 * failure on a context.  The caller owns every host buffer; the library owns device
 * objects until their *_release call.  Every object (bank, sketch, table) must be
 * released before the context it was created on is destroyed.  A context is used from one host thread at a
 * time; separate contexts are independent.  Each context owns one CUDA stream for its
 * work, and a second one for the asynchronous upload and export calls.
 *
 * Reference interfaces (paths inside the fastBact repository) that each group
 * replaces are cited next to the declarations.
 */
#ifndef FBK_H
#define FBK_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FBK_API __attribute__((visibility("default")))

typedef int fbk_status;
enum {
    FBK_OK = 0,
    FBK_ERR_INVALID = 1,     /* bad argument (size, k out of range, null pointer) */
    FBK_ERR_CUDA = 2,        /* CUDA runtime error; message in fbk_last_error */
    FBK_ERR_OOM = 3,         /* device pool or cudaMalloc exhausted */
    FBK_ERR_TABLE_FULL = 4,  /* solid table probe limit hit (retried internally first) */
    FBK_ERR_TIMEOUT = 5,     /* a bounded device wait gave up */
    FBK_ERR_IO = 6,          /* file open/read failure */
    FBK_ERR_FORMAT = 7,      /* malformed or desynchronised FASTQ */
    FBK_ERR_EMPTY = 8,       /* no valid read pairs */
    FBK_ERR_BUSY = 9,        /* admission refused: not enough free device memory / slots */
    FBK_ERR_NOT_READY = 10,  /* asynchronous work not finished yet */
    FBK_ERR_NO_DEVICE = 11   /* no CUDA device visible */
};

typedef struct fbk_ctx fbk_ctx;       /* device, stream, memory pool, status words */
typedef struct fbk_bank fbk_bank;     /* device-resident ReadBank */
typedef struct fbk_cms fbk_cms;       /* device-resident CountMinSketch */
typedef struct fbk_table fbk_table;   /* device-resident solid k-mer table */
typedef struct fbk_hll fbk_hll;       /* device-resident HyperLogLog */
typedef struct fbk_hbank fbk_hbank;   /* host-resident ReadBank (ingest output) */

/* One BitSeqArena (src/common/bitseq.rs:145-149): base i of the arena lives at bits
 * 2*(i%32) of data[i/32] (LSB first, A=0 C=1 G=2 T=3); offsets[id] is the arena base
 * index of sequence id, lengths[id] its length.  pair_idx (optional, may be NULL) is
 * the 0-based input pair each read came from, used by the subsampler. */
typedef struct {
    const uint64_t* data;
    uint64_t n_words;
    const uint64_t* offsets;
    const uint32_t* lengths;
    uint64_t n_seqs;
    const uint32_t* pair_idx;
} fbk_arena_view;

/* ExactCountStats — src/ingest/estimator.rs:34-51 */
typedef struct {
    uint64_t exact_read_pairs;
    uint64_t total_bases_r1;
    uint64_t total_bases_r2;
    uint64_t total_bases;
    uint64_t min_read_len;
    uint64_t max_read_len;
    double mean_read_len;
    uint64_t median_read_len;
} fbk_count_stats;

/* GenomeEstimate — src/ingest/estimator.rs:55-83 (kmers is the Vec<usize> ladder;
 * confidence: 0 High, 1 LowCoverageWarning, 2 Unreliable). */
typedef struct {
    uint64_t genome_size;
    uint64_t exact_read_pairs;
    uint64_t total_bases;
    uint64_t median_read_len;
    uint64_t max_read_len;
    double estimated_cov;
    double subsample_factor;
    uint64_t kmers[8];
    uint64_t n_kmers;
    int32_t confidence;
    int32_t _pad;
    uint64_t u_ge_1;
    uint64_t u_ge_2;
    double sample_kmer_depth;
    uint64_t pairs_sampled; /* pairs consumed before the sample loop ended */
    uint64_t m_sample;      /* k-mer occurrences in the consumed pairs */
} fbk_genome_estimate;

/* Estimator parameters.  fbk_estimator_defaults() fills the reference constants:
 * k = 21, CMS width 1<<23 nibbles, HLL p = 14, sample cap 150000 pairs,
 * checkpoints every 2000 pairs from 6000 (src/ingest/estimator.rs:299-375). */
typedef struct {
    uint32_t k;
    uint32_t cms_log2_width;
    uint32_t hll_p;          /* 14 (reference) or 16 */
    uint32_t _pad;
    uint64_t sample_cap;     /* 150000 */
    uint64_t max_pairs;      /* estimate_genome's max_pairs argument */
    double target_cov;       /* estimate_genome's target_cov argument */
} fbk_estimator_params;

/* Subsampler (src/ingest/trim_merge.rs:324-348): input pair i (1-based) is kept iff
 * factor >= 0.999 or splitmix64(i ^ seed) <= (u64)(factor * 2^64). */
typedef struct {
    double factor;
    uint64_t seed;
} fbk_subsample;

/* Front-end build parameters (src/graph/build.rs:67-328).  t_solid is the CMS gate
 * (target_solid_cov.unwrap_or(2)); min_trans_cov the per-edge mask threshold
 * (target_solid_cov or 3).  counter_bits 4 = reference nibble CMS, 16 = u16 CMS. */
typedef struct {
    uint32_t k;
    uint32_t key_bits;        /* 64 (k<=31), 128 (k<=63), 256 (k<=127) */
    uint32_t cms_log2_width;  /* 0 = width_for_genome_size(genome_size) */
    uint32_t counter_bits;    /* 4 or 16 */
    uint32_t t_solid;
    uint32_t min_trans_cov;
    uint32_t table_log2_cap;  /* 0 = sized from the pass-1 distinct-k-mer sketch */
    uint32_t _pad;
    uint64_t genome_size;     /* used when cms_log2_width == 0 (build.rs:74-84) */
} fbk_build_params;

/* ---- status, context ------------------------------------------------------- */
FBK_API const char* fbk_status_str(fbk_status s);
FBK_API const char* fbk_version(void);
/* pool_bytes = 0: objects are allocated one by one; > 0: carved from one pool. */
FBK_API fbk_status fbk_ctx_create(int device, uint64_t pool_bytes, fbk_ctx** out);
FBK_API fbk_status fbk_ctx_destroy(fbk_ctx* ctx);
/* A second context on the same device with its own stream, sharing the parent's
 * memory pool (work on the two streams may overlap).  Destroy forks before or after
 * the parent; the pool lives until its last context is destroyed. */
FBK_API fbk_status fbk_ctx_fork(fbk_ctx* parent, fbk_ctx** out);
/* Free bytes and the largest free block of the context's pool (device free memory
 * when the context has no pool). */
FBK_API fbk_status fbk_ctx_pool_free(const fbk_ctx* ctx, uint64_t* free_bytes, uint64_t* largest_block);
FBK_API fbk_status fbk_last_error(const fbk_ctx* ctx, char* buf, size_t len);
FBK_API fbk_status fbk_ctx_sync(fbk_ctx* ctx);
/* Kernel timing with CUDA events on the context's stream (off by default). */
FBK_API fbk_status fbk_ctx_set_timing(fbk_ctx* ctx, int enable);
/* Sum of event-timed milliseconds and launch count of kernels whose name starts
 * with `prefix` since the last reset ("" = all kernels). */
FBK_API fbk_status fbk_ctx_timing(fbk_ctx* ctx, const char* prefix, double* ms, uint64_t* launches);
FBK_API fbk_status fbk_ctx_timing_reset(fbk_ctx* ctx);
/* CUDA events on the context stream: record marker `slot` (0..15) now; elapsed
 * milliseconds between two recorded markers (waits for the later one). */
FBK_API fbk_status fbk_ctx_event_record(fbk_ctx* ctx, int slot);
FBK_API fbk_status fbk_ctx_event_elapsed(fbk_ctx* ctx, int slot_a, int slot_b, double* ms);
/* Launch and sizing parameters (the autotuner sets these): "sweep_bytes" (sketch
 * bytes per pass-1 / solidity sweep), "bucket_bytes" (table bytes per pass-2 record
 * bucket), "stripes", "load_factor", "pass2_mode" (1 buckets, 0 direct sweep),
 * "record_factor" (record capacity over the expected count; a full bucket falls back
 * to the direct sweep),
 * "block_pass1", "grid_pass1", "block_pass2", "grid_pass2", "block_emit" (blocks of
 * 32..256 threads in steps of 32; grid 0 = occupancy), "sketch_mode" (1: a build that does not return its
 * sketch keeps only a threshold-ladder gate; 0: counted sketch), "ladder_ilp" (1 or 2
 * windows per lane in the ladder pass 1, 3 = pipelined over chunks, 4 = one lane per read
 * with rolled k-mers, 5 = the same rolling two windows per step; 0 = by key width),
 * "emit_lookahead" (record emit with the gate loads 1 or 2 chunks ahead read by read,
 * 3 = 2 ahead over a flattened window stream, 4 = one lane per read with rolled k-mers
 * (the default), 5 = the same at two blocks per SM for every key width), "acc_filter"
 * (keys that cannot become SolidKmerNodes stay out of the table, see fbk_table_flags:
 * 0 never, 1 where it pays, 2 always), "upsert_all" (1: an unfiltered pass upserts every
 * bucket in one persistent launch), "upsert_queue" (1: filtered upserts queue the
 * filter's survivors per warp before probing), "filter_sizing" (1: a filtered pass sizes
 * its table from the first bucket's survivors, at load "filter_load"), "batch_pass1"
 * (0 autotuned, 1 one multi-isolate launch, 2 a launch per isolate).  Results do not
 * depend on any of them. */
FBK_API fbk_status fbk_ctx_set_tuning(fbk_ctx* ctx, const char* name, double value);
FBK_API fbk_status fbk_ctx_get_tuning(const fbk_ctx* ctx, const char* name, double* value);
/* Number of kernels launched on this context since creation. */
FBK_API fbk_status fbk_ctx_launch_count(const fbk_ctx* ctx, uint64_t* n);
FBK_API fbk_status fbk_ctx_mem_info(const fbk_ctx* ctx, uint64_t* pool_used, uint64_t* pool_size);

/* ---- read bank (ReadBank, src/common/bitseq.rs:350-399) ---------------------- */
/* arenas[0..3] = merged_reads, pe_forward, pe_reverse (iteration order of
 * build.rs:90).  Copies host data to the device (page-locked host memory is copied
 * asynchronously on the context stream; larger pageable buffers through pinned
 * staging, after which the host buffers may be reused at once). */
FBK_API fbk_status fbk_bank_upload(fbk_ctx* ctx, const fbk_arena_view arenas[3], fbk_bank** out);
/* The same, returning once the copies are queued when every arena buffer is
 * page-locked (else it copies as fbk_bank_upload does): the copies run on the
 * context's copy stream while the caller queues other work (the genome estimate of
 * the sample, say), and every call that reads the bank orders its work after them.
 * The host buffers must stay valid and unchanged until fbk_bank_wait returns or
 * the bank is released. */
FBK_API fbk_status fbk_bank_upload_async(fbk_ctx* ctx, const fbk_arena_view arenas[3], fbk_bank** out);
FBK_API fbk_status fbk_bank_wait(const fbk_bank* b);  /* blocks until an asynchronous upload's copies are done */
FBK_API fbk_status fbk_bank_info(const fbk_bank* b, uint64_t* n_reads, uint64_t* n_bases);
FBK_API fbk_status fbk_bank_release(fbk_bank* b);

/* ---- CountMinSketch (src/common/sketch.rs:121-253) -------------------------- */
FBK_API uint64_t fbk_cms_width_for_genome_size(uint64_t genome_size); /* sketch.rs:165-168 */
FBK_API fbk_status fbk_cms_create(fbk_ctx* ctx, uint32_t log2_width, uint32_t counter_bits, fbk_cms** out);
FBK_API fbk_status fbk_cms_clear(fbk_cms* c);
/* CountMinSketch::add over host keys (sketch.rs:191-223). */
FBK_API fbk_status fbk_cms_add_keys(fbk_cms* c, const uint64_t* keys, uint64_t n);
/* CountMinSketch::estimate over host keys (sketch.rs:227-246). */
FBK_API fbk_status fbk_cms_estimate_keys(fbk_cms* c, const uint64_t* keys, uint64_t n, uint32_t* out);
/* Pass 1 of build_cdbg_with_contigs_ext (build.rs:90-116): add the canonical
 * k-mer fold of every k-mer of every read with len >= k.  ss may be NULL. */
FBK_API fbk_status fbk_cms_add_bank(fbk_cms* c, const fbk_bank* b, uint32_t k, uint32_t key_bits, const fbk_subsample* ss);
/* Pass 1 in one call: a new sketch of 4 x 2^log2_width counters holding every k-mer
 * of the bank (fbk_cms_create + fbk_cms_add_bank; build.rs:74-116). */
FBK_API fbk_status fbk_cms_build(fbk_ctx* ctx, const fbk_bank* b, uint32_t k, uint32_t key_bits, uint32_t log2_width,
                                 uint32_t counter_bits, fbk_cms** out);
/* Prior contigs add x10 per k-mer (build.rs:118-138); ascii concatenated, offs has n+1 entries. */
FBK_API fbk_status fbk_cms_add_contigs(fbk_cms* c, const uint8_t* ascii, const uint64_t* offs, uint64_t n, uint32_t k, uint32_t key_bits);
/* Raw table in the reference byte layout (4*w/2 bytes, nibble) or 4*w u16 (LE). */
FBK_API fbk_status fbk_cms_nbytes(const fbk_cms* c, uint64_t* nbytes);
FBK_API fbk_status fbk_cms_export(fbk_cms* c, uint8_t* out, uint64_t nbytes);
/* dst = min(cap, dst + src) counter by counter: merging sketches of disjoint read
 * sets equals the sketch of their union. */
/* Replaces the counters with bytes in the fbk_cms_export layout, e.g. the merged
 * sketch of reads counted on several ranks (no counterpart in the reference). */
FBK_API fbk_status fbk_cms_import(fbk_cms* c, const uint8_t* in, uint64_t nbytes);
FBK_API fbk_status fbk_cms_merge(fbk_cms* dst, const fbk_cms* src);
/* The sketch's device counters — 4 rows of 2^log2_width u32 counts, row-major, each
 * at most 65535 between calls — so that a collective library can reduce them in place
 * (an all-reduce SUM over ranks that counted disjoint read shares: the merged gate is
 * exact, min(cap, sum of min(65535, a_r)) = min(cap, sum a_r)).  Synchronise the
 * context before handing the pointer to another stream; call fbk_cms_clamp_counts
 * after the reduction.  Replaces the CountMinSketch merge of build.rs:93-116 across
 * processes (no counterpart in the reference, which runs in one process). */
FBK_API fbk_status fbk_cms_counts_device(fbk_cms* c, uint32_t** counts, uint64_t* n);
FBK_API fbk_status fbk_cms_clamp_counts(fbk_cms* c);
FBK_API fbk_status fbk_cms_release(fbk_cms* c);

/* ---- HyperLogLog (src/common/sketch.rs:24-115) ------------------------------ */
FBK_API fbk_status fbk_hll_create(fbk_ctx* ctx, uint32_t p, fbk_hll** out);
FBK_API fbk_status fbk_hll_add_hashes(fbk_hll* h, const uint64_t* hashes, uint64_t n);           /* add_hash */
FBK_API fbk_status fbk_hll_add_canonical_hashes(fbk_hll* h, const uint64_t* hashes, uint64_t n); /* add_canonical_hash */
FBK_API fbk_status fbk_hll_merge(fbk_hll* dst, const fbk_hll* src);
FBK_API fbk_status fbk_hll_export(fbk_hll* h, uint8_t* regs, uint64_t n);
FBK_API fbk_status fbk_hll_estimate(fbk_hll* h, double* out);
FBK_API fbk_status fbk_hll_release(fbk_hll* h);
/* HyperLogLog::estimate over host registers (f64, register order). */
FBK_API double fbk_hll_estimate_registers(const uint8_t* regs, uint32_t p); /* NaN unless regs and 4 <= p <= 18 */

/* ---- ntHash (src/common/kmer.rs:385-477) --------------------------------------
 * Canonical ntHash of every window of length k of each read in the arena
 * (RollingNtHash::new + roll), computed on the device.  out has one entry per window,
 * reads in order; returns the number written in *n_out. */
FBK_API fbk_status fbk_nthash_arena(fbk_ctx* ctx, const fbk_arena_view* arena, uint32_t k, uint64_t* out, uint64_t cap, uint64_t* n_out);
/* Canonical k-mers (big-endian words, key_bits/64 per window) and is_rc flags of
 * every window of each read (RollingKmer::roll_next, kmer.rs:344-378). */
FBK_API fbk_status fbk_canonical_kmers_arena(fbk_ctx* ctx, const fbk_arena_view* arena, uint32_t k, uint32_t key_bits, uint64_t* out_words, uint8_t* out_is_rc, uint64_t cap, uint64_t* n_out);

/* ---- solid table (build.rs:141-328) ----------------------------------------- */
/* Pass 2 + conversion: CMS-gated transitions accumulated in an open-addressing
 * device table, then the SolidKmerNode conversion (mask, cov).  ss may be NULL. */
FBK_API fbk_status fbk_solid_build(fbk_ctx* ctx, const fbk_bank* b, const fbk_cms* cms, const fbk_build_params* p,
                                   const fbk_subsample* ss, const uint8_t* contig_ascii, const uint64_t* contig_offs,
                                   uint64_t n_contigs, fbk_table** out);
/* Passes 1 + 2 + conversion in one call: the front end of build_cdbg_with_contigs_ext
 * (build.rs:67-328).  cms_out (optional) keeps the pass-1 sketch alive. */
FBK_API fbk_status fbk_build_front(fbk_ctx* ctx, const fbk_bank* b, const fbk_build_params* p, const fbk_subsample* ss,
                                   const uint8_t* contig_ascii, const uint64_t* contig_offs, uint64_t n_contigs,
                                   fbk_table** out, fbk_cms** cms_out);
/* n_keys: accumulated keys; n_solid: SolidKmerNode entries (mask != 0). */
FBK_API fbk_status fbk_table_info(const fbk_table* t, uint64_t* n_keys, uint64_t* n_solid, uint64_t* capacity);
/* FBK_TABLE_ACC_FILTERED: the accumulator holds only the keys that may become
 * SolidKmerNodes.  A key's edge counter grows by at most one per window of the key,
 * so a key seen in fewer than min_trans_cov windows has an empty mask; with the
 * tuning acc_filter = 2 such keys are kept out of the table when the pass runs in one
 * read chunk without prior contigs; acc_filter = 1 (default) does so where the saving
 * outweighs the cost of counting: 256-bit keys, and passes whose distinct k-mers
 * exceed a fifth of their windows.  The SolidKmerNode rows, their
 * digest and fbk_table_pushes are unchanged; n_keys and fbk_table_export_acc cover
 * the kept keys only (each with its exact KmerAcc), a superset of the keys with
 * mask != 0.  Callers that need every accumulated key (e.g. to sum accumulators
 * across ranks) set acc_filter = 0. */
#define FBK_TABLE_ACC_FILTERED 1u
FBK_API fbk_status fbk_table_flags(const fbk_table* t, uint32_t* flags);
/* Converted entries in device order (unsorted): keys (key_bits/64 big-endian words
 * each), cov, mask.  cap = rows the buffers hold. */
FBK_API fbk_status fbk_table_export(fbk_table* t, uint64_t* keys, uint16_t* cov, uint8_t* mask, uint64_t cap, uint64_t* n_out);
/* The same into page-locked buffers, returning once the copies are queued on the
 * context's copy stream (n_out is known at once): the next build can start while the
 * rows travel.  The buffers hold the rows after fbk_table_export_wait; releasing the
 * table waits for the copies first. */
FBK_API fbk_status fbk_table_export_async(fbk_table* t, uint64_t* keys, uint16_t* cov, uint8_t* mask, uint64_t cap,
                                          uint64_t* n_out);
FBK_API fbk_status fbk_table_export_wait(fbk_table* t);
/* Every accumulated key with its KmerAcc (cov and edge_counts[8], saturated at 65535). */
FBK_API fbk_status fbk_table_export_acc(fbk_table* t, uint64_t* keys, uint16_t* cov, uint16_t* edges, uint64_t cap, uint64_t* n_out);
/* Sum over every key of its raw edge counters (= transition pushes made by pass 2,
 * weighted by the per-push increment); used for the algorithmic-bytes count. */
FBK_API fbk_status fbk_table_pushes(const fbk_table* t, uint64_t* pushes);
/* Order-independent digest of the converted entries (same formula as the oracle's). */
FBK_API fbk_status fbk_table_digest(fbk_table* t, uint64_t* digest, uint64_t* n_solid);
/* Order-independent digest of the whole accumulator — every key of the
 * FxHashMap<K, KmerAcc> shards with its cov and 8 edge counts (build.rs:145-196) — as
 * the sum mod 2^64 over keys of splitmix64(kd ^ splitmix64(v0 ^ splitmix64(v1 ^
 * splitmix64(e7)))), kd = the key's big-endian words folded through splitmix64,
 * v0 = cov | e0<<16 | e1<<32 | e2<<48, v1 = e3 | e4<<16 | e5<<32 | e6<<48.  Compares
 * accumulators of tens of millions of keys without exporting them.  For a table built
 * with the record filter (fbk_table_flags) it covers the kept keys only. */
FBK_API fbk_status fbk_table_acc_digest(fbk_table* t, uint64_t* digest, uint64_t* n_keys);
/* One isolate across ranks (the 64 FxHashMap shards of build.rs:141-196 partitioned by
 * rank instead of by mutex).  fbk_table_export_acc_owned writes every accumulated key
 * of a table into the DEVICE buffer rows (cap_rows rows of key_bits/64 + 2 u64 words:
 * the key's big-endian words, then the 8 edge counts as u16 fields, e0 | e1 << 16 |
 * e2 << 32 | e3 << 48 and e4 .. e7 likewise), grouped by owner rank
 * splitmix64(fold(key)) mod world, and the rows per owner into owner_counts[world]
 * (host).  fbk_table_from_acc_rows builds an owner's table from the rows it received
 * from every rank (DEVICE buffer; equal keys add up, capped at 65535 when read) and
 * converts it to SolidKmerNodes (build.rs:295-328). */
FBK_API fbk_status fbk_table_export_acc_owned(fbk_table* t, uint32_t world, uint64_t* rows, uint64_t cap_rows,
                                              uint64_t* owner_counts);
FBK_API fbk_status fbk_table_from_acc_rows(fbk_ctx* ctx, uint32_t k, uint32_t key_bits, uint32_t min_trans_cov,
                                           const uint64_t* rows, uint64_t n, fbk_table** out);
FBK_API fbk_status fbk_table_release(fbk_table* t);

/* ---- estimator (src/ingest/estimator.rs:104-440) ----------------------------- */
FBK_API void fbk_estimator_defaults(fbk_estimator_params* p);
/* Sample loop on the device + f64 post-math on the host.  sample holds raw (untrimmed)
 * reads interleaved R1,R2 per pair (2*n_pairs sequences); stats is count_fastx_exact
 * over the whole input.  regs_total / regs_solid (optional, 1<<p bytes) receive the
 * HLL registers at the point the sample loop stopped. */
FBK_API fbk_status fbk_estimate_sample(fbk_ctx* ctx, const fbk_arena_view* sample, uint64_t n_pairs,
                                       const fbk_count_stats* stats, const fbk_estimator_params* p,
                                       fbk_genome_estimate* out, uint8_t* regs_total, uint8_t* regs_solid);
/* Same as fbk_estimate_sample with the sample already resident: reads 0 .. 2*n_pairs-1
 * of `sample` are R1,R2 interleaved per pair; read_lengths is the host copy of their
 * lengths (used for the window bases and m_sample). */
FBK_API fbk_status fbk_estimate_bank(fbk_ctx* ctx, const fbk_bank* sample, const uint32_t* read_lengths, uint64_t n_pairs,
                                     const fbk_count_stats* stats, const fbk_estimator_params* p, fbk_genome_estimate* out,
                                     uint8_t* regs_total, uint8_t* regs_solid);
/* fbk_estimate_sample for callers that cannot allocate device memory: hosts whose
 * device memory belongs to another runtime's allocator (a service with its own pool,
 * a framework that reserved the GPU), and loops that must not take allocator locks
 * or the synchronisation a cudaFree can cause.  This entry point has no counterpart
 * in the reference.  It takes no context and allocates nothing: its scratch is one
 * fixed device array of FBK_NOALLOC_SCRATCH_BYTES that every GPU loading the library
 * holds until exit.  Limits: at most 20000 sampled pairs, 2^23 sample bases,
 * cms_log2_width <= 18, hll_p <= 14 — larger requests return FBK_ERR_INVALID with a
 * message in err, before anything is copied or launched.  The first call on a device
 * looks up the array's address (cudaGetSymbolAddress).  Calls share the array: each
 * clears what it reads, and calls whose GPU work overlaps race, so serialise them.
 * stream: a cudaStream_t (NULL = default).  The call blocks: it synchronises the
 * stream and finishes the estimate on the host, so it cannot be recorded into a CUDA
 * graph (on a capturing stream it fails and ends the capture). */
#define FBK_NOALLOC_SCRATCH_BYTES (8u << 20)
FBK_API fbk_status fbk_estimate_sample_noalloc(int device, void* stream, const fbk_arena_view* sample, uint64_t n_pairs,
                                               const fbk_count_stats* stats, const fbk_estimator_params* p,
                                               fbk_genome_estimate* out, uint8_t* regs_total, uint8_t* regs_solid,
                                               char* err, size_t errlen);
/* count_fastx_exact (estimator.rs:167-283), host-side FASTQ scan. */
FBK_API fbk_status fbk_count_fastx_exact(const char* r1, const char* r2, fbk_count_stats* out, char* err, size_t errlen);
/* estimate_genome (estimator.rs:286-440): FASTQ scan on the host, sample on the device. */
FBK_API fbk_status fbk_estimate_genome(fbk_ctx* ctx, const char* r1, const char* r2, uint64_t max_pairs, double target_cov,
                                       fbk_genome_estimate* out);
FBK_API int fbk_compute_dynamic_kmers(uint64_t median_len, int64_t target_max_k, uint64_t* out, int cap); /* estimator.rs:104-161 */

/* Sharded estimator: the sample loop of estimate_genome (estimator.rs:296-379) split
 * over ranks, one process per GPU, with the single-process result bit for bit.
 * Occurrence t (pairs in order, R1 then R2, windows in order) makes the estimate >= 2
 * exactly when every row's counter was touched by some t' < t, so:
 *   1. each rank runs fbk_est_shard_firstpos on its pair range [pair_begin, pair_end)
 *      (global occurrence indices) -> first[4 << cms_log2_width], the smallest t that
 *      touched each counter (0xFFFFFFFF if none); the caller all-reduces with MIN;
 *   2. each rank runs fbk_est_shard_segments with the merged array -> its HLL register
 *      maxima per checkpoint segment, regs[2][n_segs][1 << hll_p] (total, then solid;
 *      segment 0 = pairs 1..6000, segment j = pairs 6000+2000(j-1)+1 .. 6000+2000j);
 *      the caller all-reduces with MAX;
 *   3. fbk_est_shard_finish (host only, no device) takes the merged registers, walks the
 *      checkpoints (early stop at lambda >= 15) and runs the post-math.
 * Every rank holds the whole sample (reads 0 .. 2*n_use-1 of `sample`, R1,R2
 * interleaved) and its read lengths; fbk_est_shard_plan gives n_use (the pairs the
 * sample loop can read) and n_segs. */
FBK_API fbk_status fbk_est_shard_plan(const uint32_t* read_lengths, uint64_t n_pairs, const fbk_count_stats* stats,
                                      const fbk_estimator_params* p, uint64_t* n_use, uint32_t* n_segs);
FBK_API fbk_status fbk_est_shard_firstpos(fbk_ctx* ctx, const fbk_bank* sample, const uint32_t* read_lengths, uint64_t n_use,
                                          uint64_t pair_begin, uint64_t pair_end, const fbk_estimator_params* p,
                                          uint32_t* first);
FBK_API fbk_status fbk_est_shard_segments(fbk_ctx* ctx, const fbk_bank* sample, const uint32_t* read_lengths, uint64_t n_use,
                                          uint64_t pair_begin, uint64_t pair_end, const fbk_estimator_params* p,
                                          const uint32_t* first, uint8_t* regs);
FBK_API fbk_status fbk_est_shard_finish(const uint32_t* read_lengths, uint64_t n_use, const fbk_count_stats* stats,
                                        const fbk_estimator_params* p, const uint8_t* regs, fbk_genome_estimate* out,
                                        uint8_t* regs_total, uint8_t* regs_solid);

/* ---- subsampler (trim_merge.rs:324-348) -------------------------------------- */
/* Bit i of keep_bits (host, ceil(n_pairs/64) words) = input pair i (0-based) kept. */
FBK_API fbk_status fbk_subsample_mask(fbk_ctx* ctx, uint64_t n_pairs, const fbk_subsample* ss, uint64_t* keep_bits);

/* ---- unitig compaction (build.rs:330-594) ------------------------------------------
 * Compacts a converted solid table into unitigs: boundary walks on the device (one
 * thread per boundary out-edge; a unitig reachable from both ends is kept from the end
 * with the smaller (row, direction, edge), the set the reference's visited marks
 * keep), isolated cycles and the k / k-1 overlap edges on the host.  Sequences are
 * min(seq, reverse complement) for linear unitigs; a cycle starts at one of its
 * k-mers (the reference starts at the first one its map order meets).  Coverage =
 * mean node coverage of the walk without its last node, as build.rs:379-435 computes
 * it. */
typedef struct fbk_unitigs fbk_unitigs;
FBK_API fbk_status fbk_compact(fbk_table* t, fbk_unitigs** out);
FBK_API fbk_status fbk_unitigs_info(const fbk_unitigs* u, uint64_t* n_unitigs, uint64_t* total_bases, uint64_t* n_edges);
/* ascii: total_bases bytes (may be NULL), offsets: n_unitigs + 1, cov and circular:
 * n_unitigs each (may be NULL). */
FBK_API fbk_status fbk_unitigs_export(const fbk_unitigs* u, uint8_t* ascii, uint64_t* offsets, float* cov, uint8_t* circular);
/* 6 u32 per edge: from unitig, from side (0 forward strand, 1 reverse), to unitig, to
 * reverse (0/1), overlap, support (cdbg.rs:113-122 merges repeats). */
FBK_API fbk_status fbk_unitigs_edges(const fbk_unitigs* u, uint32_t* edges, uint64_t cap, uint64_t* n_out);
FBK_API fbk_status fbk_unitigs_release(fbk_unitigs* u);

/* filter_active_reads (src/graph/local_multik.rs:259-333), the multi-k upgrade's input
 * filter: keep_out gets one byte per read of the bank, in bank order (merged,
 * pe_forward, pe_reverse): merged reads are kept when active, a pair (pe_forward[i],
 * pe_reverse[i], i < min of the two arena sizes) when either read is.  The unitigs are
 * the graph's sequences (ASCII, offsets: n_unitigs + 1), circular flags and the number
 * of edges on each side (edges_fwd.len(), edges_rev.len()); graph_k is the graph's k. */
FBK_API fbk_status fbk_filter_active_reads(fbk_ctx* ctx, const fbk_bank* bank, const uint8_t* unitig_ascii,
                                           const uint64_t* unitig_offsets, const uint8_t* circular, const uint32_t* edges_fwd,
                                           const uint32_t* edges_rev, uint64_t n_unitigs, uint32_t graph_k, uint8_t* keep_out,
                                           uint64_t* n_kept);

/* index_terminal_kmers (src/resolve/mapper.rs:89-136): canonical k-mers folded to u64
 * (KmerInt::to_u64) of the first and last 1000 k-mers of every unitig (all of them when
 * it has at most 2000), those occurring exactly once, with their unitig, strand
 * (DirUnitigId is_rc) and k-mer position; sorted by key.  Fills up to cap entries and
 * returns the total in n_out (call with cap 0 to size the outputs). */
FBK_API fbk_status fbk_index_terminal_kmers(fbk_ctx* ctx, const uint8_t* unitig_ascii, const uint64_t* unitig_offsets,
                                            uint64_t n_unitigs, uint32_t k, uint32_t key_bits, uint64_t* keys, uint32_t* unitig,
                                            uint8_t* is_rc, uint32_t* pos, uint64_t cap, uint64_t* n_out);

/* Subsampling policy of the pipeline driver (src/main.rs:76-180): decides the
 * subsample factor from an estimate.  reason: 0 EXPLICIT_NO_SUBSAMPLE_FLAG,
 * 1 EXPLICIT_GENOME_SIZE_ZERO_INVALID, 2 AUTO_SUBSAMPLE_EXPLICIT_GENOME_SIZE,
 * 3 AUTO_SUBSAMPLE_EXPLICIT_GENOME_SIZE_WITHIN_TARGET, 4 AUTO_SUBSAMPLE_HIGH_CONFIDENCE,
 * 5 AUTO_SUBSAMPLE_HIGH_CONFIDENCE_WITHIN_TARGET, 6 AUTO_SUBSAMPLE_INTERCEPTED_LOW_COVERAGE_WARNING,
 * 7 AUTO_SUBSAMPLE_INTERCEPTED_UNRELIABLE, 8 GENOME_SIZE_PRIOR_PROVIDED_SUBSAMPLING_NOT_ENABLED,
 * 9 DISABLED_BY_DEFAULT_SAFE_FALLBACK.  An invalid threshold ratio (not finite or
 * below 1) is FBK_ERR_INVALID, as main.rs:76-81 bails. */
typedef struct {
    int32_t no_subsample;           /* --no-subsample */
    int32_t enable_auto_subsample;  /* --enable-auto-subsample */
    int32_t has_genome_size;        /* --genome-size given */
    int32_t _pad;
    uint64_t genome_size;           /* its value */
    double depth;                   /* --depth (120 by default) */
    double threshold_ratio;         /* --subsample-threshold-ratio (1.5 by default) */
} fbk_subsample_policy;
FBK_API void fbk_subsample_policy_defaults(fbk_subsample_policy* p);
FBK_API fbk_status fbk_subsample_decide(const fbk_subsample_policy* p, const fbk_genome_estimate* e, double* factor,
                                        int32_t* reason);

/* ---- batches: many isolates per launch ------------------------------------------
 * The reference runs one isolate per process (src/main.rs: estimate_genome, the
 * subsampling policy, ingest, then build_cdbg per k).  A batch runs those counting
 * stages for many isolates at once; it has no counterpart in the reference.  Per
 * isolate it computes exactly what the single-isolate calls compute
 * (fbk_estimate_bank, fbk_subsample_decide, fbk_build_front with the batch's k,
 * sketch width and thresholds); the sketches, bitmaps, tables and record buckets
 * are carved from the context's pool, and each phase is one launch over every
 * isolate of a wave (optionally one CUDA graph per phase).  Waves are sized by the
 * free pool memory.  A batch belongs to one context and one host thread. */
typedef struct fbk_batch fbk_batch;
typedef struct {
    uint32_t k;               /* 31 */
    uint32_t key_bits;        /* 64 */
    uint32_t cms_log2_width;  /* 22 */
    uint32_t counter_bits;    /* 16 */
    uint32_t t_solid;         /* 2: target_solid_cov.unwrap_or(2) */
    uint32_t min_trans_cov;   /* 3 */
    uint32_t use_graphs;      /* 1: each phase of a wave runs as one CUDA graph */
    uint32_t autotune;        /* 1: launch shapes chosen by timing candidates on the first wave */
    uint32_t keep_sketch;     /* 1: keep each isolate's sketch until the batch is released */
    uint32_t max_wave;        /* isolates per wave (<= 256) */
    uint64_t est_max_pairs;   /* estimate_genome's max_pairs: 250000 (main.rs:65) */
    uint64_t subsample_seed;  /* --subsample-seed: 0 */
    uint64_t max_wave_bytes;  /* 0: all free pool memory */
    fbk_subsample_policy policy;
} fbk_batch_params;

typedef struct {
    int32_t state;            /* 0 queued, 1 estimated, 2 counted, 3 done, -1 failed */
    int32_t subsample_reason;
    int32_t fallback;         /* 1: redone by the single-isolate path (bucket or table overflow) */
    int32_t wave;
    double subsample_factor;
    fbk_genome_estimate estimate;
    uint64_t n_keys, n_solid, digest, pushes;
    uint64_t kmers;           /* k-mer occurrences of pass 1 + pass 2 (kept reads) */
    uint64_t table_capacity;
    fbk_status status;        /* error of a failed isolate */
    int32_t _pad;
} fbk_batch_result;

typedef struct {
    uint64_t isolates_done, waves, fallbacks, graph_launches, kernel_launches;
    double ms_estimate, ms_phase_a, ms_phase_b, ms_host;   /* device time (events) and host planning */
    /* launch shapes in use: block, grid (0 = occupancy), and sketch rows per sweep
     * (pass1_rows 0: the ladder pass 1 runs as one single-isolate launch per isolate) */
    int32_t pass1_block, pass1_grid, pass1_rows, solid_block, solid_grid, solid_rows;
    int32_t emit_block, emit_grid, upsert_block, upsert_grid;
    int32_t tuned;
    int32_t emit_form;  /* record emit in use: 3 flat window stream, 4 one lane per read (rolled) */
    double tune_ms;
} fbk_batch_stats;

FBK_API void fbk_batch_defaults(fbk_batch_params* p);
FBK_API fbk_status fbk_batch_create(fbk_ctx* ctx, const fbk_batch_params* p, fbk_batch** out);
/* Uploads one isolate: its ReadBank (3 arenas, pair indices needed for subsampling),
 * the raw sample pairs for the estimator (R1,R2 interleaved, sample_pairs pairs) and
 * its count_fastx_exact statistics.  The host buffers may be reused on return. */
FBK_API fbk_status fbk_batch_submit(fbk_batch* b, const fbk_arena_view bank[3], const fbk_arena_view* sample, uint64_t sample_pairs,
                                    const fbk_count_stats* stats, uint64_t* id);
/* Counts every submitted isolate that is not done yet; returns when all are done. */
FBK_API fbk_status fbk_batch_run(fbk_batch* b);
FBK_API fbk_status fbk_batch_get_result(const fbk_batch* b, uint64_t id, fbk_batch_result* out);
/* Hands the isolate's solid table to the caller (release with fbk_table_release). */
FBK_API fbk_status fbk_batch_take_table(fbk_batch* b, uint64_t id, fbk_table** out);
/* Frees the isolate's device state (reads, sketch, table if not taken). */
FBK_API fbk_status fbk_batch_drop(fbk_batch* b, uint64_t id);
FBK_API fbk_status fbk_batch_get_stats(const fbk_batch* b, fbk_batch_stats* out);
FBK_API fbk_status fbk_batch_release(fbk_batch* b);

/* ---- serving: a request loop with continuous batching ----------------------------
 * No counterpart in the reference (one isolate per process).  A request is one
 * isolate (reads, raw sample pairs, count statistics); the server computes for it
 * exactly what a batch does.  Admission: a request enters when the reserved device
 * bytes of all admitted requests plus its own estimate (reads, sketch, bitmap,
 * solid table and record buckets; replaced by the exact sizes after pass 1) fit
 * the budget.  Continuous batching: each worker (its own stream on the shared pool)
 * takes every admitted request waiting for the same stage as one wave, so requests
 * that arrive while others run join the next wave and waves of different stages
 * overlap on the device.  Finished tables stay on the device (their bytes stay
 * reserved) until the caller takes or releases them.  Calls may come from any
 * host thread. */
typedef struct fbk_server fbk_server;
typedef struct {
    fbk_batch_params batch;   /* counting parameters of every request */
    uint32_t workers;         /* concurrent waves, one stream each: 2 */
    uint32_t _pad;
    uint64_t budget_bytes;    /* admission budget; 0: 90% of the pool (of free memory without a pool) */
} fbk_server_params;
/* Request states: 0 queued, 1 admitted (reads being uploaded), 2 estimated (reads on
 * the device, host buffers no longer used), 3 counted (pass 1 done), 4 done (table
 * ready), 5 drained (table taken or released), -1 failed. */
typedef struct {
    int32_t state;
    int32_t status;           /* fbk_status of a failed request */
    double t_submit_ms, t_admit_ms, t_done_ms;   /* server clock: ms since fbk_server_create */
    double t_uploaded_ms, t_estimated_ms, t_counted_ms;  /* stage ends: reads on the device, estimate, pass 1 */
    uint64_t reserved_bytes;
    fbk_batch_result result;
} fbk_request_info;
typedef struct {
    uint64_t submitted, done, failed, waves_a, waves_b, isolates_a, isolates_b;
    uint64_t reserved_bytes, peak_reserved_bytes, budget_bytes;
    uint64_t peak_in_flight;  /* most requests admitted and not yet done */
    double busy_ms;           /* summed worker time inside waves */
    double ms_estimate, ms_phase_a, ms_phase_b;  /* summed device time of the workers' stages */
} fbk_server_stats;

FBK_API void fbk_server_defaults(fbk_server_params* p);
FBK_API fbk_status fbk_server_create(fbk_ctx* ctx, const fbk_server_params* p, fbk_server** out);
/* Queues one isolate.  The host buffers must stay valid until the request's state is
 * 2 or more (or -1). */
FBK_API fbk_status fbk_server_submit(fbk_server* s, const fbk_arena_view bank[3], const fbk_arena_view* sample,
                                     uint64_t sample_pairs, const fbk_count_stats* stats, uint64_t* id);
FBK_API fbk_status fbk_server_poll(fbk_server* s, uint64_t id, fbk_request_info* out);
/* Waits until the request is done or failed; FBK_ERR_NOT_READY after timeout_ms
 * (NaN or <= 0: no wait; values above 1e12, infinity included, count as 1e12). */
FBK_API fbk_status fbk_server_wait(fbk_server* s, uint64_t id, double timeout_ms, fbk_request_info* out);
/* Hands a done request's table to the caller (release it with fbk_table_release before
 * destroying the context) and frees the request's remaining device state. */
FBK_API fbk_status fbk_server_take_table(fbk_server* s, uint64_t id, fbk_table** out);
FBK_API fbk_status fbk_server_release_request(fbk_server* s, uint64_t id);
FBK_API fbk_status fbk_server_get_stats(fbk_server* s, fbk_server_stats* out);
/* Finishes in-flight waves, fails queued requests, frees all request state. */
FBK_API fbk_status fbk_server_destroy(fbk_server* s);

/* ---- device ingest: FASTQ text to a device bank (trim_merge.rs:307-417) ------------
 * The same reads, trimming, merging, subsampling and arena layout as fbk_ingest_fastq,
 * computed on the device from the two files' bytes (plain 4-line FASTQ records; a '\r'
 * before a newline is dropped; blank lines between records are refused with
 * FBK_ERR_FORMAT — the host ingest reads those).  IngestStats: trim_merge.rs:270-290. */
typedef struct {
    uint64_t input_read_pairs, retained_read_pairs, bases_before_trim, bases_after_trim;
    uint64_t merged_pairs_count, merged_bases, unmerged_pairs_count;
} fbk_ingest_stats;
FBK_API fbk_status fbk_ingest_fastq_device(fbk_ctx* ctx, const uint8_t* r1, uint64_t r1_len, const uint8_t* r2, uint64_t r2_len,
                                           double subsample_factor, uint64_t min_len, uint32_t min_qual, int enable_trim,
                                           int enable_merge, uint64_t seed, fbk_bank** out, fbk_ingest_stats* stats);
/* A device bank back on the host: words (fbk_bank_words of them), bank-global base offsets, lengths, pair indices (n_reads each; any pointer may be NULL). */
FBK_API fbk_status fbk_bank_export(const fbk_bank* b, uint64_t* words, uint64_t* offsets, uint32_t* lengths, uint32_t* pair_idx);
/* Reads per arena (merged, pe_forward, pe_reverse) and words of a bank. */
FBK_API fbk_status fbk_bank_arena_counts(const fbk_bank* b, uint64_t* counts3);
FBK_API fbk_status fbk_bank_words(const fbk_bank* b, uint64_t* n_words);

/* ---- host ingest (trim_merge.rs:17-417), CPU side ----------------------------- */
FBK_API fbk_status fbk_ingest_fastq(const char* r1, const char* r2, double subsample_factor, uint64_t min_len, uint32_t min_qual,
                                    int enable_trim, int enable_merge, uint64_t seed, fbk_hbank** out, char* err, size_t errlen);
FBK_API fbk_status fbk_hbank_arena(const fbk_hbank* hb, int arena, fbk_arena_view* view);
FBK_API fbk_status fbk_hbank_stats(const fbk_hbank* hb, uint64_t* input_pairs, uint64_t* retained_pairs, uint64_t* merged_pairs,
                                   uint64_t* unmerged_pairs, uint64_t* bases_before_trim, uint64_t* bases_after_trim);
FBK_API void fbk_hbank_free(fbk_hbank* hb);
/* Single-pair helpers exposed for their known-answer tests.  fbk_trim_adapter returns
 * the kept length; fbk_trim_quality the kept length or -1 (read dropped, or no quality
 * string); fbk_merge_read_pair the merged length (merged_out holds l1 + l2 bytes) or -1
 * (no acceptable overlap, or a missing buffer). */
FBK_API uint64_t fbk_trim_adapter(const uint8_t* seq, uint64_t len);
FBK_API int64_t fbk_trim_quality(const uint8_t* seq, const uint8_t* qual, uint64_t len, uint32_t min_qual, uint64_t min_len);
FBK_API int64_t fbk_merge_read_pair(const uint8_t* r1, const uint8_t* q1, uint64_t l1, const uint8_t* r2, const uint8_t* q2,
                                    uint64_t l2, uint64_t min_overlap, double max_mismatch_ratio, uint8_t* merged_out,
                                    uint64_t* overlap_len, uint64_t* mismatches);

#ifdef __cplusplus
}
#endif
#endif /* FBK_H */
