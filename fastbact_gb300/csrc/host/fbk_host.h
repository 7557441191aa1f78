// fbk_host.h — host-only (CPU) pieces of the library: FASTQ reading, exact pair
// counting, adapter/quality trimming, pair merging and the host read bank.
#pragma once
#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>

#include "../../../include/fbk.h"

namespace fbk {

// ASCII_TO_2BIT — src/common/bitseq.rs:67-81 (non-ACGT -> A)
inline uint8_t ascii_2bit(uint8_t c) {
    switch (c) {
        case 'C': case 'c': return 1;
        case 'G': case 'g': return 2;
        case 'T': case 't': return 3;
        default: return 0;
    }
}

inline uint64_t splitmix64(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
    return z ^ (z >> 31);
}

// BitSeqArena (bitseq.rs:145-222) plus the input pair of each read.
struct HostArena {
    std::vector<uint64_t> data;
    std::vector<uint64_t> off;
    std::vector<uint32_t> len;
    std::vector<uint32_t> pair_idx;
    uint64_t n_bases = 0;
    void push_ascii(const uint8_t* s, uint64_t n, uint32_t pair);  // push_seq, bitseq.rs:195-222
    void push_codes(const uint8_t* c, uint64_t n, uint32_t pair);
    fbk_arena_view view() const;
    void clear() { data.clear(); off.clear(); len.clear(); pair_idx.clear(); n_bases = 0; }
};

// Plain 4-line FASTQ (the record forms needletail reads for these inputs).
class FastqReader {
  public:
    explicit FastqReader(const char* path);
    ~FastqReader();
    bool ok() const { return f_ != nullptr; }
    // 1 = record, 0 = end of input, -1 = malformed (err set)
    int next(std::string& err);
    std::string id, seq, qual;

  private:
    bool line(std::string& s);
    FILE* f_ = nullptr;
    std::vector<char> buf_;
    size_t pos_ = 0, end_ = 0;
    bool eof_ = false;
};

std::string read_id_prefix(const std::string& id);  // estimator.rs:89-99
fbk_status count_fastx_exact_impl(const char* r1, const char* r2, fbk_count_stats* out, std::string& err);

// Trim / merge (trim_merge.rs:17-238)
uint64_t trim_adapter_len(const uint8_t* seq, uint64_t len);
int64_t trim_quality_len(const uint8_t* seq, const uint8_t* qual, uint64_t len, uint64_t qual_len, uint32_t min_qual,
                         uint64_t min_len);
// Returns merged length or -1 when unmerged; merged bytes written to out (l1+l2 capacity).
int64_t merge_pair(const uint8_t* r1, const uint8_t* q1, uint64_t l1, uint64_t ql1, const uint8_t* r2, const uint8_t* q2,
                   uint64_t l2, uint64_t ql2, uint64_t min_overlap, double max_mismatch_ratio, uint8_t* out,
                   uint64_t* overlap_len, uint64_t* mismatches);

struct IngestStats {
    uint64_t input_read_pairs = 0, retained_read_pairs = 0, bases_before_trim = 0, bases_after_trim = 0,
             merged_pairs_count = 0, merged_bases = 0, unmerged_pairs_count = 0;
};

struct IngestParams {
    double subsample_factor = 1.0;
    uint64_t min_len = 30;
    uint32_t min_qual = 20;
    bool enable_trim = true, enable_merge = true;
    uint64_t seed = 0;
};

// Per-pair ingest step of ingest_reads_ext_with_seed (trim_merge.rs:327-399);
// pair_idx1 is the 1-based input pair number.  Appends to the three arenas.
struct PairIngester {
    IngestParams p;
    uint64_t keep_threshold = 0;
    bool should_subsample = false;
    std::vector<uint8_t> merged;
    explicit PairIngester(const IngestParams& pp);
    void ingest(uint64_t pair_idx1, const uint8_t* s1, const uint8_t* q1, uint64_t l1, uint64_t ql1, const uint8_t* s2,
                const uint8_t* q2, uint64_t l2, uint64_t ql2, HostArena* arenas, IngestStats& st);
};

}  // namespace fbk

struct fbk_hbank {
    fbk::HostArena a[3];  // merged, pe_forward, pe_reverse
    fbk::IngestStats stats;
};
