// fbk_ingest.cpp — CPU side of ingest: FASTQ reading, count_fastx_exact,
// adapter/quality trimming, FLASH-style pair merging and the host read bank.
// These produce the ReadBank that the device kernels count; they follow
// src/ingest/trim_merge.rs and src/ingest/estimator.rs:167-283 line by line in
// behaviour (messages included) but are not on the device hot path.
#include <algorithm>
#include <cstring>
#include <memory>

#include "fbk_host.h"

namespace fbk {

// ---------------------------------------------------------------------------
// host arena — push_seq (bitseq.rs:195-222)
// ---------------------------------------------------------------------------
void HostArena::push_codes(const uint8_t* c, uint64_t n, uint32_t pair) {
    off.push_back(n_bases);
    len.push_back((uint32_t)n);
    pair_idx.push_back(pair);
    if (n == 0) return;
    const uint64_t end = n_bases + n;
    const uint64_t need = (end + 31) / 32;
    if (data.size() < need) data.resize(need, 0);
    uint64_t g = n_bases;
    for (uint64_t i = 0; i < n; ++i, ++g) data[g >> 5] |= (uint64_t)(c[i] & 3) << ((g & 31) << 1);
    n_bases = end;
}

void HostArena::push_ascii(const uint8_t* s, uint64_t n, uint32_t pair) {
    off.push_back(n_bases);
    len.push_back((uint32_t)n);
    pair_idx.push_back(pair);
    if (n == 0) return;
    const uint64_t end = n_bases + n;
    const uint64_t need = (end + 31) / 32;
    if (data.size() < need) data.resize(need, 0);
    uint64_t g = n_bases;
    for (uint64_t i = 0; i < n; ++i, ++g) data[g >> 5] |= (uint64_t)ascii_2bit(s[i]) << ((g & 31) << 1);
    n_bases = end;
}

fbk_arena_view HostArena::view() const {
    fbk_arena_view v;
    v.data = data.data();
    v.n_words = data.size();
    v.offsets = off.data();
    v.lengths = len.data();
    v.n_seqs = off.size();
    v.pair_idx = pair_idx.empty() ? nullptr : pair_idx.data();
    return v;
}

// ---------------------------------------------------------------------------
// FASTQ reader
// ---------------------------------------------------------------------------
FastqReader::FastqReader(const char* path) : buf_(1 << 20) { f_ = fopen(path, "rb"); }
FastqReader::~FastqReader() {
    if (f_) fclose(f_);
}

bool FastqReader::line(std::string& s) {
    s.clear();
    bool any = false;
    for (;;) {
        if (pos_ == end_) {
            if (eof_) break;
            end_ = fread(buf_.data(), 1, buf_.size(), f_);
            pos_ = 0;
            if (end_ == 0) {
                eof_ = true;
                break;
            }
        }
        const char* b = buf_.data() + pos_;
        const char* nl = (const char*)memchr(b, '\n', end_ - pos_);
        any = true;
        if (nl) {
            s.append(b, nl - b);
            pos_ += (nl - b) + 1;
            break;
        }
        s.append(b, end_ - pos_);
        pos_ = end_;
    }
    if (!s.empty() && s.back() == '\r') s.pop_back();
    return any;
}

int FastqReader::next(std::string& err) {
    for (;;) {
        if (!line(id)) return 0;
        if (!id.empty()) break;
    }
    if (id[0] != '@') {
        err = "expected '@' at the start of a FASTQ record";
        return -1;
    }
    std::string plus;
    if (!line(seq)) { err = "truncated FASTQ record (missing sequence line)"; return -1; }
    if (!line(plus) || plus.empty() || plus[0] != '+') { err = "truncated FASTQ record (missing '+' line)"; return -1; }
    if (!line(qual)) { err = "truncated FASTQ record (missing quality line)"; return -1; }
    if (qual.size() != seq.size()) { err = "sequence and quality lengths differ"; return -1; }
    id.erase(0, 1);
    return 1;
}

std::string read_id_prefix(const std::string& id) {
    size_t ws = id.size();
    for (size_t i = 0; i < id.size(); ++i) {
        const char c = id[i];
        if (c == ' ' || c == '\t' || c == '\n' || c == '\r' || c == '\f') { ws = i; break; }
    }
    std::string s = id.substr(0, ws);
    if (s.size() >= 2 && s[s.size() - 2] == '/' && (s.back() == '1' || s.back() == '2')) s.resize(s.size() - 2);
    return s;
}

// count_fastx_exact — estimator.rs:167-283
fbk_status count_fastx_exact_impl(const char* r1, const char* r2, fbk_count_stats* out, std::string& err) {
    FastqReader a(r1), b(r2);
    if (!a.ok()) { err = std::string("Failed to open file \"") + r1 + "\""; return FBK_ERR_IO; }
    if (!b.ok()) { err = std::string("Failed to open file \"") + r2 + "\""; return FBK_ERR_IO; }
    uint64_t pairs = 0, tb1 = 0, tb2 = 0, mn = UINT64_MAX, mx = 0;
    std::vector<uint64_t> hist(4096, 0), overflow;
    std::string e1, e2;
    char msg[1024];
    for (;;) {
        const int x = a.next(e1), y = b.next(e2);
        if (x == 1 && y == 1) {
            pairs++;
            if (read_id_prefix(a.id) != read_id_prefix(b.id)) {
                snprintf(msg, sizeof msg,
                         "FASTQ paired-end synchronization error at pair #%llu: R1 ID '\"%s\"' does not match R2 ID '\"%s\"'",
                         (unsigned long long)pairs, a.id.c_str(), b.id.c_str());
                err = msg;
                return FBK_ERR_FORMAT;
            }
            const uint64_t l1 = a.seq.size(), l2 = b.seq.size();
            tb1 += l1;
            tb2 += l2;
            mn = std::min(mn, std::min(l1, l2));
            mx = std::max(mx, std::max(l1, l2));
            if (l1 < 4096) hist[l1]++; else overflow.push_back(l1);
            if (l2 < 4096) hist[l2]++; else overflow.push_back(l2);
        } else if (x == 0 && y == 0) {
            break;
        } else if (x == 1 && y == 0) {
            snprintf(msg, sizeof msg, "FASTQ pairing mismatch: R1 has more reads than R2 (R2 ended prematurely after %llu pairs)",
                     (unsigned long long)pairs);
            err = msg;
            return FBK_ERR_FORMAT;
        } else if (x == 0 && y == 1) {
            snprintf(msg, sizeof msg, "FASTQ pairing mismatch: R2 has more reads than R1 (R1 ended prematurely after %llu pairs)",
                     (unsigned long long)pairs);
            err = msg;
            return FBK_ERR_FORMAT;
        } else if (x < 0) {
            snprintf(msg, sizeof msg, "Corrupted/truncated FASTQ record in R1 at pair #%llu: %s", (unsigned long long)(pairs + 1),
                     e1.c_str());
            err = msg;
            return FBK_ERR_FORMAT;
        } else {
            snprintf(msg, sizeof msg, "Corrupted/truncated FASTQ record in R2 at pair #%llu: %s", (unsigned long long)(pairs + 1),
                     e2.c_str());
            err = msg;
            return FBK_ERR_FORMAT;
        }
    }
    if (pairs == 0) {
        err = "Input FASTQ files contain 0 valid read pairs";
        return FBK_ERR_EMPTY;
    }
    const uint64_t total = tb1 + tb2, reads = pairs * 2, target = (reads + 1) / 2;
    uint64_t cum = 0, med = 0;
    for (uint64_t l = 0; l < 4096; ++l) {
        cum += hist[l];
        if (cum >= target) { med = l; break; }
    }
    if (med == 0 && !overflow.empty()) {
        std::sort(overflow.begin(), overflow.end());
        med = overflow[std::min(overflow.size() / 2, overflow.size() - 1)];
    }
    out->exact_read_pairs = pairs;
    out->total_bases_r1 = tb1;
    out->total_bases_r2 = tb2;
    out->total_bases = total;
    out->min_read_len = mn;
    out->max_read_len = mx;
    out->mean_read_len = (double)total / (double)reads;
    out->median_read_len = med;
    return FBK_OK;
}

// ---------------------------------------------------------------------------
// trimming and merging — trim_merge.rs:12-238
// ---------------------------------------------------------------------------
static inline uint8_t upper(uint8_t c) { return (c >= 'a' && c <= 'z') ? (uint8_t)(c - 32) : c; }
static const uint8_t ADAPTER_TRUSEQ[] = "AGATCGGAAGAGC";        // trim_merge.rs:12
static const uint8_t ADAPTER_NEXTERA[] = "AGATGTGTATAAGAGACAG";  // :13
static const uint8_t ADAPTER_NEXTERA_RC[] = "CTGTCTCTTATACACATCT";  // :14

// <= 1 mismatch over the first 10 adapter bases (eq_ignore_ascii_case)
static inline bool adapter_hit(const uint8_t* w, const uint8_t* adapter) {
    int mm = 0;
    for (int j = 0; j < 10; ++j)
        if (upper(w[j]) != adapter[j] && ++mm > 1) return false;
    return true;
}

// trim_adapter (trim_merge.rs:17-76): the cut is the first position where an
// adapter prefix matches; later positions can only keep the minimum.
uint64_t trim_adapter_len(const uint8_t* seq, uint64_t len) {
    if (len < 10) return len;
    const uint64_t start = len > 100 ? len - 100 : 0;
    for (uint64_t i = start; i + 10 <= len; ++i) {
        const uint8_t b0 = upper(seq[i]), b1 = upper(seq[i + 1]);
        const bool is_agat = b0 == 'A' || b1 == 'G';
        const bool is_ctgt = b0 == 'C' || b1 == 'T';
        if (!is_agat && !is_ctgt) continue;
        if (is_agat && (adapter_hit(seq + i, ADAPTER_TRUSEQ) || adapter_hit(seq + i, ADAPTER_NEXTERA))) return i;
        if (is_ctgt && adapter_hit(seq + i, ADAPTER_NEXTERA_RC)) return i;
    }
    return len;
}

// trim_quality (trim_merge.rs:79-115); returns the kept length or -1 for None.
int64_t trim_quality_len(const uint8_t* seq, const uint8_t* qual, uint64_t len, uint64_t qual_len, uint32_t min_qual,
                         uint64_t min_len) {
    (void)seq;
    if (len < min_len || qual_len != len) return -1;
    uint64_t cut = len;
    const uint64_t ws = 4;
    if (qual_len >= ws) {
        auto wsum = [&](uint64_t c) {
            uint64_t s = 0;
            for (uint64_t i = c - ws; i < c; ++i) s += qual[i] > 33 ? qual[i] - 33 : 0;
            return s;
        };
        if (wsum(cut) >= (uint64_t)min_qual * ws) return (int64_t)len;
        while (cut >= ws) {
            if (wsum(cut) / ws >= min_qual) break;
            cut -= 1;
        }
    }
    if (cut < min_len) return -1;
    return (int64_t)cut;
}

// merge_read_pair (trim_merge.rs:135-238)
int64_t merge_pair(const uint8_t* r1, const uint8_t* q1, uint64_t l1, uint64_t ql1, const uint8_t* r2, const uint8_t* q2,
                   uint64_t l2, uint64_t ql2, uint64_t min_overlap, double max_mismatch_ratio, uint8_t* out,
                   uint64_t* overlap_len, uint64_t* mismatches) {
    if (l1 < min_overlap || l2 < min_overlap) return -1;
    // a base other than ACGT becomes 'A' when R2 has at most 512 bases (the stack path,
    // trim_merge.rs:152-162) and 'T' when it is longer (reverse_complement_ascii,
    // bitseq.rs:90-98, reads it as A and complements it)
    const uint8_t other = l2 <= 512 ? 'A' : 'T';
    std::vector<uint8_t> rc2(l2);
    for (uint64_t i = 0; i < l2; ++i) {
        const uint8_t c = r2[l2 - 1 - i];
        rc2[i] = (c == 'A' || c == 'a') ? 'T' : (c == 'C' || c == 'c') ? 'G' : (c == 'G' || c == 'g') ? 'C' : (c == 'T' || c == 't') ? 'A' : other;
    }
    const uint64_t max_d = std::min(l1, l2);
    uint64_t best_d = 0, best_mm = 0;
    double best_score = -__builtin_inf();
    for (int64_t dd = (int64_t)max_d; dd >= (int64_t)min_overlap; --dd) {
        const uint64_t d = (uint64_t)dd;
        const uint8_t* s1 = r1 + (l1 - d);
        const uint64_t max_allowed = (uint64_t)((double)d * max_mismatch_ratio);
        uint64_t mm = 0;
        for (uint64_t i = 0; i < d; ++i)
            if (upper(s1[i]) != upper(rc2[i]) && ++mm > max_allowed) break;
        if (mm <= max_allowed) {
            const double score = (double)d - 2.5 * (double)mm;
            if (score > best_score) {
                best_score = score;
                best_d = d;
                best_mm = mm;
            }
        }
        if ((double)d <= best_score) break;
    }
    if (!(best_d >= min_overlap)) return -1;
    uint64_t n = 0;
    for (uint64_t i = 0; i < l1 - best_d; ++i) out[n++] = r1[i];
    for (uint64_t i = 0; i < best_d; ++i) {
        const uint8_t b1 = r1[l1 - best_d + i], b2 = rc2[i];
        const uint8_t qa = (l1 - best_d + i) < ql1 ? q1[l1 - best_d + i] : (uint8_t)'I';
        const uint8_t qb = i < l2 ? ((l2 - 1 - i) < ql2 ? q2[l2 - 1 - i] : (uint8_t)'I') : (uint8_t)'I';
        if (upper(b1) == upper(b2)) out[n++] = upper(b1);
        else if (qa >= qb) out[n++] = upper(b1);
        else out[n++] = upper(b2);
    }
    for (uint64_t i = best_d; i < l2; ++i) out[n++] = rc2[i];
    if (overlap_len) *overlap_len = best_d;
    if (mismatches) *mismatches = best_mm;
    return (int64_t)n;
}

// ---------------------------------------------------------------------------
// per-pair ingest — ingest_reads_ext_with_seed (trim_merge.rs:307-417)
// ---------------------------------------------------------------------------
PairIngester::PairIngester(const IngestParams& pp) : p(pp) {
    should_subsample = p.subsample_factor < 0.999;
    const double x = p.subsample_factor * 18446744073709551616.0;
    keep_threshold = !(x > 0.0) ? 0 : x >= 18446744073709551616.0 ? UINT64_MAX : (uint64_t)x;
}

void PairIngester::ingest(uint64_t pair_idx1, const uint8_t* s1, const uint8_t* q1, uint64_t l1, uint64_t ql1,
                          const uint8_t* s2, const uint8_t* q2, uint64_t l2, uint64_t ql2, HostArena* arenas, IngestStats& st) {
    st.input_read_pairs++;
    st.bases_before_trim += l1 + l2;
    if (should_subsample && splitmix64(pair_idx1 ^ p.seed) > keep_threshold) return;
    uint64_t t1, t2;
    if (p.enable_trim) {
        const uint64_t a1 = trim_adapter_len(s1, l1), a2 = trim_adapter_len(s2, l2);
        const int64_t x1 = trim_quality_len(s1, q1, a1, std::min(a1, ql1), p.min_qual, p.min_len);
        const int64_t x2 = trim_quality_len(s2, q2, a2, std::min(a2, ql2), p.min_qual, p.min_len);
        if (x1 < 0 || x2 < 0) return;
        t1 = (uint64_t)x1;
        t2 = (uint64_t)x2;
    } else {
        if (l1 < p.min_len || l2 < p.min_len) return;
        t1 = l1;
        t2 = l2;
    }
    st.retained_read_pairs++;
    st.bases_after_trim += t1 + t2;
    const uint32_t pair0 = (uint32_t)(pair_idx1 - 1);
    if (p.enable_merge) {
        if (merged.size() < t1 + t2) merged.resize(t1 + t2);
        const int64_t m = merge_pair(s1, q1, t1, std::min(t1, ql1), s2, q2, t2, std::min(t2, ql2), 15, 0.10, merged.data(),
                                     nullptr, nullptr);
        if (m >= 0) {
            st.merged_pairs_count++;
            st.merged_bases += (uint64_t)m;
            arenas[0].push_ascii(merged.data(), (uint64_t)m, pair0);
            return;
        }
    }
    st.unmerged_pairs_count++;
    arenas[1].push_ascii(s1, t1, pair0);
    arenas[2].push_ascii(s2, t2, pair0);
}

}  // namespace fbk

using namespace fbk;

extern "C" {

FBK_API fbk_status fbk_count_fastx_exact(const char* r1, const char* r2, fbk_count_stats* out, char* err, size_t errlen) {
    if (!r1 || !r2 || !out) return FBK_ERR_INVALID;
    std::string e;
    fbk_status st = count_fastx_exact_impl(r1, r2, out, e);
    if (st && err && errlen) snprintf(err, errlen, "%s", e.c_str());
    return st;
}

FBK_API fbk_status fbk_ingest_fastq(const char* r1, const char* r2, double subsample_factor, uint64_t min_len, uint32_t min_qual,
                                    int enable_trim, int enable_merge, uint64_t seed, fbk_hbank** out, char* err, size_t errlen) {
    if (!r1 || !r2 || !out) return FBK_ERR_INVALID;
    auto fail = [&](fbk_status st, const std::string& m) {
        if (err && errlen) snprintf(err, errlen, "%s", m.c_str());
        return st;
    };
    FastqReader a(r1), b(r2);
    if (!a.ok()) return fail(FBK_ERR_IO, std::string("Failed to open file \"") + r1 + "\"");
    if (!b.ok()) return fail(FBK_ERR_IO, std::string("Failed to open file \"") + r2 + "\"");
    IngestParams p;
    p.subsample_factor = subsample_factor;
    p.min_len = min_len;
    p.min_qual = min_qual;
    p.enable_trim = enable_trim != 0;
    p.enable_merge = enable_merge != 0;
    p.seed = seed;
    PairIngester ing(p);
    std::unique_ptr<fbk_hbank> hb(new fbk_hbank());
    uint64_t pair_idx = 0;
    std::string e1, e2;
    for (;;) {
        const int x = a.next(e1), y = b.next(e2);
        if (x == 1 && y == 1) {
            pair_idx++;
            ing.ingest(pair_idx, (const uint8_t*)a.seq.data(), (const uint8_t*)a.qual.data(), a.seq.size(), a.qual.size(),
                       (const uint8_t*)b.seq.data(), (const uint8_t*)b.qual.data(), b.seq.size(), b.qual.size(), hb->a, hb->stats);
        } else if (x < 0) {
            return fail(FBK_ERR_FORMAT, "Corrupted record in R1 FASTQ: " + e1);
        } else if (y < 0) {
            return fail(FBK_ERR_FORMAT, "Corrupted record in R2 FASTQ: " + e2);
        } else if (x != y) {
            return fail(FBK_ERR_FORMAT, "Mismatched paired-end FASTQ mate counts between R1 and R2");
        } else {
            break;
        }
    }
    if (hb->a[0].off.size() + hb->a[1].off.size() + hb->a[2].off.size() == 0)
        return fail(FBK_ERR_EMPTY, "No valid reads survived trimming and quality filtering (check input FASTQ files)");
    *out = hb.release();
    return FBK_OK;
}

FBK_API fbk_status fbk_hbank_arena(const fbk_hbank* hb, int arena, fbk_arena_view* view) {
    if (!hb || !view || arena < 0 || arena > 2) return FBK_ERR_INVALID;
    *view = hb->a[arena].view();
    return FBK_OK;
}

FBK_API fbk_status fbk_hbank_stats(const fbk_hbank* hb, uint64_t* input_pairs, uint64_t* retained_pairs, uint64_t* merged_pairs,
                                   uint64_t* unmerged_pairs, uint64_t* bases_before_trim, uint64_t* bases_after_trim) {
    if (!hb) return FBK_ERR_INVALID;
    if (input_pairs) *input_pairs = hb->stats.input_read_pairs;
    if (retained_pairs) *retained_pairs = hb->stats.retained_read_pairs;
    if (merged_pairs) *merged_pairs = hb->stats.merged_pairs_count;
    if (unmerged_pairs) *unmerged_pairs = hb->stats.unmerged_pairs_count;
    if (bases_before_trim) *bases_before_trim = hb->stats.bases_before_trim;
    if (bases_after_trim) *bases_after_trim = hb->stats.bases_after_trim;
    return FBK_OK;
}

FBK_API void fbk_hbank_free(fbk_hbank* hb) { delete hb; }

FBK_API uint64_t fbk_trim_adapter(const uint8_t* seq, uint64_t len) { return seq ? trim_adapter_len(seq, len) : 0; }

FBK_API int64_t fbk_trim_quality(const uint8_t* seq, const uint8_t* qual, uint64_t len, uint32_t min_qual, uint64_t min_len) {
    if (!qual && len) return -1;
    return trim_quality_len(seq, qual, len, len, min_qual, min_len);
}

FBK_API int64_t fbk_merge_read_pair(const uint8_t* r1, const uint8_t* q1, uint64_t l1, const uint8_t* r2, const uint8_t* q2,
                                    uint64_t l2, uint64_t min_overlap, double max_mismatch_ratio, uint8_t* merged_out,
                                    uint64_t* overlap_len, uint64_t* mismatches) {
    if ((!r1 && l1) || (!r2 && l2) || !merged_out) return -1;
    return merge_pair(r1, q1, l1, q1 ? l1 : 0, r2, q2, l2, q2 ? l2 : 0, min_overlap, max_mismatch_ratio, merged_out, overlap_len,
                      mismatches);
}

}  // extern "C"
