// fbk_synth.cpp — seeded synthetic isolates (genome + paired reads) streamed
// straight into a host ReadBank.  See include/fbk_synth.h for the model.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <memory>
#include <thread>

#include "../../../include/fbk_synth.h"
#include "../host/fbk_host.h"

namespace fbk {

// splitmix64 generator (state += golden ratio, output = finaliser)
struct Rng {
    uint64_t s;
    explicit Rng(uint64_t seed) : s(seed) {}
    uint64_t next() {
        s += 0x9E3779B97F4A7C15ULL;
        return splitmix64(s);
    }
    double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }  // [0,1)
    // Irwin-Hall: the sum of 12 uniforms minus 6 has mean 0 and variance 1.  It uses
    // only IEEE additions, so x86 and Arm hosts generate identical isolates.
    double normal() {
        double s = 0.0;
        for (int i = 0; i < 12; ++i) s += uniform();
        return s - 6.0;
    }
};

static const uint8_t BASES[4] = {'A', 'C', 'G', 'T'};

static inline uint8_t gc_base(Rng& r, uint64_t gc_thr) {
    const bool is_gc = r.next() < gc_thr;
    const bool bit = r.next() & 1;
    return is_gc ? (bit ? 'G' : 'C') : (bit ? 'T' : 'A');
}

static inline uint8_t comp(uint8_t c) {
    switch (c) {
        case 'A': return 'T';
        case 'C': return 'G';
        case 'G': return 'C';
        default: return 'A';
    }
}

static uint64_t gc_threshold(double gc) {
    const double x = gc * 18446744073709551616.0;
    return !(x > 0.0) ? 0 : x >= 18446744073709551616.0 ? UINT64_MAX : (uint64_t)x;
}

static void make_genome(const fbk_synth_params& p, uint8_t* g) {
    const uint64_t G = p.genome_len, thr = gc_threshold(p.gc);
    Rng r(splitmix64(p.seed ^ 0x47454e4f4d45ULL));
    for (uint64_t i = 0; i < G; ++i) g[i] = gc_base(r, thr);
    // near-identical repeat copies, spread evenly
    if (p.n_repeats && p.repeat_len && p.repeat_len < G) {
        std::vector<uint8_t> unit(p.repeat_len);
        for (auto& c : unit) c = gc_base(r, thr);
        const double mut = (1.0 - p.repeat_identity) * 0.5;
        for (uint32_t c = 0; c < p.n_repeats; ++c) {
            const uint64_t pos = (uint64_t)(((double)c + 0.5) * (double)G / (double)p.n_repeats);
            for (uint32_t j = 0; j < p.repeat_len; ++j) {
                uint8_t b = unit[j];
                if (r.uniform() < mut) b = BASES[(std::find(BASES, BASES + 4, b) - BASES + 1 + r.next() % 3) % 4];
                g[(pos + j) % G] = b;
            }
        }
    }
    // tandem array, placed between the first two repeat copies
    if (p.tandem_copies && p.tandem_unit) {
        std::vector<uint8_t> unit(p.tandem_unit);
        for (auto& c : unit) c = gc_base(r, thr);
        const uint64_t pos = p.n_repeats ? (uint64_t)(1.0 * (double)G / (double)p.n_repeats) : G / 3;
        for (uint64_t j = 0; j < (uint64_t)p.tandem_copies * p.tandem_unit; ++j) g[(pos + j) % G] = unit[j % p.tandem_unit];
    }
}

// One read walked along template T (length tl) with substitutions and indels.
static void walk_read(Rng& r, const uint8_t* T, uint64_t tl, const fbk_synth_params& p, uint8_t* out, uint8_t* q) {
    uint64_t j = 0;
    for (uint32_t o = 0; o < p.read_len; ++o) {
        const double u = r.uniform();
        uint8_t b;
        if (u < p.indel_rate * 0.5) {
            b = BASES[r.next() & 3];  // insertion: template position unchanged
        } else {
            if (u < p.indel_rate) j++;  // deletion: skip one template base
            b = j < tl ? T[j] : BASES[r.next() & 3];
            j++;
            if (r.uniform() < p.sub_rate) b = BASES[(std::find(BASES, BASES + 4, b) - BASES + 1 + r.next() % 3) % 4];
        }
        out[o] = b;
        const uint32_t span = p.q_hi >= p.q_lo ? p.q_hi - p.q_lo + 1 : 1;
        double qq = (double)(p.q_lo + (uint32_t)(r.next() % span));
        const uint32_t tail_start = p.read_len > p.tail_len ? p.read_len - p.tail_len : 0;
        if (p.tail_len && o >= tail_start) {
            const double f = (double)(o - tail_start + 1) / (double)p.tail_len;
            qq = qq + ((double)p.tail_q - qq) * f;
        }
        q[o] = (uint8_t)(33 + (int)std::lround(qq));
    }
}

static void make_pair(const fbk_synth_params& p, const uint8_t* g, uint64_t i, uint8_t* r1, uint8_t* q1, uint8_t* r2,
                      uint8_t* q2, std::vector<uint8_t>& tmpl) {
    const uint64_t G = p.genome_len;
    Rng r(splitmix64(p.seed ^ splitmix64(i + 0x5041495253ULL)));
    double fl = std::round(p.frag_mean + p.frag_sd * r.normal());
    const double lo = (double)p.read_len + 16.0, hi = std::max(lo, 4.0 * p.frag_mean);
    fl = std::min(std::max(fl, lo), hi);
    const uint64_t L = (uint64_t)fl;
    const uint64_t pos = r.next() % G;
    const bool strand = r.next() & 1;
    tmpl.resize(L);
    for (uint64_t j = 0; j < L; ++j) tmpl[j] = g[(pos + j) % G];
    if (strand) {
        std::reverse(tmpl.begin(), tmpl.end());
        for (auto& c : tmpl) c = comp(c);
    }
    walk_read(r, tmpl.data(), L, p, r1, q1);
    std::reverse(tmpl.begin(), tmpl.end());
    for (auto& c : tmpl) c = comp(c);
    walk_read(r, tmpl.data(), L, p, r2, q2);
}

}  // namespace fbk

using namespace fbk;

extern "C" {

FBK_API void fbk_synth_defaults(fbk_synth_params* p) {
    if (!p) return;
    memset(p, 0, sizeof(*p));
    p->seed = 42;
    p->genome_len = 1000000;
    p->gc = 0.50;
    p->repeat_len = 5000;
    p->repeat_identity = 0.99;
    p->tandem_unit = 60;
    p->read_len = 150;
    p->coverage = 50.0;
    p->frag_mean = 350.0;
    p->frag_sd = 30.0;
    p->sub_rate = 0.005;
    p->indel_rate = 0.0;
    p->q_lo = 30;
    p->q_hi = 40;
    p->tail_len = 20;
    p->tail_q = 15;
}

FBK_API uint64_t fbk_synth_n_pairs(const fbk_synth_params* p) {
    if (!p || p->read_len == 0) return 0;
    return (uint64_t)std::llround(p->coverage * (double)p->genome_len / (2.0 * (double)p->read_len));
}

FBK_API fbk_status fbk_synth_genome(const fbk_synth_params* p, uint8_t* out) {
    if (!p || !out || p->genome_len == 0) return FBK_ERR_INVALID;
    make_genome(*p, out);
    return FBK_OK;
}

FBK_API fbk_status fbk_synth_pairs(const fbk_synth_params* p, const uint8_t* genome, uint64_t first, uint64_t n, uint8_t* r1,
                                   uint8_t* q1, uint8_t* r2, uint8_t* q2) {
    if (!p || !genome || !r1 || !q1 || !r2 || !q2 || p->read_len == 0) return FBK_ERR_INVALID;
    std::vector<uint8_t> tmpl;
    const uint64_t L = p->read_len;
    for (uint64_t i = 0; i < n; ++i) make_pair(*p, genome, first + i, r1 + i * L, q1 + i * L, r2 + i * L, q2 + i * L, tmpl);
    return FBK_OK;
}

FBK_API fbk_status fbk_synth_write_fastq(const fbk_synth_params* p, const char* r1_path, const char* r2_path) {
    if (!p || !r1_path || !r2_path || p->genome_len == 0 || p->read_len == 0) return FBK_ERR_INVALID;
    std::vector<uint8_t> g(p->genome_len);
    make_genome(*p, g.data());
    FILE* f1 = fopen(r1_path, "wb");
    FILE* f2 = fopen(r2_path, "wb");
    if (!f1 || !f2) {
        if (f1) fclose(f1);
        if (f2) fclose(f2);
        return FBK_ERR_IO;
    }
    const uint64_t n = fbk_synth_n_pairs(p), L = p->read_len;
    std::vector<uint8_t> a(L), qa(L), b(L), qb(L), tmpl;
    for (uint64_t i = 0; i < n; ++i) {
        make_pair(*p, g.data(), i, a.data(), qa.data(), b.data(), qb.data(), tmpl);
        fprintf(f1, "@fbk_%llu/1\n%.*s\n+\n%.*s\n", (unsigned long long)(i + 1), (int)L, (const char*)a.data(), (int)L,
                (const char*)qa.data());
        fprintf(f2, "@fbk_%llu/2\n%.*s\n+\n%.*s\n", (unsigned long long)(i + 1), (int)L, (const char*)b.data(), (int)L,
                (const char*)qb.data());
    }
    const bool bad = ferror(f1) || ferror(f2);
    fclose(f1);
    fclose(f2);
    return bad ? FBK_ERR_IO : FBK_OK;
}

FBK_API fbk_status fbk_synth_isolate(const fbk_synth_params* p, int threads, uint64_t min_len, uint32_t min_qual, int enable_trim,
                                     int enable_merge, fbk_hbank** bank, uint64_t sample_pairs, fbk_hbank** sample,
                                     fbk_count_stats* stats) {
    if (!p || !bank || p->genome_len == 0 || p->read_len == 0) return FBK_ERR_INVALID;
    const uint64_t n = fbk_synth_n_pairs(p);
    if (n == 0 || n > 0xFFFFFFFFULL) return FBK_ERR_INVALID;
    std::vector<uint8_t> g(p->genome_len);
    make_genome(*p, g.data());
    if (threads <= 0) threads = (int)std::max(1u, std::thread::hardware_concurrency());
    const uint64_t chunk = 16384;
    const uint64_t n_chunks = (n + chunk - 1) / chunk;
    IngestParams ip;
    ip.min_len = min_len;
    ip.min_qual = min_qual;
    ip.enable_trim = enable_trim != 0;
    ip.enable_merge = enable_merge != 0;
    // Each chunk of pairs is ingested into its own arenas; chunks are then
    // concatenated in pair order, which equals one sequential ingest.
    std::vector<std::unique_ptr<fbk_hbank>> parts(n_chunks);
    std::atomic<uint64_t> next(0);
    auto worker = [&]() {
        PairIngester ing(ip);
        std::vector<uint8_t> a(p->read_len), qa(p->read_len), b(p->read_len), qb(p->read_len), tmpl;
        for (;;) {
            const uint64_t c = next.fetch_add(1);
            if (c >= n_chunks) break;
            parts[c].reset(new fbk_hbank());
            const uint64_t e = std::min(n, (c + 1) * chunk);
            for (uint64_t i = c * chunk; i < e; ++i) {
                make_pair(*p, g.data(), i, a.data(), qa.data(), b.data(), qb.data(), tmpl);
                ing.ingest(i + 1, a.data(), qa.data(), p->read_len, p->read_len, b.data(), qb.data(), p->read_len, p->read_len,
                           parts[c]->a, parts[c]->stats);
            }
        }
    };
    std::vector<std::thread> ts;
    for (int t = 0; t < threads; ++t) ts.emplace_back(worker);
    for (auto& t : ts) t.join();
    std::unique_ptr<fbk_hbank> out(new fbk_hbank());
    for (int a = 0; a < 3; ++a) {
        HostArena& dst = out->a[a];
        uint64_t nb = 0, ns = 0;
        for (auto& pt : parts) {
            nb += pt->a[a].n_bases;
            ns += pt->a[a].off.size();
        }
        dst.data.assign((nb + 31) / 32, 0);
        dst.off.reserve(ns);
        dst.len.reserve(ns);
        dst.pair_idx.reserve(ns);
        // bit-shifted append of each part's packed words
        uint64_t base = 0;
        for (auto& pt : parts) {
            const HostArena& s = pt->a[a];
            for (size_t i = 0; i < s.off.size(); ++i) {
                dst.off.push_back(s.off[i] + base);
                dst.len.push_back(s.len[i]);
                dst.pair_idx.push_back(s.pair_idx[i]);
            }
            const uint64_t sh = (base & 31) * 2, w0 = base >> 5;
            for (size_t w = 0; w < s.data.size(); ++w) {
                const uint64_t v = s.data[w];
                if (w0 + w < dst.data.size()) dst.data[w0 + w] |= v << sh;
                if (sh && w0 + w + 1 < dst.data.size()) dst.data[w0 + w + 1] |= v >> (64 - sh);
            }
            base += s.n_bases;
        }
        dst.n_bases = nb;
    }
    for (auto& pt : parts) {
        IngestStats& s = pt->stats;
        out->stats.input_read_pairs += s.input_read_pairs;
        out->stats.retained_read_pairs += s.retained_read_pairs;
        out->stats.bases_before_trim += s.bases_before_trim;
        out->stats.bases_after_trim += s.bases_after_trim;
        out->stats.merged_pairs_count += s.merged_pairs_count;
        out->stats.merged_bases += s.merged_bases;
        out->stats.unmerged_pairs_count += s.unmerged_pairs_count;
    }
    if (stats) {
        // every raw read has read_len bases (walk_read emits fixed-length reads)
        stats->exact_read_pairs = n;
        stats->total_bases_r1 = n * p->read_len;
        stats->total_bases_r2 = n * p->read_len;
        stats->total_bases = 2 * n * p->read_len;
        stats->min_read_len = p->read_len;
        stats->max_read_len = p->read_len;
        stats->mean_read_len = (double)(2 * n * p->read_len) / (double)(2 * n);
        stats->median_read_len = p->read_len;
    }
    if (sample && sample_pairs > 0) {
        const uint64_t m = std::min(sample_pairs, n);
        std::unique_ptr<fbk_hbank> s(new fbk_hbank());
        std::vector<uint8_t> a(p->read_len), qa(p->read_len), b(p->read_len), qb(p->read_len), tmpl;
        for (uint64_t i = 0; i < m; ++i) {
            make_pair(*p, g.data(), i, a.data(), qa.data(), b.data(), qb.data(), tmpl);
            s->a[0].push_ascii(a.data(), p->read_len, (uint32_t)i);
            s->a[0].push_ascii(b.data(), p->read_len, (uint32_t)i);
        }
        *sample = s.release();
    }
    *bank = out.release();
    return FBK_OK;
}

}  // extern "C"
