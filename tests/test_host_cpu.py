"""CPU tests of the product's host side: the C ABI exports every declared symbol,
the synthetic generator is deterministic, and the host ingest reproduces the
reference's known answers (src/ingest/trim_merge.rs:423-508, estimator.rs:448-546,
bitseq.rs:448-506)."""
import ctypes as C
import re
import subprocess
from pathlib import Path

import numpy as np
import pytest

from fastbact_gb300 import _native as N
from fastbact_gb300 import api
from oracle import orc

ROOT = Path(__file__).resolve().parent.parent
M64 = (1 << 64) - 1


def declared_symbols():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        txt = h.read_text()
        for m in re.finditer(r"FBK_API\s+[^;{]*?\b(fbk_\w+)\s*\(", txt):
            names.add(m.group(1))
    return names


def _exports(path):
    out = subprocess.run(["nm", "-D", "--defined-only", str(path)], capture_output=True, text=True, check=True).stdout
    return {ln.split()[-1] for ln in out.splitlines() if " T " in ln}


def test_library_exports_every_declared_symbol():
    """fbk.h is exported by libfbk.so, fbk_synth.h by the generator's libfbk_synth.so,
    and the generator library does not need the device library."""
    declared = declared_symbols()
    assert len(declared) > 50
    synth_declared = {n for n in declared if n.startswith("fbk_synth_")}
    dev_declared = declared - synth_declared
    dev_exported = _exports(N.LIB_PATH)
    assert dev_declared <= dev_exported, sorted(dev_declared - dev_exported)
    assert not (synth_declared & dev_exported), "the generator must live outside the device library"
    synth_exported = _exports(N.SYNTH_LIB_PATH)
    assert synth_declared <= synth_exported, sorted(synth_declared - synth_exported)
    assert dev_declared == set(N.SIGNATURES), sorted(dev_declared ^ set(N.SIGNATURES))
    assert synth_declared == {n for n in N.SYNTH_SIGNATURES if n.startswith("fbk_synth_")}
    needed = subprocess.run(["readelf", "-d", str(N.SYNTH_LIB_PATH)], capture_output=True, text=True, check=True).stdout
    assert "libfbk.so" not in needed and "libcuda" not in needed and "libcudart" not in needed
    N.lib()  # binds every signature
    N.synth_lib()


def test_no_device_is_reported_not_faked():
    # On a host without a GPU the context refuses with FBK_ERR_NO_DEVICE (no CPU fallback).
    h = C.c_void_p()
    st = N.lib().fbk_ctx_create(0, 0, C.byref(h))
    if st == 0:
        N.lib().fbk_ctx_destroy(h)
        pytest.skip("a device is present")
    assert st == 11


def lcg_bases(seed, n):
    out, s = [], seed
    for _ in range(n):
        s = (s * 6364136223846793005 + 1442695040888963407) & M64
        out.append(b"ACGT"[s % 4])
    return bytes(out)


def test_arena_roundtrip_lengths_1_to_500():  # bitseq.rs:472-506
    seqs, s = [], 0x123456789ABCDEF
    for n in range(1, 501):
        seq = []
        for _ in range(n):
            s = (s * 6364136223846793005 + 1442695040888963407) & M64
            seq.append(b"ACGT"[s % 4])
        seqs.append(bytes(seq))
    a = api.BitSeqArena.from_seqs(seqs)
    for i in (0, 1, 30, 31, 32, 33, 63, 64, 255, 499):
        assert a.extract_ascii(i) == seqs[i]
    assert a.total_bases() == sum(range(1, 501))


def test_arena_packing_kat():  # bitseq.rs:448-470
    a = api.BitSeqArena.from_seqs([b"ACGTACGTACGTACGT", b"TGCATGCA", b"AAGGCCTT"])
    assert [a.extract_ascii(i) for i in range(3)] == [b"ACGTACGTACGTACGT", b"TGCATGCA", b"AAGGCCTT"]
    assert list(a.offsets) == [0, 16, 24]


def splitmix_py(z):
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & M64
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & M64
    return z ^ (z >> 31)


def rc(s: bytes) -> bytes:
    return s[::-1].translate(bytes.maketrans(b"ACGT", b"TGCA"))


def test_merge_230bp_fragment_with_errors():  # trim_merge.rs:424-471
    frag = bytes(b"ACGT"[splitmix_py(0x5EEDCAFE12345678 + i) % 4] for i in range(230))
    r1 = bytearray(frag[:150])
    q1 = bytearray(b"I" * 150)
    r1[130] = ord("C") if r1[130] == ord("A") else ord("A")
    q1[130] = ord("!")
    r2 = bytearray(rc(frag[80:230]))
    q2 = bytearray(b"I" * 150)
    r2[129] = ord("T") if r2[129] == ord("A") else ord("A")
    q2[129] = ord("!")
    res = api.merge_read_pair(bytes(r1), bytes(q1), bytes(r2), bytes(q2), 15, 0.10)
    assert res is not None
    seq, ov, mm = res
    assert (len(seq), ov, mm) == (230, 70, 2)
    assert seq == frag


def test_long_fragment_stays_unmerged():  # trim_merge.rs:473-497
    frag = bytes(b"ACGT"[splitmix_py(0xABCDEF0123456789 + i) % 4] for i in range(450))
    assert api.merge_read_pair(frag[:150], b"I" * 150, rc(frag[300:450]), b"I" * 150) is None


def test_adapter_trimming():  # trim_merge.rs:499-507
    seq = b"ACGTACGTACGTACGT" + b"AGATCGGAAGAGCextra"
    assert api.trim_adapter(seq) == b"ACGTACGTACGTACGT"


def test_quality_trim_window():  # trim_merge.rs:79-115
    seq = b"A" * 40
    assert api.trim_quality(seq, b"I" * 40, 20, 30) == (seq, b"I" * 40)
    q = b"I" * 34 + b"#" * 6  # Phred 2 tail
    s, qq = api.trim_quality(seq, q, 20, 30)
    assert len(s) == 34 + 2  # window of 4 ending at 36 has mean (40+40+2+2)/4 = 21 >= 20
    assert api.trim_quality(b"A" * 20, b"I" * 20, 20, 30) is None


def write_fastq(path, recs):
    with open(path, "w") as f:
        for name, seq, qual in recs:
            f.write(f"@{name}\n{seq}\n+\n{qual}\n")


def test_count_fastx_exact_kats(tmp_path):  # estimator.rs:463-526
    r1, r2 = tmp_path / "x_1.fq", tmp_path / "x_2.fq"
    write_fastq(r1, [(f"pair_{i}/1", "ACGTACGTACGT", "I" * 12) for i in range(1, 11)])
    write_fastq(r2, [(f"pair_{i}/2", "TGCATGCATGCA", "I" * 12) for i in range(1, 11)])
    s = api.count_fastx_exact(r1, r2)
    assert (s.exact_read_pairs, s.total_bases_r1, s.total_bases_r2, s.total_bases) == (10, 120, 120, 240)
    assert (s.min_read_len, s.max_read_len, s.median_read_len, s.mean_read_len) == (12, 12, 12, 12.0)
    write_fastq(r1, [(f"pair_{i}/1", "ACGT", "IIII") for i in range(1, 6)])
    write_fastq(r2, [(f"pair_{i}/2", "ACGT", "IIII") for i in range(1, 5)])
    with pytest.raises(N.FbkError, match="R1 has more reads than R2"):
        api.count_fastx_exact(r1, r2)
    write_fastq(r1, [("pair_A/1", "ACGT", "IIII")])
    write_fastq(r2, [("pair_B/2", "ACGT", "IIII")])
    with pytest.raises(N.FbkError, match="synchronization error"):
        api.count_fastx_exact(r1, r2)
    write_fastq(r1, [])
    write_fastq(r2, [])
    with pytest.raises(N.FbkError, match="0 valid read pairs"):
        api.count_fastx_exact(r1, r2)


def test_read_id_prefix_rules(tmp_path):  # estimator.rs:448-461 through the pairing check
    r1, r2 = tmp_path / "p_1.fq", tmp_path / "p_2.fq"
    write_fastq(r1, [("SRR28349173.1 1 length=150", "ACGT", "IIII"), ("read1/1", "ACGT", "IIII")])
    write_fastq(r2, [("SRR28349173.1 2 length=150", "ACGT", "IIII"), ("read1/2", "ACGT", "IIII")])
    assert api.count_fastx_exact(r1, r2).exact_read_pairs == 2


def test_compute_dynamic_kmers_matches_oracle():  # estimator.rs:528-546
    for med in [30, 50, 74, 75, 99, 100, 101, 150, 250, 300]:
        for tgt in [None, 21, 40, 63, 80, 127, 200]:
            out = (C.c_uint64 * 16)()
            n = orc.lib().orc_compute_dynamic_kmers(med, -1 if tgt is None else tgt, out, 16)
            assert api.compute_dynamic_kmers(med, tgt) == [out[i] for i in range(n)]
    k = api.compute_dynamic_kmers(150)
    assert k[0] == 31 and k[-1] == 127


def small_params(**kw):
    d = dict(seed=7, genome_len=40_000, coverage=20.0)
    d.update(kw)
    return api.synth_params(**d)


def test_synth_is_deterministic_and_thread_independent():
    p = small_params()
    b1, s1, smp1, n1, c1 = api.synth_isolate(p, threads=1, sample_pairs=500)
    b2, s2, smp2, n2, c2 = api.synth_isolate(p, threads=4, sample_pairs=500)
    for a, b in zip(b1.arenas, b2.arenas):
        assert np.array_equal(a.data, b.data) and np.array_equal(a.offsets, b.offsets)
        assert np.array_equal(a.lengths, b.lengths) and np.array_equal(a.pair_idx, b.pair_idx)
    assert np.array_equal(smp1.data, smp2.data) and n1 == n2 == 500
    assert c1 == c2 and c1.exact_read_pairs == api.N.synth_lib().fbk_synth_n_pairs(C.byref(p))
    # tail trimming and merging happened
    assert s1.retained_read_pairs <= s1.input_read_pairs
    assert len(b1.pe_forward) == len(b1.pe_reverse) > 0
    assert b1.pe_forward.lengths.max() <= 150 and b1.pe_forward.lengths.min() >= 30


def test_synth_fastq_roundtrip_through_ingest(tmp_path):
    p = small_params(genome_len=20_000, coverage=10.0)
    r1, r2 = tmp_path / "s_1.fq", tmp_path / "s_2.fq"
    api.synth_write_fastq(p, r1, r2)
    bank_f, st_f = api.ingest_reads_ext_with_seed(r1, r2, 1.0, 30, 20, True, True, 0)
    bank_m, st_m, _, _, cs = api.synth_isolate(p, threads=2, sample_pairs=0)
    for a, b in zip(bank_f.arenas, bank_m.arenas):
        assert np.array_equal(a.data, b.data) and np.array_equal(a.lengths, b.lengths)
    assert st_f == st_m
    s = api.count_fastx_exact(r1, r2)
    assert s == cs


def test_ingest_subsample_matches_keep_rule(tmp_path):
    p = small_params(genome_len=20_000, coverage=10.0)
    r1, r2 = tmp_path / "t_1.fq", tmp_path / "t_2.fq"
    api.synth_write_fastq(p, r1, r2)
    full, _ = api.ingest_reads_ext_with_seed(r1, r2, 1.0, 30, 20, True, True, 0)
    sub, st = api.ingest_reads_ext_with_seed(r1, r2, 0.4, 30, 20, True, True, 11)
    thr = int(0.4 * 2.0 ** 64)
    kept = {i for i in range(st.input_read_pairs) if splitmix_py((i + 1) ^ 11) <= thr}
    for a_full, a_sub in zip(full.arenas, sub.arenas):
        sel = [j for j, pi in enumerate(a_full.pair_idx) if int(pi) in kept]
        assert list(a_sub.pair_idx) == [int(a_full.pair_idx[j]) for j in sel]
        assert [a_sub.extract_ascii(i) for i in range(min(20, len(a_sub)))] == \
               [a_full.extract_ascii(j) for j in sel[:20]]


def test_tuning_rejects_out_of_range_without_device():
    # validation happens before any device work; a NULL context is rejected outright
    assert N.lib().fbk_ctx_set_tuning(None, b"sweep_bytes", 1e6) == 1


def _estimate(cov, total_bases, confidence):
    e = N.GenomeEstimate()
    e.genome_size, e.total_bases, e.estimated_cov, e.confidence = 5_000_000, total_bases, cov, confidence
    return api.GenomeEstimate.from_c(e)


def test_subsample_policy_branches():  # src/main.rs:76-180
    auto = dict(enable_auto_subsample=True, depth=110.0, threshold_ratio=150.0 / 110.0)
    hi = _estimate(200.0, 1_000_000_000, 0)
    cases = [
        (dict(no_subsample=True, **auto), hi, 1.0, "EXPLICIT_NO_SUBSAMPLE_FLAG"),
        (dict(), hi, 1.0, "DISABLED_BY_DEFAULT_SAFE_FALLBACK"),
        (dict(genome_size=4_000_000), hi, 1.0, "GENOME_SIZE_PRIOR_PROVIDED_SUBSAMPLING_NOT_ENABLED"),
        (auto, hi, 110.0 / 200.0, "AUTO_SUBSAMPLE_HIGH_CONFIDENCE"),
        (auto, _estimate(140.0, 1, 0), 1.0, "AUTO_SUBSAMPLE_HIGH_CONFIDENCE_WITHIN_TARGET"),
        (auto, _estimate(150.0, 1, 0), 1.0, "AUTO_SUBSAMPLE_HIGH_CONFIDENCE_WITHIN_TARGET"),
        (auto, _estimate(400.0, 1, 1), 1.0, "AUTO_SUBSAMPLE_INTERCEPTED_LOW_COVERAGE_WARNING"),
        (auto, _estimate(400.0, 1, 2), 1.0, "AUTO_SUBSAMPLE_INTERCEPTED_UNRELIABLE"),
        (dict(genome_size=0, **auto), hi, 1.0, "EXPLICIT_GENOME_SIZE_ZERO_INVALID"),
        (dict(genome_size=5_000_000, **auto), hi, 110.0 / 200.0, "AUTO_SUBSAMPLE_EXPLICIT_GENOME_SIZE"),
        (dict(genome_size=8_000_000, **auto), hi, 1.0, "AUTO_SUBSAMPLE_EXPLICIT_GENOME_SIZE_WITHIN_TARGET"),
        (auto, _estimate(1e6, 1, 0), 0.01, "AUTO_SUBSAMPLE_HIGH_CONFIDENCE"),   # clamp(0.01, 1.0)
        (dict(enable_auto_subsample=True, depth=0.0), hi, 1.0, "AUTO_SUBSAMPLE_HIGH_CONFIDENCE_WITHIN_TARGET"),
    ]
    for kw, est, f, why in cases:
        assert api.subsample_decide(api.subsample_policy(**kw), est) == (f, why), (kw, why)
    with pytest.raises(N.FbkError):   # main.rs:76-81 rejects a ratio below 1 or not finite
        api.subsample_decide(api.subsample_policy(threshold_ratio=0.5), hi)
    with pytest.raises(N.FbkError):
        api.subsample_decide(api.subsample_policy(threshold_ratio=float("nan")), hi)


def test_host_only_calls_at_their_edges():
    """Host-only calls on edge inputs: sketch widths clamp at both ends (sketch.rs:165-168)
    without overflowing g * 16; register estimates refuse what they cannot read; the
    k ladder can be counted without an output buffer."""
    lib = N.lib()
    assert lib.fbk_cms_width_for_genome_size(0) == 1 << 21
    assert lib.fbk_cms_width_for_genome_size(1_000_000) == 1 << 24
    assert lib.fbk_cms_width_for_genome_size(5_000_000) == 1 << 27
    for g in ((1 << 27) // 16, (1 << 27) // 16 + 1, 1 << 59, (1 << 60) + 1, (1 << 64) - 1):
        assert lib.fbk_cms_width_for_genome_size(g) == 1 << 27
    regs = np.zeros(1 << 14, dtype=np.uint8)
    ptr = regs.ctypes.data_as(C.POINTER(C.c_uint8))
    assert lib.fbk_hll_estimate_registers(ptr, 14) == 0.0   # all registers empty: zero cardinality
    for p in (3, 19, 64):
        assert np.isnan(lib.fbk_hll_estimate_registers(ptr, p))
    assert np.isnan(lib.fbk_hll_estimate_registers(None, 14))
    n = lib.fbk_compute_dynamic_kmers(150, -1, None, 16)
    assert n == len(api.compute_dynamic_kmers(150)) and n > 0


def test_single_pair_helpers_refuse_missing_buffers():
    lib = N.lib()
    assert lib.fbk_trim_adapter(None, 10) == 0
    assert lib.fbk_trim_quality(None, None, 10, 20, 5) == -1
    seq = np.frombuffer(b"ACGT" * 10, dtype=np.uint8)
    ptr = seq.ctypes.data_as(C.POINTER(C.c_uint8))
    assert lib.fbk_merge_read_pair(ptr, None, len(seq), None, None, len(seq), 10, 0.1, None, None, None) == -1
    assert lib.fbk_merge_read_pair(ptr, None, len(seq), ptr, None, len(seq), 10, 0.1, None, None, None) == -1


def test_cohort_draws_stay_in_their_ranges():
    """Cohort members (batches and serving) come from a splitmix64 stream per seed:
    genome 2-7 Mbp, GC 0.30-0.68, depth 30-200x, the same values on every call."""
    from fastbact_gb300 import cohort

    draws = [cohort.draw(1000 + i) for i in range(64)]
    assert draws == [cohort.draw(1000 + i) for i in range(64)]
    for d in draws:
        assert 2_000_000 <= d["genome_len"] <= 7_000_000
        assert 0.30 <= d["gc"] <= 0.68
        assert 30.0 <= d["coverage"] <= 200.0
    assert len({d["genome_len"] for d in draws}) == 64
    assert any(d["coverage"] > 150.0 for d in draws) and any(d["coverage"] < 110.0 for d in draws)
    small = cohort.draw(1000, scale=0.001)
    assert small["genome_len"] == 20_000 and small["gc"] == draws[0]["gc"]
    m = cohort.make(1, first_seed=1000, scale=0.002, sample_pairs=5000)[0]
    assert m.params == cohort.draw(1000, scale=0.002)
    assert m.sample_pairs == min(5000, m.stats.exact_read_pairs) and len(m.sample) == 2 * m.sample_pairs
    assert m.ingest.input_read_pairs == m.stats.exact_read_pairs
    assert cohort.policy().threshold_ratio == 150.0 / 110.0


def test_headers_compile_as_strict_c_and_link(tmp_path):
    """The C ABI is usable from plain C (cgo, bindgen and ctypes callers see the same
    declarations): both headers compile as C11 with -pedantic -Werror, and a C program
    links against the library and calls host-only entry points."""
    import shutil
    gcc = shutil.which("gcc")
    if gcc is None:
        pytest.skip("no C compiler")
    lib_dir = Path(N.lib()._name).parent
    src = tmp_path / "caller.c"
    src.write_text(
        '#include "fbk.h"\n#include "fbk_synth.h"\n#include <stdio.h>\n'
        "int main(void) {\n"
        '    printf("%s %llu %d\\n", fbk_status_str(FBK_ERR_INVALID),\n'
        "           (unsigned long long)fbk_cms_width_for_genome_size(1000000),\n"
        "           fbk_ctx_set_tuning(NULL, \"stripes\", 8.0));\n"
        "    return 0;\n}\n")
    exe = tmp_path / "caller"
    r = subprocess.run([gcc, "-std=c11", "-Wall", "-Wextra", "-Werror", "-pedantic", f"-I{ROOT / 'include'}",
                        str(src), f"-L{lib_dir}", "-lfbk", f"-Wl,-rpath,{lib_dir}", "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
    assert out.returncode == 0, out.stderr
    msg, width, st = out.stdout.split()[:-2], int(out.stdout.split()[-2]), int(out.stdout.split()[-1])
    assert " ".join(msg) == N.lib().fbk_status_str(1).decode()
    assert width == 1 << 24 and st == 1


STRUCT_MIRRORS = {
    "fbk_arena_view": "ArenaView", "fbk_count_stats": "CountStats", "fbk_genome_estimate": "GenomeEstimate",
    "fbk_estimator_params": "EstimatorParams", "fbk_subsample": "Subsample", "fbk_build_params": "BuildParams",
    "fbk_subsample_policy": "SubsamplePolicy", "fbk_batch_params": "BatchParams", "fbk_batch_result": "BatchResult",
    "fbk_batch_stats": "BatchStats", "fbk_ingest_stats": "IngestStatsC", "fbk_server_params": "ServerParams",
    "fbk_request_info": "RequestInfo", "fbk_server_stats": "ServerStats", "fbk_synth_params": "SynthParams",
}


def test_ctypes_mirrors_match_the_c_layouts(tmp_path):
    """Every struct of the C headers has a ctypes mirror with the same size and the same
    field offsets (measured by the C compiler), and every declared function is bound with
    as many arguments as the header declares."""
    import shutil
    gcc = shutil.which("gcc")
    if gcc is None:
        pytest.skip("no C compiler")
    declared = set()
    for h in (ROOT / "include").glob("*.h"):
        declared |= set(re.findall(r"\}\s*(fbk_\w+);", h.read_text()))
    assert declared == set(STRUCT_MIRRORS)
    lines = ['#include "fbk.h"', '#include "fbk_synth.h"', "#include <stddef.h>", "#include <stdio.h>",
             "int main(void) {"]
    for cname, pyname in STRUCT_MIRRORS.items():
        py = getattr(N, pyname)
        lines.append(f'    printf("{cname} size %zu\\n", sizeof({cname}));')
        for fname, _ in py._fields_:
            lines.append(f'    printf("{cname} {fname} %zu\\n", offsetof({cname}, {fname}));')
    lines += ["    return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    r = subprocess.run([gcc, "-std=c11", f"-I{ROOT / 'include'}", str(src), "-o", str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60).stdout.split("\n")
    for ln in filter(None, out):
        cname, what, val = ln.split()
        py = getattr(N, STRUCT_MIRRORS[cname])
        got = C.sizeof(py) if what == "size" else getattr(py, what).offset
        assert got == int(val), (cname, what, got, val)
    # argument counts of every declared function
    for h in (ROOT / "include").glob("*.h"):
        txt = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        for m in re.finditer(r"FBK_API\s+[^;{]*?\b(fbk_\w+)\s*\(([^;]*?)\)\s*;", txt, flags=re.S):
            name, params = m.group(1), m.group(2).strip()
            n = 0 if params in ("", "void") else params.count(",") + 1
            sig = N.SIGNATURES.get(name) or N.SYNTH_SIGNATURES.get(name)
            assert sig is not None, name
            assert len(sig[1]) == n, (name, len(sig[1]), n)
