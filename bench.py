#!/usr/bin/env python3
"""Benchmark of the GB300 k-mer counting front end.

Workload (one step): the isolate-scale configuration — a synthetic 5 Mbp genome
(GC 0.51, seven inserted 5 kb repeat copies at >= 99% identity), 150 bp pairs at
100x (1.67M pairs), fragments N(350, 30), 0.5% substitutions, Phred 30-40 with the
last 20 bases decaying to 15, ingested (trim/merge) into a ReadBank.  A step runs
the genome estimator (ntHash k=21 + CMS 4 x 2^23 nibbles + two HLL p=14 over the
first <= 150k raw pairs, with the reference's early stop) and then the build front
end (pass-1 CMS 4 x 2^24 u16, pass-2 solid table, SolidKmerNode conversion) for
the multi-k pass k = 21, 33, 55 (64/128-bit keys) and 77 (256-bit keys).

Metric: k-mers/s = (estimator k-mer occurrences consumed + pass-1 and pass-2 k-mer
occurrences of every k) / step time.  `value` keeps the bank and the estimator
sample resident in HBM; `e2e` runs the same step through the C ABI from pinned
host buffers (bank and sample uploaded, every solid table exported every step).

--impl reference times the reference's algorithm on the host cores instead: the
oracle's C++ restatement in its multithreaded (rayon-like) mode, on a bounded
sample of the same workload per step.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

from fastbact_gb300 import workloads  # noqa: E402

PLAIN_MODES = {"plain": workloads.ISOLATE_5MBP, "plain1m": workloads.PLAIN_1MBP}
COUNTER_BITS = 16


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--counter-bits", type=int, default=COUNTER_BITS, choices=[4, 16])
    ap.add_argument("--scale", type=float, default=1.0, help="coverage multiplier (quick runs)")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=15.0, help="budget of the CPU-baseline sample")
    ap.add_argument("--mode", choices=["plain", "plain1m", "batch", "serve", "stress"], default="plain",
                    help="plain: the isolate-scale workload, one isolate per step (the headline line); plain1m: the "
                         "1 Mbp 50x workload; batch: a cohort in multi-isolate waves; serve: Poisson arrivals through "
                         "the request loop; stress: 12 Mbp at 300x, k = 127")
    ap.add_argument("--no-check", action="store_true",
                    help="skip the parity check of the timed step's outputs against the oracle")
    ap.add_argument("--no-counted", action="store_true", help="skip timing the counted-sketch form of the step")
    ap.add_argument("--isolates", type=int, default=64, help="cohort size (batch and serve modes)")
    ap.add_argument("--genome-scale", type=float, default=1.0, help="cohort genome-size multiplier (quick runs)")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", str(rank)))
    return rank, world, local


def kmers_in(bank, k: int, min_len: int) -> int:
    tot = 0
    for a in bank.arenas:
        L = a.lengths.astype(np.int64)
        L = L[L >= min_len]
        tot += int((L - k + 1).sum())
    return tot


# ---------------------------------------------------------------------------
# clocks during the timed region
# ---------------------------------------------------------------------------
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines: list[str] = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                                          "-i", str(self.device), "-lms", "200"], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (FileNotFoundError, OSError):
            self.proc = None

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def stop(self) -> dict:
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.t.join(timeout=2)
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


# ---------------------------------------------------------------------------
# workload
# ---------------------------------------------------------------------------
def make_workload(wl: dict, rank: int, scale: float):
    t0 = time.time()
    p, bank, st, sample, n_sample, stats = workloads.generate(wl, rank=rank, coverage_scale=scale)
    return p, bank, st, sample, n_sample, stats, time.time() - t0


def plain_config(wl: dict, p, bank, stats, scale: float) -> dict:
    """The workload as both arms name it: what was generated, not what came out."""
    return {"workload": wl["text"] + (f" (coverage x{scale})" if scale != 1.0 else ""),
            "genome_len": int(p.genome_len), "pairs": int(stats.exact_read_pairs), "bank_reads": bank.total_reads(),
            "bank_bases": bank.total_bases(), "ks": list(wl["ks"]),
            "cms": f"4 x 2^{wl['cms_log2w']} u16", "hll_p": wl["hll_p"], "t_solid": 2, "min_trans_cov": 3}


def step_kmers(bank, ks) -> dict:
    return {k: (kmers_in(bank, k, k), kmers_in(bank, k, k + 1)) for k in ks}


_PINNED: list = []  # keeps the page-locked blocks alive for the process


def pinned_copy(a: np.ndarray) -> np.ndarray:
    """Copy of `a` in page-locked host memory (torch allocator)."""
    import torch

    t = torch.empty(max(a.nbytes, 8), dtype=torch.uint8, pin_memory=True)
    _PINNED.append(t)
    out = t.numpy().view(a.dtype)[: a.size].reshape(a.shape)
    out[...] = a
    return out


def pinned_bank(bank):
    from fastbact_gb300 import api

    arenas = []
    for a in bank.arenas:
        arenas.append(api.BitSeqArena(pinned_copy(a.data), pinned_copy(a.offsets), pinned_copy(a.lengths),
                                      pinned_copy(a.pair_idx) if a.pair_idx is not None else None))
    return api.ReadBank(*arenas)


def ascii_reads(arena, n: int) -> list:
    """The first n reads of an arena as ASCII (vectorised decode, for the oracle)."""
    if n == 0:
        return []
    end = int(arena.offsets[n - 1]) + int(arena.lengths[n - 1])
    g = np.arange(end, dtype=np.uint64)
    codes = (arena.data[g >> np.uint64(5)] >> ((g & np.uint64(31)) << np.uint64(1))) & np.uint64(3)
    s = np.frombuffer(b"ACGT", np.uint8)[codes.astype(np.intp)].tobytes()
    return [s[int(o):int(o) + int(L)] for o, L in zip(arena.offsets[:n], arena.lengths[:n])]


EST_FIELDS = ("genome_size", "exact_read_pairs", "total_bases", "median_read_len", "max_read_len", "estimated_cov",
              "subsample_factor", "kmers", "n_kmers", "confidence", "u_ge_1", "u_ge_2", "sample_kmer_depth",
              "pairs_sampled", "m_sample")


def parity_check(wl, bank, sample, n_sample, stats, ge, regs, res) -> dict:
    """Checks the timed step's outputs against the oracle on the same inputs: every
    GenomeEstimate field and both HLL register arrays, and per k the SolidKmerNode
    digest and row count (the same order-free digest the device computes)."""
    from fastbact_gb300 import api
    from oracle import orc

    t0 = time.perf_counter()
    out = {"estimate": True, "registers": True, "tables": {}}
    rc, oe, ort, ors = orc.estimate_from_reads(ascii_reads(sample, 2 * n_sample), orc.count_stats(**stats.__dict__),
                                               workloads.EST_MAX_PAIRS, workloads.EST_TARGET_COV, hll_p=wl["hll_p"])
    gc = ge.to_c()
    for f in EST_FIELDS:
        g, o = getattr(gc, f), getattr(oe, f)
        if f == "kmers":
            g, o = list(g), list(o)
        if rc != 0 or g != o:
            out["estimate"] = False
            out.setdefault("estimate_mismatch", []).append(f)
    out["registers"] = bool(np.array_equal(regs[0], ort) and np.array_equal(regs[1], ors))
    for (k, _, n_solid, _, digest) in res:
        _, o_tab, _, mtc = orc.build_front(bank, k, api.key_bits_for_k(k), wl["cms_log2w"], 16, None, threads=0)
        od, on = o_tab.digest(mtc)
        del o_tab
        out["tables"][str(k)] = {"digest_equal": od == digest, "n_solid": n_solid, "n_solid_equal": on == n_solid}
    out["ok"] = out["estimate"] and out["registers"] and all(
        v["digest_equal"] and v["n_solid_equal"] for v in out["tables"].values())
    out["seconds"] = time.perf_counter() - t0
    out["what"] = ("oracle (C++ restatement of the reference) on the same inputs: every GenomeEstimate field, both "
                   "HLL register arrays, per k the SolidKmerNode digest and count of the last timed step")
    return out


# ---------------------------------------------------------------------------
# our arm
# ---------------------------------------------------------------------------
def env_tuning(ctx) -> dict:
    """Tuning values from FBK_TUNE ("name=value,name=value"), set on the context."""
    tune = {}
    for kv in filter(None, os.environ.get("FBK_TUNE", "").split(",")):
        name, v = kv.split("=")
        tune[name] = float(v)
    if tune:
        ctx.set_tuning(**tune)
    return tune


def run_ours(args, rank, world, local):
    import torch

    from fastbact_gb300 import api
    from fastbact_gb300.build import build

    build()
    torch.cuda.set_device(local)
    if world > 1:
        torch.distributed.init_process_group("nccl", device_id=torch.device("cuda", local))

    wl = PLAIN_MODES[args.mode]
    KS, LOG2W, HLL_P = wl["ks"], wl["cms_log2w"], wl["hll_p"]
    p, bank, ist, sample, n_sample, stats, gen_s = make_workload(wl, rank, args.scale)
    ctx = api.Context(local, pool_bytes=int(os.environ.get("FBK_POOL_BYTES", str(60 << 30))))
    tune = env_tuning(ctx)
    dbank = api.DeviceBank(ctx, bank)
    dsample = api.DeviceBank(ctx, sample)
    ctx.sync()
    cb = COUNTER_BITS

    def step(ctx, dbank, dsample, sample_lengths, export=False, outs=None):
        ge, _, _ = api.estimate_bank(ctx, dsample, sample_lengths, n_sample, stats, max_pairs=workloads.EST_MAX_PAIRS,
                                     target_cov=workloads.EST_TARGET_COV, hll_p=HLL_P)
        res = []
        prev = None  # a table whose rows are still being copied out while the next k builds
        for k in KS:
            t = api.build_cdbg_ext(dbank, k, None, ge.genome_size, ctx=ctx, counter_bits=cb, cms_log2_width=LOG2W)
            info = t.info()
            res.append((k, info[0], info[1], t.pushes(), t.digest()[0]))
            if prev is not None:
                prev.export_wait()
                prev.release()
                prev = None
            if export:
                o = outs.get(k) if outs else None
                if o is not None and len(o[1]) >= info[1]:
                    t.export_async(o)  # page-locked buffers kept from step to step
                    prev = t
                    continue
                t.export(out=o)
            t.release()
        if prev is not None:
            prev.export_wait()
            prev.release()
        return ge, res

    sample_len = np.ascontiguousarray(sample.lengths)
    for _ in range(args.warmup):
        ge, res = step(ctx, dbank, dsample, sample_len)
    kmers_est = ge.m_sample
    kmers_pass = step_kmers(bank, KS)
    kmers_build = sum(a + b for a, b in kmers_pass.values())
    kmers_step = kmers_est + kmers_build

    def timed_region(n_steps):
        clocks = ClockSampler(local)
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()
        ctx.sync()
        ctx.timing_reset()
        ctx.set_timing(True)
        launches0 = ctx.launch_count()
        clocks.start()
        ctx.record(0)
        for _ in range(n_steps):
            out = step(ctx, dbank, dsample, sample_len)
        ctx.record(1)
        ms = ctx.elapsed_ms(0, 1)
        clk = clocks.stop()
        ctx.sync()
        torch.cuda.synchronize()
        launches = ctx.launch_count() - launches0
        kms = {n: ctx.timing(n) for n in ("pass1", "solid", "pass2_emit", "pass2_count", "pass2_upsert", "pass2_direct",
                                          "convert", "table_init", "est_", "clamp", "cms_clamp", "subsample", "")}
        ctx.set_timing(False)
        if world > 1:
            t = torch.tensor([ms], dtype=torch.float64, device="cuda")
            torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
            ms = float(t.item())
        return out, ms, clk, launches, kms

    # ---- device-resident timed region -------------------------------------------
    (ge, res), ms, clk, launches, kernel_ms = timed_region(args.steps)
    total_kmers = kmers_step * args.steps * world
    value = total_kmers / (ms / 1e3)

    # ---- one more (untimed) step with the device time of each k's kernel families ----
    per_k = {}
    ctx.set_timing(True)
    for k in KS:
        ctx.sync()
        ctx.timing_reset()
        t = api.build_cdbg_ext(dbank, k, None, ge.genome_size, ctx=ctx, counter_bits=cb, cms_log2_width=LOG2W)
        t.release()
        ctx.sync()
        per_k[str(k)] = {f: round(ctx.timing(f)[0], 3) for f in ("pass1", "pass2_emit", "pass2_count", "pass2_upsert",
                                                                  "convert", "table_init") if ctx.timing(f)[0] > 0}
    ctx.set_timing(False)

    # ---- the same step with the counted u16 sketch (what a caller asking for the
    # sketch gets); the headline keeps only the t_solid-level gate ladder -----------
    counted = None
    if not args.no_counted:
        old_mode = ctx.get_tuning("sketch_mode")
        ctx.set_tuning(sketch_mode=0)
        step(ctx, dbank, dsample, sample_len)
        (_, res_c), ms_c, clk_c, _, kms_c = timed_region(max(1, min(args.steps, 5)))
        ctx.set_tuning(sketch_mode=old_mode)
        n_c = max(1, min(args.steps, 5))
        counted = {"value": kmers_step * n_c * world / (ms_c / 1e3), "unit": "k-mers/s", "ms_per_step": ms_c / n_c,
                   "steps": n_c, "same_tables": [r[4] for r in res_c] == [r[4] for r in res],
                   "kernel_ms_per_step": {k: v[0] / n_c for k, v in kms_c.items() if v[0] > 0 and k},
                   "clocks": clk_c,
                   "what": "pass 1 keeps exact u32 counts (read as u16 saturating), 4 row-slice sweeps, solidity "
                           "bitmap from the counts; same tables as the ladder gate"}

    # ---- roofline of the dominant pass --------------------------------------------
    # Algorithmic bytes per pass (per k-mer occurrence): pass 1 = packed input +
    # 4 counters read and written (8 c_b); pass 2 = packed input + 4 counters read
    # (4 c_b) + 2 x (entry read + written) per transition push, entry = key + cov (2)
    # + 8 edge counters (16); c_b = 2 bytes (u16 sketch).
    c_b = 2.0
    bank_bytes = bank.total_bases() / 4.0
    key_bytes = {k: 8 * (api.key_bits_for_k(k) // 64) for k in KS}
    pushes = {r[0]: r[3] for r in res}
    fam_ms = {
        "pass1": kernel_ms["pass1"][0],
        "pass2": kernel_ms["solid"][0] + kernel_ms["pass2_emit"][0] + kernel_ms["pass2_count"][0]
                 + kernel_ms["pass2_upsert"][0] + kernel_ms["pass2_direct"][0],
    }
    alg = {
        "pass1": sum(bank_bytes + kmers_pass[k][0] * 8 * c_b for k in KS),
        "pass2": sum(bank_bytes + kmers_pass[k][1] * 4 * c_b + pushes[k] * 2 * (key_bytes[k] + 2 + 16) for k in KS),
    }
    dom = max(fam_ms, key=fam_ms.get)
    per_pass_ms = fam_ms[dom] / (args.steps * len(KS))
    per_pass_bytes = alg[dom] / len(KS)
    achieved = per_pass_bytes / (per_pass_ms / 1e3) / 1e9
    peaks_path = ROOT / "MEASURED_PEAKS.json"
    if peaks_path.exists():
        peak = json.loads(peaks_path.read_text())["hbm_gbs"]
        peak_src = "measured"
    else:
        peak = 6800.0
        peak_src = "fallback"
    traffic, traffic_src = None, None
    tpath = ROOT / "profiles" / "traffic.txt"
    if tpath.exists() and args.mode == "plain":
        for ln in tpath.read_text().splitlines():
            f = ln.split()
            if len(f) >= 2 and f[0] == f"{dom}_u16":
                traffic, traffic_src = float(f[1]), ("mean DRAM bytes of one pass (one k) of pass 2 in the full-size "
                                                      "ncu capture of profiles/pass2_traffic_isolate5M_100x.md")

    # ---- end to end through the C ABI from pinned host memory ------------------------
    e2e = None
    if not args.no_e2e:
        pb = pinned_bank(bank)
        ps = api.BitSeqArena(pinned_copy(sample.data), pinned_copy(sample.offsets), pinned_copy(sample.lengths))
        h2d = sum(a.data.nbytes + a.offsets.nbytes + a.lengths.nbytes + (a.pair_idx.nbytes if a.pair_idx is not None else 0)
                  for a in pb.arenas) + ps.data.nbytes + ps.offsets.nbytes + ps.lengths.nbytes

        # the solid rows land in pinned host buffers that a caller keeps from step to
        # step (sized from the warm-up step; a larger table gets fresh arrays)
        outs = {}

        def e2e_step():
            # the sample first (the estimate reads it); the bank's copies then run on the
            # copy stream while the estimate runs, and each table's rows are copied out
            # while the next k builds
            ds = api.DeviceBank(ctx, ps)
            db = api.DeviceBank(ctx, pb, async_upload=True)
            ge2, res2 = step(ctx, db, ds, ps.lengths, export=True, outs=outs)
            db.release()
            ds.release()
            return ge2, res2

        _, res0 = e2e_step()
        for (k, _, n_solid, _, _) in res0:
            nw = key_bytes[k] // 8
            outs[k] = (pinned_copy(np.zeros((n_solid, nw), np.uint64)), pinned_copy(np.zeros(n_solid, np.uint16)),
                       pinned_copy(np.zeros(n_solid, np.uint8)))
        e2e_step()
        if world > 1:
            torch.distributed.barrier()
        ctx.sync()
        t0 = time.perf_counter()
        ctx.record(2)
        for _ in range(args.steps):
            ge2, res2 = e2e_step()
        ctx.record(3)
        e_ms = ctx.elapsed_ms(2, 3)
        wall = (time.perf_counter() - t0) * 1e3
        e_ms = max(e_ms, wall)
        if world > 1:
            t = torch.tensor([e_ms], dtype=torch.float64, device="cuda")
            torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
            e_ms = float(t.item())
        d2h = sum(n_solid * ((key_bytes[k]) + 2 + 1) for (k, _, n_solid, _, _) in res2)
        e2e = {"value": total_kmers / (e_ms / 1e3), "unit": "k-mers/s", "h2d_bytes_per_step": int(h2d),
               "d2h_bytes_per_step": int(d2h), "ms_per_step": e_ms / args.steps,
               "same_tables": [r[4] for r in res2] == [r[4] for r in res],
               "overlap": "bank copies on the copy stream during the genome estimate (fbk_bank_upload_async); "
                          "each table's rows copied out while the next k builds (fbk_table_export_async)"}

    # ---- parity of the timed step against the oracle ----------------------------
    parity = None
    if rank == 0 and not args.no_check:
        _, rt, rs = api.estimate_bank(ctx, dsample, sample_len, n_sample, stats, want_registers=True,
                                      max_pairs=workloads.EST_MAX_PAIRS, target_cov=workloads.EST_TARGET_COV,
                                      hll_p=HLL_P)
        parity = parity_check(wl, bank, sample, n_sample, stats, ge, (rt, rs), res)

    # ---- CPU baseline (oracle restatement, bounded sample) ------------------------
    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        cpu = cpu_arm(wl, bank, sample, n_sample, stats, budget_s=args.cpu_seconds, single_s=3.0)

    if rank == 0:
        est_ms = kernel_ms["est_"][0] / args.steps
        build_ms = ms / args.steps - est_ms
        line = {
            "metric": "k-mers/s ntHash+CMS+HLL+count (estimator + multi-k build front end)",
            "value": value, "unit": "k-mers/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "u64/u16 integer", "data": "synthetic (seeded generator; no dataset)",
            "config": dict(plain_config(wl, p, bank, stats, args.scale),
                           parallelism=f"replicas x{world} (one isolate per GPU)",
                           l2="inputs larger than L2: bank + 4 x 2^w sketch gate + solid tables of GBs per k"),
            "parity_checked": bool(parity and parity["ok"]),
            "parity": parity,
            "results": {"estimator_kmers": kmers_est, "pass_kmers": {str(k): kmers_pass[k] for k in KS},
                        "solid": {str(r[0]): r[2] for r in res}, "table_keys": {str(r[0]): r[1] for r in res},
                        "digests": {str(r[0]): hex(r[4]) for r in res}, "genome_size_est": ge.genome_size,
                        "generation_s": round(gen_s, 1), "tuning": tune,
                        "gate": "t_solid-level threshold ladder (exact: the gate reads only min_r count_r >= t_solid)"},
            "stages": {"estimator": {"kmers": kmers_est, "ms_per_step": est_ms,
                                     "kmers_per_s": kmers_est / (est_ms / 1e3) if est_ms > 0 else None,
                                     "note": "device kernel time of the estimator stages"},
                       "build": {"kmers": kmers_build, "ms_per_step": build_ms,
                                 "kmers_per_s": kmers_build / (build_ms / 1e3),
                                 "note": "step time minus the estimator kernels"}},
            "counted_sketch": counted,
            "kernel_ms": {k or "all": {"ms": v[0], "launches": v[1]} for k, v in kernel_ms.items()},
            "kernel_ms_per_k": per_k,
            "roofline": {"kernel": ({"pass1": "pass 1 (k_pass1_sweep: 4 row-slice sweeps)",
                                     "pass2": "pass 2 (k_solid_sweep + k_emit + k_upsert)"} if kernel_ms["solid"][0] > 0 else
                                    {"pass1": "pass 1 (k_ladder_pass1 / k_ladder_pass1_roll: one sweep, t_solid-level "
                                               "gate ladder)",
                                     "pass2": "pass 2 (record emit k_emit_roll / k_emit_flat + k_count_records + "
                                              "k_upsert / k_upsert_all)"})[dom],
                         "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "peak_source": peak_src, "traffic": traffic,
                         "traffic_source": traffic_src,
                         "alg_bytes_per_pass": per_pass_bytes, "ms_per_pass": per_pass_ms,
                         "note": "per pass = one k of one step; achieved = algorithmic bytes / event-timed kernel time"},
            # the second figure the path is bound by: L2 atomics, counted as the edge-counter
            # atomics of the upserts (one per transition push) over the upsert time
            "l2_atomics": {"kind": "edge-counter atomics of pass 2 (one per transition push)",
                           "ops_per_step": sum(pushes.values()),
                           "per_s": sum(pushes.values()) * args.steps / (kernel_ms["pass2_upsert"][0] / 1e3)
                           if kernel_ms["pass2_upsert"][0] > 0 else None},
            "gpu_launches": launches,
            "clocks": clk,
            "e2e": e2e,
            "cpu_baseline": cpu,
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()
    ctx.close()
    if parity is not None and not parity["ok"]:
        sys.exit(1)


# ---------------------------------------------------------------------------
# batch mode: a cohort counted in multi-isolate waves vs one isolate at a time
# ---------------------------------------------------------------------------
BATCH_K, BATCH_LOG2W = 31, 22


def plain_isolate(api, ctx, dbank, dsample, m):
    """The one-isolate-at-a-time GPU path for a cohort member: estimate, policy,
    build front end at k = 31 (CMS 4 x 2^22 u16)."""
    from fastbact_gb300 import cohort

    ge, _, _ = api.estimate_bank(ctx, dsample, m.sample.lengths, m.sample_pairs, m.stats, max_pairs=250_000, target_cov=110.0)
    f, _ = api.subsample_decide(cohort.policy(), ge)
    t = api.build_cdbg_ext(dbank, BATCH_K, None, ctx=ctx, key_bits=64, counter_bits=16, cms_log2_width=BATCH_LOG2W,
                           subsample=(f, 0))
    return ge, f, t


def run_batch_mode(args):
    import torch

    from fastbact_gb300 import api, cohort
    from fastbact_gb300.build import build

    build()
    torch.cuda.set_device(0)
    t0 = time.time()
    members = cohort.make(args.isolates, scale=args.genome_scale)
    gen_s = time.time() - t0
    ctx = api.Context(0, pool_bytes=int(os.environ.get("FBK_POOL_BYTES", str(200 << 30))))
    tune = env_tuning(ctx)
    params = api.batch_params(policy=cohort.policy(), k=BATCH_K, cms_log2_width=BATCH_LOG2W, counter_bits=16)
    b = api.Batch(ctx, params)
    # warm-up (and autotuning) on the first two members
    ids = [b.submit(m.bank, m.sample, m.sample_pairs, m.stats) for m in members[:2]]
    b.run()
    for i in ids:
        b.drop(i)
    tune_ms = b.stats().tune_ms

    # ---- batched, inputs resident in HBM ------------------------------------------
    ids = [b.submit(m.bank, m.sample, m.sample_pairs, m.stats) for m in members]
    ctx.sync()
    s0 = b.stats()
    launches0 = ctx.launch_count()
    clocks = ClockSampler(0)
    clocks.start()
    t0 = time.perf_counter()
    b.run()
    ctx.sync()
    batch_s = time.perf_counter() - t0
    clk = clocks.stop()
    s1 = b.stats()
    res = [b.result(i) for i in ids]
    digests = [(r.digest, r.n_solid, r.n_keys) for r in res]
    kmers = sum(r.kmers + r.estimate.m_sample for r in res)
    for i in ids:
        b.drop(i)

    # ---- batched, end to end from pinned host memory ------------------------------
    pinned = [(pinned_bank(m.bank), api.BitSeqArena(pinned_copy(m.sample.data), pinned_copy(m.sample.offsets),
                                                    pinned_copy(m.sample.lengths)), m) for m in members]
    h2d = sum(sum(a.data.nbytes + a.offsets.nbytes + a.lengths.nbytes + (a.pair_idx.nbytes if a.pair_idx is not None else 0)
                  for a in pb.arenas) + ps.data.nbytes + ps.offsets.nbytes + ps.lengths.nbytes for pb, ps, _ in pinned)
    ctx.sync()
    t0 = time.perf_counter()
    ids = [b.submit(pb, ps, m.sample_pairs, m.stats) for pb, ps, m in pinned]
    b.run()
    d2h = 0
    for i in ids:
        t = b.take_table(i)
        keys, cov, mask = t.export()
        d2h += keys.nbytes + cov.nbytes + mask.nbytes
        t.release()
        b.drop(i)
    e2e_s = time.perf_counter() - t0

    # ---- one isolate at a time (same device-resident inputs) -----------------------
    dev = [(api.DeviceBank(ctx, m.bank), api.DeviceBank(ctx, m.sample), m) for m in members]
    ctx.sync()
    t0 = time.perf_counter()
    plain = []
    for dbank, dsample, m in dev:
        ge, f, t = plain_isolate(api, ctx, dbank, dsample, m)
        info = t.info()
        plain.append((t.digest()[0], info[1], info[0]))
        t.release()
    ctx.sync()
    plain_s = time.perf_counter() - t0
    for dbank, dsample, _ in dev:
        dbank.release()
        dsample.release()
    mismatches = sum(1 for a, c in zip(digests, plain) if a != c)
    st = b.stats()
    b.release()

    # ---- diagnostics: per-kernel device time of both paths (stream launches, events) --
    fams = ("batch_pass1", "batch_solid", "batch_count", "batch_emit", "batch_prefix", "batch_filter", "batch_upsert", "pass1", "solid",
            "pass2_emit", "pass2_count", "pass2_upsert", "pass2_direct", "table_init", "convert", "est_", "subsample", "clamp")

    def timed_families(fn):
        ctx.sync()
        ctx.timing_reset()
        ctx.set_timing(True)
        fn()
        ctx.sync()
        out = {f: round(ctx.timing(f)[0], 2) for f in fams}
        ctx.set_timing(False)
        return {f: v for f, v in out.items() if v > 0}

    def diag_batch():
        bd = api.Batch(ctx, api.batch_params(policy=cohort.policy(), k=BATCH_K, cms_log2_width=BATCH_LOG2W, counter_bits=16,
                                             use_graphs=0, autotune=0))
        ids_d = [bd.submit(m.bank, m.sample, m.sample_pairs, m.stats) for m in members]
        bd.run()
        bd.release()

    def diag_plain():
        for m in members:
            db, ds = api.DeviceBank(ctx, m.bank), api.DeviceBank(ctx, m.sample)
            _, _, t = plain_isolate(api, ctx, db, ds, m)
            t.release()
            db.release()
            ds.release()

    diag = {"batch_ms": timed_families(diag_batch), "plain_ms": timed_families(diag_plain)}
    line = {
        "metric": "isolates/h (batched k=31 counting front end: estimator + subsampling policy + passes 1-2)",
        "value": args.isolates / batch_s * 3600.0, "unit": "isolates/h", "n_gpus": 1, "steps": 1, "warmup": 1,
        "ms_per_step": batch_s * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "u64/u16 integer", "data": "synthetic cohort (seeded generator; no dataset)",
        "config": {"workload": f"cohort of {args.isolates} isolates: genome 2-7 Mbp x{args.genome_scale}, GC 0.30-0.68, "
                               "depth 30-200x, PE150; >150x subsampled to 110x; k=31, CMS 4 x 2^22 u16, HLL p=14",
                   "isolates": args.isolates, "bank_bases": int(sum(m.bank.total_bases() for m in members)),
                   "subsampled": int(sum(1 for r in res if r.subsample_factor < 1.0)),
                   "generation_s": round(gen_s, 1), "tuning": tune},
        "plain": {"value": args.isolates / plain_s * 3600.0, "unit": "isolates/h", "seconds": plain_s},
        "kmers_per_s": kmers / batch_s,
        "identical_to_plain": mismatches == 0, "mismatches": mismatches,
        "e2e": {"value": args.isolates / e2e_s * 3600.0, "unit": "isolates/h", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h), "seconds": e2e_s},
        "batch": {"waves": s1.waves - s0.waves, "fallbacks": s1.fallbacks - s0.fallbacks,
                  "graphs": s1.graph_launches - s0.graph_launches,
                  "ms_estimate": s1.ms_estimate - s0.ms_estimate, "ms_phase_a": s1.ms_phase_a - s0.ms_phase_a,
                  "ms_phase_b": s1.ms_phase_b - s0.ms_phase_b, "ms_host": s1.ms_host - s0.ms_host,
                  "tune_ms": tune_ms,
                  "shapes": {"pass1": [st.pass1_block, st.pass1_grid, st.pass1_rows],
                             "solid": [st.solid_block, st.solid_grid, st.solid_rows],
                             "emit": [st.emit_block, st.emit_grid], "emit_form": st.emit_form,
                             "upsert": [st.upsert_block, st.upsert_grid]}},
        "gpu_launches": s1.kernel_launches - launches0 if s1.kernel_launches >= launches0 else None,
        "kernel_ms": diag,
        "clocks": clk,
    }
    print(json.dumps(line), flush=True)
    ctx.close()


# ---------------------------------------------------------------------------
# stress mode: 12 Mbp GC 0.66 genome, repeats and a tandem array, 300x, k = 127
# ---------------------------------------------------------------------------
STRESS = workloads.STRESS_12MBP["gen"]


def run_stress_mode(args):
    import torch

    from fastbact_gb300 import api
    from fastbact_gb300.build import build

    build()
    torch.cuda.set_device(0)
    wl = dict(STRESS)
    wl["coverage"] = STRESS["coverage"] * args.scale
    t0 = time.time()
    bank, ist, sample, n_sample, stats = api.synth_isolate(api.synth_params(**wl), threads=0, sample_pairs=150_000)
    gen_s = time.time() - t0
    ctx = api.Context(0, pool_bytes=int(os.environ.get("FBK_POOL_BYTES", str(200 << 30))))
    dbank, dsample = api.DeviceBank(ctx, bank), api.DeviceBank(ctx, sample)
    k, kb, log2w = 127, 256, 26
    runs = {}
    clocks = ClockSampler(0)
    clocks.start()

    def timed(name, fn, kmers):
        ctx.sync()
        ctx.record(0)
        out = fn()
        ctx.record(1)
        ms = ctx.elapsed_ms(0, 1)
        runs[name] = {"ms": ms, "kmers": kmers, "kmers_per_s": kmers / (ms / 1e3)}
        return out

    # estimator with HLL p = 16 over the raw sample
    ge, _, _ = api.estimate_bank(ctx, dsample, sample.lengths, n_sample, stats, max_pairs=250_000, target_cov=110.0, hll_p=16)
    ge, _, _ = timed("estimator_p16", lambda: api.estimate_bank(ctx, dsample, sample.lengths, n_sample, stats, max_pairs=250_000,
                                                                target_cov=110.0, hll_p=16), 0)
    runs["estimator_p16"]["kmers"] = ge.m_sample
    runs["estimator_p16"]["kmers_per_s"] = ge.m_sample / (runs["estimator_p16"]["ms"] / 1e3)
    occ = kmers_in(bank, k, k) + kmers_in(bank, k, k + 1)
    api.build_cdbg_ext(dbank, k, None, ctx=ctx, key_bits=kb, counter_bits=16, cms_log2_width=log2w).release()  # warm-up
    t = timed("full_input", lambda: api.build_cdbg_ext(dbank, k, None, ctx=ctx, key_bits=kb, counter_bits=16,
                                                        cms_log2_width=log2w), occ)
    runs["full_input"].update(dict(zip(("table_keys", "solid", "capacity"), t.info())))
    t.release()
    # the counted sketch, to see its saturation
    t, cms = timed("full_input_counted_sketch", lambda: api.build_cdbg_ext(dbank, k, None, ctx=ctx, key_bits=kb, counter_bits=16,
                                                                            cms_log2_width=log2w, keep_cms=True), occ)
    vals = cms.export().view(np.uint16)
    runs["full_input_counted_sketch"]["saturated_counters"] = float((vals == 65535).mean())
    runs["full_input_counted_sketch"]["max_counter"] = int(vals.max())
    t.release()
    cms.release()
    # subsampled to 110x by the pipeline driver's policy
    f, why = api.subsample_decide(api.subsample_policy(enable_auto_subsample=True, depth=110.0, threshold_ratio=150.0 / 110.0), ge)
    n_pairs = int(stats.exact_read_pairs)
    keep = api.subsample_mask(ctx, n_pairs, f, 0)
    kept = np.unpackbits(keep.view(np.uint8), bitorder="little")[:n_pairs].astype(bool)
    sub = api.select_reads(bank, np.concatenate([kept[a.pair_idx.astype(np.int64)].astype(np.uint8) for a in bank.arenas]))
    occ_sub = kmers_in(sub, k, k) + kmers_in(sub, k, k + 1)
    t = timed("subsampled_110x", lambda: api.build_cdbg_ext(dbank, k, None, ctx=ctx, key_bits=kb, counter_bits=16,
                                                             cms_log2_width=log2w, subsample=(f, 0)), occ_sub)
    runs["subsampled_110x"].update(dict(zip(("table_keys", "solid", "capacity"), t.info())))
    runs["subsampled_110x"]["factor"] = f
    runs["subsampled_110x"]["policy"] = why
    t.release()
    clk = clocks.stop()
    line = {
        "metric": "k-mers/s at k = 127 (stress: 12 Mbp GC 0.66, repeats + tandem array, 300x, 1% subs, 0.05% indels)",
        "value": runs["full_input"]["kmers_per_s"], "unit": "k-mers/s", "n_gpus": 1, "steps": 1, "warmup": 1,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u64x4 integer",
        "data": "synthetic (seeded generator; no dataset)",
        "config": {"workload": "stress: 12 Mbp GC 0.66, 10 x 5 kb repeats, 200 x 60 bp tandem array, PE150 at "
                               f"{wl['coverage']:.0f}x, 1% substitutions, 0.05% indels; k = 127 (256-bit keys), "
                               "CMS 4 x 2^26 u16, estimator HLL p = 16",
                   "bank_reads": bank.total_reads(), "bank_bases": bank.total_bases(), "generation_s": round(gen_s, 1),
                   "genome_size_est": ge.genome_size, "estimated_cov": ge.estimated_cov},
        "runs": runs,
        "clocks": clk,
    }
    print(json.dumps(line), flush=True)
    ctx.close()


# ---------------------------------------------------------------------------
# serve mode: Poisson arrivals through the request loop
# ---------------------------------------------------------------------------
SERVE_RATES = [20.0, 50.0, 100.0, 200.0]  # requests per minute


def run_serve_mode(args):
    import torch

    from fastbact_gb300 import api, cohort
    from fastbact_gb300.build import build

    build()
    torch.cuda.set_device(0)
    t0 = time.time()
    members = cohort.make(args.isolates, scale=args.genome_scale)
    gen_s = time.time() - t0
    n_req = max(8, 3 * args.isolates // 2)
    ctx = api.Context(0, pool_bytes=int(os.environ.get("FBK_POOL_BYTES", str(200 << 30))))
    sp = api.server_params(policy=cohort.policy(), k=BATCH_K, cms_log2_width=BATCH_LOG2W, counter_bits=16,
                           workers=int(os.environ.get("FBK_SERVE_WORKERS", "2")),
                           use_graphs=int(os.environ.get("FBK_SERVE_GRAPHS", "1")))
    srv = api.Server(ctx, sp)

    def consume(i):
        # downstream graph construction takes the resident table
        srv.wait(i)
        t = srv.take_table(i)
        keys, cov, mask = t.export()
        t.release()
        return srv.poll(i)

    for m in members[:2]:  # warm-up and autotuning
        consume(srv.submit(m.bank, m.sample, m.sample_pairs, m.stats))

    def session(arrivals):
        ids, infos = [], {}
        drained = threading.Event()

        def drainer():
            k = 0
            while k < len(arrivals):
                while k >= len(ids):
                    time.sleep(0.0005)
                infos[k] = consume(ids[k])
                k += 1
            drained.set()

        th = threading.Thread(target=drainer, daemon=True)
        th.start()
        start = time.perf_counter()
        for j, ta in enumerate(arrivals):
            d = start + ta - time.perf_counter()
            if d > 0:
                time.sleep(d)
            m = members[j % len(members)]
            ids.append(srv.submit(m.bank, m.sample, m.sample_pairs, m.stats))
        drained.wait()
        lat = np.array([infos[k].t_done_ms - infos[k].t_submit_ms for k in range(len(arrivals))])
        span = max(infos[k].t_done_ms for k in infos) - min(infos[k].t_submit_ms for k in infos)
        return lat, span, [infos[k] for k in range(len(arrivals))]

    # one isolate at a time, end to end from host memory: per-member service times
    plain_ms = []
    for m in members:
        ctx.sync()
        a = time.perf_counter()
        db, ds = api.DeviceBank(ctx, m.bank), api.DeviceBank(ctx, m.sample)
        ge, f, t = plain_isolate(api, ctx, db, ds, m)
        t.export()
        t.release()
        db.release()
        ds.release()
        ctx.sync()
        plain_ms.append((time.perf_counter() - a) * 1e3)

    def fifo_replay(arrivals_s):
        # latency of a one-at-a-time FIFO server with the measured service times
        end, out = 0.0, []
        for j, ta in enumerate(arrivals_s):
            t = ta * 1e3
            st_ = max(t, end)
            end = st_ + plain_ms[j % len(plain_ms)]
            out.append(end - t)
        return np.array(out)

    rng = np.random.default_rng(7)
    rates = {}
    clocks = ClockSampler(0)
    clocks.start()
    for rate in SERVE_RATES:
        arr = np.cumsum(rng.exponential(60.0 / rate, n_req))
        arr -= arr[0]
        s0 = srv.stats()
        lat, span, infos = session(list(arr))
        s1 = srv.stats()
        pl = fifo_replay(list(arr))
        rates[str(int(rate))] = {
            "requests": n_req, "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
            "mean_ms": float(lat.mean()), "throughput_iso_per_h": n_req / (span / 1e3) * 3600.0,
            "mean_wave_a": (s1.isolates_a - s0.isolates_a) / max(1, s1.waves_a - s0.waves_a),
            "plain_fifo_p50_ms": float(np.percentile(pl, 50)), "plain_fifo_p99_ms": float(np.percentile(pl, 99)),
            "stage_median_ms": {
                "queue": float(np.median([x.t_admit_ms - x.t_submit_ms for x in infos])),
                "upload": float(np.median([x.t_uploaded_ms - x.t_admit_ms for x in infos])),
                "estimate": float(np.median([x.t_estimated_ms - x.t_uploaded_ms for x in infos])),
                "pass1": float(np.median([x.t_counted_ms - x.t_estimated_ms for x in infos])),
                "pass2": float(np.median([x.t_done_ms - x.t_counted_ms for x in infos])),
            },
        }
    # saturation: every request at once
    s0 = srv.stats()
    lat, span, infos = session([0.0] * n_req)
    s1 = srv.stats()
    clk = clocks.stop()
    burst = {"requests": n_req, "throughput_iso_per_h": n_req / (span / 1e3) * 3600.0,
             "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
             "mean_wave_a": (s1.isolates_a - s0.isolates_a) / max(1, s1.waves_a - s0.waves_a),
             "peak_in_flight": s1.peak_in_flight}
    plain_tput = len(plain_ms) / (sum(plain_ms) / 1e3) * 3600.0
    st = srv.stats()
    srv.release()
    line = {
        "metric": "serving latency p50/p99 (ms) under Poisson arrivals 20-200/min; throughput isolates/h",
        "value": burst["throughput_iso_per_h"], "unit": "isolates/h (saturated)", "n_gpus": 1, "steps": len(SERVE_RATES) + 1,
        "warmup": 2, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u64/u16 integer",
        "data": "synthetic cohort (seeded generator; no dataset)",
        "config": {"workload": f"Poisson request stream (seed 7) at 20/50/100/200 per minute, {n_req} requests per rate, "
                               f"drawn from a cohort of {args.isolates} isolates (2-7 Mbp x{args.genome_scale}, GC 0.30-0.68, "
                               "30-200x; >150x subsampled to 110x); k=31, CMS 4 x 2^22 u16; 2 workers",
                   "generation_s": round(gen_s, 1)},
        "rates": rates, "burst": burst,
        "plain": {"throughput_iso_per_h": plain_tput, "mean_service_ms": float(np.mean(plain_ms)),
                  "note": "one isolate at a time end to end (upload, estimate, policy, build, export); latency at each "
                          "rate = FIFO replay of these measured service times on the same arrivals"},
        "server": {"waves_a": st.waves_a, "waves_b": st.waves_b, "peak_in_flight": st.peak_in_flight,
                   "peak_reserved_gb": st.peak_reserved_bytes / 1e9, "budget_gb": st.budget_bytes / 1e9,
                   "failed": st.failed, "busy_ms": st.busy_ms, "device_ms": {"estimate": st.ms_estimate,
                   "phase_a": st.ms_phase_a, "phase_b": st.ms_phase_b}, "requests": st.submitted,
                   "graphs": sp.batch.use_graphs, "workers": sp.workers},
        "clocks": clk,
    }
    print(json.dumps(line), flush=True)
    ctx.close()


# ---------------------------------------------------------------------------
# CPU arm: the oracle restatement of the reference algorithm, multithreaded
# ---------------------------------------------------------------------------
def cpu_arm(wl, bank, sample, n_sample, stats, budget_s: float, threads: int = 0, single_s: float = 0.0):
    """Times the reference algorithm on the host cores, with the GPU step's mix of work.

    The estimator's sample loop (sequential in the reference, estimator.rs:309-379) runs
    on its whole sample; the build passes 1-2 for each k (rayon-parallel in the
    reference, build.rs:93-116,243-289) run on a bounded prefix of each arena's reads,
    sized to the budget.  `value` is the step's k-mers (estimator + every pass of every
    k, the GPU step's own count) over the estimator's measured time plus the build
    k-mers at the measured build rate: the same estimator:build mix as the GPU step.
    With single_s > 0 the build passes are also timed on one thread."""
    from fastbact_gb300 import api
    from oracle import orc

    ks, log2w = wl["ks"], wl["cms_log2w"]
    cores = threads or os.cpu_count() or 1
    reads = ascii_reads(sample, 2 * min(n_sample, 150_000))
    ost = orc.count_stats(**stats.__dict__)
    t0 = time.perf_counter()
    rc, oe, _, _ = orc.estimate_from_reads(reads, ost, workloads.EST_MAX_PAIRS, workloads.EST_TARGET_COV,
                                           hll_p=wl["hll_p"])
    t_est = time.perf_counter() - t0
    est_kmers = oe.m_sample

    def sub_bank(frac):
        arenas = []
        for a in bank.arenas:
            n = int(len(a) * frac)
            if n == 0:
                arenas.append(api.BitSeqArena())
                continue
            end_base = int(a.offsets[n - 1]) + int(a.lengths[n - 1])
            nw = (end_base + 31) // 32
            arenas.append(api.BitSeqArena(np.ascontiguousarray(a.data[:nw]), np.ascontiguousarray(a.offsets[:n]),
                                          np.ascontiguousarray(a.lengths[:n])))
        return api.ReadBank(*arenas)

    # calibrate on 0.5% of the reads, then size the sample to the budget
    def run(frac, nt):
        b = sub_bank(frac)
        t = time.perf_counter()
        km = 0
        for k in ks:
            kb = api.key_bits_for_k(k)
            cms, tab, _, _ = orc.build_front(b, k, kb, log2w, 4, None, threads=nt)
            del cms, tab
            km += kmers_in(b, k, k) + kmers_in(b, k, k + 1)
        return km, time.perf_counter() - t

    km, dt = run(0.005, cores)
    rate = km / max(dt, 1e-6)
    full = sum(kmers_in(bank, k, k) + kmers_in(bank, k, k + 1) for k in ks)
    frac = min(1.0, max(0.005, (budget_s - t_est) * rate / max(full, 1)))
    km, dt = run(frac, cores)
    build_rate = km / max(dt, 1e-9)
    step_s = t_est + full / build_rate  # the whole step at the measured stage rates
    out = {"value": (est_kmers + full) / step_s, "unit": "k-mers/s", "cores": cores, "kind": "port",
           "sample": f"estimator sample loop over its whole sample ({est_kmers} k-mers, sequential as in the "
                     f"reference) + passes 1-2 at k={ks} over the first {frac:.3%} of each arena's reads (nibble CMS, "
                     f"64 mutex shards); value = the step's k-mers over estimator time + build k-mers at the build rate",
           "seconds": dt + t_est, "projected_step_s": step_s,
           "stages": {"estimator": {"kmers": est_kmers, "seconds": t_est, "kmers_per_s": est_kmers / max(t_est, 1e-9)},
                      "build": {"kmers_sampled": km, "kmers_step": full, "seconds": dt, "kmers_per_s": build_rate}}}
    if single_s > 0:
        km1, dt1 = run(0.001, 1)
        f1 = min(1.0, max(0.001, single_s * (km1 / max(dt1, 1e-6)) / max(full, 1)))
        km1, dt1 = run(f1, 1)
        r1 = km1 / max(dt1, 1e-9)
        out["single_thread"] = {"value": (est_kmers + full) / (t_est + full / r1), "build_kmers_per_s": r1,
                                "sample": f"passes 1-2 over the first {f1:.3%} of each arena's reads on one thread, "
                                          f"plus the same estimator sample loop (which is sequential anyway)",
                                "seconds": dt1 + t_est}
    return out


def run_reference(args, rank, world):
    if rank != 0:
        return
    if args.mode not in PLAIN_MODES:
        print(json.dumps({"impl": "reference", "unavailable": f"--mode {args.mode} has no CPU counterpart in the "
                          "reference (it counts one isolate per process)"}), flush=True)
        return
    from fastbact_gb300.build import build
    from oracle import orc

    build()  # compiles; loads nothing (the generator and the oracle are host-only libraries)
    orc.build()
    wl = PLAIN_MODES[args.mode]
    p, bank, _, sample, n_sample, stats, _ = make_workload(wl, 0, args.scale)
    per_step = min(args.cpu_seconds, max(5.0, min(20.0, 150.0 / max(args.steps + args.warmup, 1))))
    vals = []
    for i in range(args.warmup + args.steps):
        last = i == args.warmup + args.steps - 1
        r = cpu_arm(wl, bank, sample, n_sample, stats, budget_s=per_step, single_s=3.0 if last else 0.0)
        if i >= args.warmup:
            vals.append(r)
    v = float(np.mean([r["value"] for r in vals]))
    est_rate = float(np.mean([r["stages"]["estimator"]["kmers_per_s"] for r in vals]))
    build_rate = float(np.mean([r["stages"]["build"]["kmers_per_s"] for r in vals]))
    line = {"impl": "reference", "metric": "k-mers/s ntHash+CMS+HLL+count (estimator + multi-k build front end)",
            "value": v, "unit": "k-mers/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": float(np.mean([r["projected_step_s"] for r in vals])) * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "u64/u8 integer", "data": "synthetic (seeded generator; no dataset)",
            "config": dict(plain_config(wl, p, bank, stats, args.scale),
                           parallelism=f"replicas x{world} (one isolate per GPU)",
                           l2="inputs larger than L2: bank + 4 x 2^w sketch gate + solid tables of GBs per k"),
            "stages": {"estimator": {"kmers_per_s": est_rate}, "build": {"kmers_per_s": build_rate}},
            "cpu_baseline": {"value": v, "unit": "k-mers/s", "cores": vals[0]["cores"], "kind": "port",
                             "sample": vals[0]["sample"], "stages": vals[-1]["stages"],
                             "single_thread": vals[-1].get("single_thread")},
            "e2e": {"value": v, "unit": "k-mers/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    rank, world, local = dist_env()
    if args.impl == "reference":
        run_reference(args, rank, world)
    elif args.mode == "batch":
        run_batch_mode(args)
    elif args.mode == "serve":
        run_serve_mode(args)
    elif args.mode == "stress":
        run_stress_mode(args)
    else:
        run_ours(args, rank, world, local)


if __name__ == "__main__":
    main()
