"""bench.py's reference arm runs on the host cores alone, so its JSON line can be checked
without a GPU: one line with the keys the measurement contract asks for, the CPU
baseline with its core count, per-stage rates and single-thread figure, an end-to-end
figure with no host-device copies, and no mapping of the device library."""
import json
import os
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent


def test_reference_arm_line():
    env = dict(os.environ, CUDA_VISIBLE_DEVICES="")
    cmd = [sys.executable, "bench.py", "--impl", "reference", "--steps", "1", "--warmup", "0", "--scale", "0.05",
           "--cpu-seconds", "1"]
    r = subprocess.run(cmd, cwd=ROOT, env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    assert d["metric"].startswith("k-mers/s")
    assert d["unit"] == "k-mers/s" and d["higher_is_better"] is True
    assert d["value"] > 0 and d["steps"] == 1 and d["warmup"] == 0
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == d["value"]
    st = cb["single_thread"]
    assert st["value"] > 0 and st["build_kmers_per_s"] > 0
    for stage in ("estimator", "build"):
        assert d["stages"][stage]["kmers_per_s"] > 0
    # the value is the GPU step's mix: estimator time + build k-mers at the build rate
    s = cb["stages"]
    est, bld = s["estimator"], s["build"]
    mix = (est["kmers"] + bld["kmers_step"]) / (est["seconds"] + bld["kmers_step"] / bld["kmers_per_s"])
    assert abs(mix - d["value"]) <= 1e-9 * mix
    assert d["config"]["ks"] == [21, 33, 55, 77] and d["config"]["cms"] == "4 x 2^24 u16"
    e2e = d["e2e"]
    assert e2e["value"] == d["value"] and e2e["unit"] == d["unit"]
    assert e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0


def test_reference_arm_maps_no_device_library():
    """The CPU arm generates its inputs with libfbk_synth.so and times the oracle; the
    device library libfbk.so is never loaded in its process."""
    code = ("import sys, runpy; sys.argv = ['bench.py', '--impl', 'reference', '--steps', '1', '--warmup', '0', "
            "'--scale', '0.02', '--cpu-seconds', '1']\n"
            "runpy.run_path('bench.py', run_name='__main__')\n"
            "maps = open('/proc/self/maps').read()\n"
            "print('MAPPED_LIBFBK' if '/libfbk.so' in maps else 'NO_LIBFBK')\n")
    env = dict(os.environ, CUDA_VISIBLE_DEVICES="")
    r = subprocess.run([sys.executable, "-c", code], cwd=ROOT, env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    assert "NO_LIBFBK" in r.stdout
