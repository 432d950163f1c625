"""bench.py's measurement plumbing, on CPU: the nvidia-smi clock summary
(samples kept inside the timed regions, throttle reasons collected), the
DRAM traffic figures read from the committed ncu summaries, the
summaries' own hygiene (each names the command that made it, and every ncu
command leaves the GPU clocks alone), and the reference arm (built and run
without this package's library, on the GPU arm's workload)."""
import json
import re
import subprocess
import sys
import time
from pathlib import Path

import bench

ROOT = Path(__file__).resolve().parents[1]


def _smi_line(ts, sm, smax=2070, reasons=("Not Active",) * 4):
    stamp = time.strftime("%Y/%m/%d %H:%M:%S", time.localtime(ts)) + f".{int((ts % 1) * 1000):03d}"
    return ", ".join([stamp, "0", str(sm), str(smax), "950.00", "0x0000000000000000", *reasons])


def _sampler(tmp_path, lines, windows):
    c = bench.ClockSampler(0)
    c.path = tmp_path / "clocks.csv"
    c.path.write_text("\n".join(lines) + "\n")
    c.proc = object()          # as if nvidia-smi had been started
    c.windows = windows
    return c


def test_clock_summary_keeps_samples_inside_timed_regions(tmp_path):
    t0 = 1_800_000_000.0
    lines = [_smi_line(t0 + 0.0, 1200),                       # before the timed region: idle clocks
             _smi_line(t0 + 1.0, 2070), _smi_line(t0 + 1.1, 2055),
             _smi_line(t0 + 1.2, 2070, reasons=("Not Active", "Not Active", "Not Active", "Active")),
             _smi_line(t0 + 5.0, 900, reasons=("Active", "Not Active", "Not Active", "Not Active")),  # after
             "garbage line", ""]
    s = _sampler(tmp_path, lines, [(t0 + 0.95, t0 + 1.25)]).summary()
    assert s["samples"] == 3 and s["sampled"] == "timed regions"
    assert s["sm_mhz"] == 2070 and s["sm_max_mhz"] == 2070
    assert s["reasons"] == ["sw_power_cap"]           # hw_slowdown came after the region: not reported


def test_clock_summary_short_regions_use_warmup_samples(tmp_path):
    t0 = 1_800_000_000.0
    lines = [_smi_line(t0 - 5.0, 800), _smi_line(t0 - 1.0, 2070), _smi_line(t0 + 0.5, 2070)]
    s = _sampler(tmp_path, lines, [(t0 + 0.01, t0 + 0.02), (t0 + 0.6, t0 + 0.61)]).summary()
    assert s["samples"] == 2 and s["sm_mhz"] == 2070 and s["sampled"].startswith("warm-up")


def test_clock_summary_without_samples(tmp_path):
    s = _sampler(tmp_path, [], [(0.0, 1.0)]).summary()
    assert s["reasons"] == ["unsampled"] and s["sm_mhz"] is None


def test_traffic_read_from_committed_profiles():
    found = sorted(ROOT.glob("profiles/pull_kernel_pagerank_ref_rmat*.md"))
    assert found
    for p in found:
        scale = re.search(r"rmat(\d+)", p.name).group(1)
        t = bench.ncu_traffic(f"rmat{scale}")
        assert t is not None and t > 1e6, p.name
    assert bench.ncu_traffic("rmat99") is None
    # The headline's layout reads its own capture: the relabelled pull
    # kernel at the headline's scale moves less DRAM than the plain one.
    relabelled, plain = bench.ncu_traffic("rmat26", "relabel"), bench.ncu_traffic("rmat26", "plain")
    assert relabelled is not None and plain is not None and relabelled < plain
    assert bench.layout_cfg("relabel") == {"relabel": 1} and bench.layout_cfg("plain") == {}


def test_profile_summaries_name_their_commands():
    for p in sorted(ROOT.glob("profiles/*")):
        text = p.read_text()
        assert p.suffix in (".md", ".txt"), p.name
        assert re.search(r"[Cc]ommand", text), p.name
        joined = text.replace("\\\n", " ")             # shell line continuations
        for cmd in re.findall(r"ncu\b[^\n]*", joined):
            if cmd.startswith("ncu -i") or "--" not in cmd:
                continue                   # reading a report, or prose naming the tool
            assert "--clock-control none" in cmd, (p.name, cmd[:120])
        assert "/root/" not in text and "_work/" not in text, p.name


def test_reference_arm_runs_without_the_library():
    """The reference arm's graph comes from the oracle; the process never
    imports graphee_gb300 nor maps libgx.so, and its config is the GPU arm's."""
    code = (
        "import runpy, sys, os\n"
        "sys.argv = ['bench.py', '--impl', 'reference', '--scale', '14', '--steps', '1', '--warmup', '0']\n"
        "try:\n"
        "    runpy.run_path('bench.py', run_name='__main__')\n"
        "except SystemExit:\n"
        "    pass\n"
        "maps = open('/proc/self/maps').read()\n"
        "print('LIB', any(m.startswith('graphee_gb300') for m in sys.modules), 'libgx.so' in maps)\n")
    r = subprocess.run([sys.executable, "-c", code], cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = r.stdout.strip().splitlines()
    assert lines[-1] == "LIB False False", lines[-1]
    line = json.loads(lines[0])
    assert line["impl"] == "reference" and line["value"] > 0
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["cpu_baseline"]["kind"] in ("port", "reference")
    import graphee_gb300 as gx
    g = gx.rmat_graph(14, 16, seed=bench.SEED, P=bench.SHARDS)

    class A:
        scale, edge_factor, iters = 14, 16, 20
    assert line["config"] == bench.base_config(A, g, 1)
