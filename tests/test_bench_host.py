"""bench.py on the CPU: the reference arm (the CPU oracle through the same
workload definition) prints one JSON line with the contract's keys, and the
ncu launch-list summariser turns a --csv log into the per-kernel table and the
per-stage DRAM traffic file that the roofline entry reads."""
from __future__ import annotations

import json
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]


def test_reference_arm_prints_the_contract_line():
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--steps", "2", "--warmup", "1",
                        "--grid", "32", "16", "16"], cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference"
    assert line["metric"] == line["unit"] == "Mcell-steps/s"
    assert line["value"] > 0 and line["steps"] == 2 and line["higher_is_better"] is True
    assert line["config"]["workload"] == "c3_channel" and line["config"]["grid"] == [32, 16, 16]
    cb = line["cpu_baseline"]
    assert cb["kind"] == "port" and cb["value"] == line["value"] and cb["cores"] >= 1
    e2e = line["e2e"]
    assert e2e["value"] == line["value"] and e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0


def _ncu_csv(rows):
    head = '"ID","Process ID","Process Name","Host Name","Kernel Name","Context","Stream","Block Size",' \
           '"Grid Size","Device","CC","Section Name","Metric Name","Metric Unit","Metric Value"\n'
    out = ["==PROF== Connected to process\n", head]
    for i, (name, metric, value) in enumerate(rows):
        out.append(f'"{i // 3}","1","python","h","{name}","1","7","(256, 1, 1)","(64, 1, 1)","0","10.3",'
                   f'"Command line profiler metrics","{metric}","",' f'"{value}"\n')
    return "".join(out)


def test_launch_list_summary_and_stage_traffic(tmp_path):
    rows = []
    # kernel names as ncu's --csv launch list prints them
    for name, t_ns, rd, wr in (("unnamed>::k_codes3_f(const float *, unsigned char *, Geo, int, int *)", 160000, 100e6,
                                5e6),
                               ("unnamed>::k_march_df(DfF, DfF, DfF, DfF, const float *)", 80000, 220e6, 80e6)):
        rows += [(name, "gpu__time_duration.sum", t_ns), (name, "dram__bytes_read.sum", rd),
                 (name, "dram__bytes_write.sum", wr)]
    csv_path = tmp_path / "launches.csv"
    csv_path.write_text(_ncu_csv(rows))
    out = tmp_path / "traffic.json"
    r = subprocess.run([sys.executable, "bench.py", "--summarize-ncu", str(csv_path), "--traffic-out", str(out)],
                       cwd=ROOT, capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr[-2000:]
    table = r.stdout
    assert "| k_codes3_f | 1 | 160.0 |" in table and "| k_march_df | 1 | 80.0 |" in table
    assert "total 240.0 us over 2 launches" in table
    traffic = json.loads(out.read_text())
    assert abs(traffic["eigen"] - 105e6) < 1.0       # one k_codes3_f launch per step
    assert abs(traffic["project"] - 300e6) < 1.0     # one k_march_df launch (k_bc_set absent here)
