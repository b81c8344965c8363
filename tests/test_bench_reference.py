"""The bench's reference arm (`bench.py --impl reference`) on the CPU: it times
the oracle (the CPU restatement of the reference's shaders) on the mid scene
read and packed by the oracle alone, prints the same metric and config block
as the GPU arm, and never maps the product library (libptgpu.so) into its
process — the ratio the two arms give would otherwise compare the product
with itself."""
import json
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent


def test_reference_arm_runs_the_oracle_alone():
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--steps", "1", "--warmup", "0",
                        "--ref-seconds", "1"], cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads([x for x in r.stdout.splitlines() if x.startswith("{")][-1])
    assert line["impl"] == "reference"
    assert line["unit"] == "Mpath-segs/s" and line["value"] > 0 and line["higher_is_better"] is True
    assert line["config"]["workload"].startswith("mid scene: 1024x1024, 128 spp")
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["cores"] >= 1
    assert line["e2e"]["value"] == line["value"] and line["e2e"]["h2d_bytes_per_step"] == 0
    libs = line["native_libraries"]
    assert any(lib.endswith("liboracle.so") for lib in libs), libs
    assert not any("libptgpu" in lib for lib in libs), libs
