"""The reference's own driver on the GPU: main.cpp and no_communication.cpp,
compiled unmodified from the reference sources and linked against
libgbflow.so in place of gpu.cu, run for 25000 steps of a 15^3 grid (fresh
and restarted from a checkpoint), eager, fused and split drop-in modes.
Every Tecplot file it writes in eager mode must equal, byte for byte, the one
the reference CPU build (cpu.cpp) writes; in fused mode its values must agree
within 1e-8 of each column's scale, in split mode (GBF_DROPIN_MODE=2, the
headline split form) within 1e-6 of it, the scale being a column's largest
magnitude over its plot kind's files
(tests/reference_driver/run_reference_driver.py).

Needs the reference sources, named by GBF_REFERENCE_DIR; skipped without
them (they are not part of this repository).
"""
import json
import os
import pathlib
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu
ROOT = pathlib.Path(__file__).resolve().parents[1]
REF = pathlib.Path(os.environ["GBF_REFERENCE_DIR"]) if os.environ.get("GBF_REFERENCE_DIR") else None


@pytest.mark.skipif(REF is None or not (REF / "main.cpp").exists(), reason="GBF_REFERENCE_DIR unset or sources absent")
def test_unmodified_reference_driver_matches_cpu_build(gpu_lib, tmp_path):
    r = subprocess.run([sys.executable, str(ROOT / "tests" / "reference_driver" / "run_reference_driver.py"),
                        str(REF), str(tmp_path)], capture_output=True, text=True, timeout=1800)
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert lines, r.stdout[-2000:] + r.stderr[-2000:]
    s = json.loads(lines[-1])
    print("\n" + json.dumps(s, indent=1))
    assert r.returncode == 0 and s["ok"]
    for scen in ("fresh", "restart"):
        res = s["scenarios"][scen]
        assert res["files"] >= 15
        for mode in ("gb300_eager", "gb300_fused", "gb300_split"):
            c = res["compare"][mode]
            assert not c["missing"] and c["byte_equal"] + len(c["differing"]) == res["files"]
        assert res["compare"]["gb300_eager"]["byte_equal"] == res["files"]
