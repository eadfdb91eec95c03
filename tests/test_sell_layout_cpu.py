"""The sliced operator's slot map (groups of four blocks, then at most three
single blocks per row) compiled from the library's own header and checked
on the host: every slot inside its slice and used once, groups aligned
(tests/sell_layout_probe.cu).  No GPU is needed."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if c and os.path.exists(c):
            return c
    return None


def test_slot_map_covers_each_slot_once(tmp_path):
    nvcc = _nvcc()
    if nvcc is None:
        pytest.skip("nvcc not found")
    exe = str(tmp_path / "sell_layout_probe")
    cmd = [nvcc, "-std=c++17", "-O1", "-I" + os.path.join(ROOT, "include"),
           "-I" + os.path.join(ROOT, "lpm-mac_gb300", "csrc"), os.path.join(ROOT, "tests", "sell_layout_probe.cu"),
           "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and r.stdout.strip() == "ok", r.stdout + r.stderr
