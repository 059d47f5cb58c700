"""Register and spill budget of the mixed step kernels, from ptxas's resource
report (no GPU).

The mixed kernels are sized for occupancy by their launch bounds: flux 40
registers (12 blocks of 128 per SM), update and distribute 32 (full
occupancy).  Spills at those budgets cost local-memory traffic on every
triangle (the distribute once moved 1.4 M local loads and stores per 4M-
triangle launch), so this test compiles the unit exactly as the build does
and holds each kernel to its budget.
"""
import os
import re
import shutil
import subprocess

import pytest

from anuga_cuda import _build as B

ENTRY = re.compile(r"Compiling entry function '(_ZN5swgpu\d+(\w+?)ILi(\d+)E\w*|_ZN5swgpu\d+(\w+?)E\w*)'")
SPILL = re.compile(r"(\d+) bytes stack frame, (\d+) bytes spill stores, (\d+) bytes spill loads")
USED = re.compile(r"Used (\d+) registers")


def _report(tmp_path, unit):
    if not (shutil.which("nvcc") or os.path.exists("/usr/local/cuda/bin/nvcc")):
        pytest.skip("nvcc not available")
    cmd = [B._nvcc()] + B.COMMON + B.UNITS[unit] + [
        "-Xptxas", "-v", "-c", os.path.join(B.CSRC, unit), "-o", str(tmp_path / "unit.o")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    out, cur = {}, None
    for line in r.stderr.splitlines():
        m = ENTRY.search(line)
        if m:
            name = m.group(2) or m.group(4)
            cur = (name, int(m.group(3)) if m.group(3) else 0)
            out[cur] = {}
            continue
        if cur is None:
            continue
        m = SPILL.search(line)
        if m:
            out[cur].update(stack=int(m.group(1)), spill_st=int(m.group(2)),
                            spill_ld=int(m.group(3)))
        m = USED.search(line)
        if m:
            out[cur]["regs"] = int(m.group(1))
    return out


def test_mixed_step_kernels_within_budget(tmp_path):
    rep = _report(tmp_path, "swgpu_mixed.cu")
    flux = {k: v for k, v in rep.items() if k[0] == "flux_mixed"}
    upd = {k: v for k, v in rep.items() if k[0] == "update_mixed"}
    dist = {k: v for k, v in rep.items() if k[0] == "distribute_mixed"}
    assert sorted(t for _, t in flux) == [64, 128, 256]
    assert sorted(b for _, b in upd) == [128, 256, 512]
    assert sorted(b for _, b in dist) == [128, 256, 512]
    for k, v in flux.items():
        assert v["regs"] <= 40 and v["spill_st"] == 0 and v["spill_ld"] == 0, (k, v)
    for k, v in upd.items():
        assert v["regs"] <= 32 and v["spill_st"] == 0 and v["spill_ld"] == 0, (k, v)
    for k, v in dist.items():
        assert v["regs"] <= 32 and v["spill_st"] <= 8 and v["spill_ld"] <= 8, (k, v)
    clock = [v for k, v in rep.items() if k[0] == "step_clock_mixed"]
    assert clock and all(v["spill_st"] == 0 for v in clock)
