"""The tensor-core pass rounds its A operand to TF32 with an integer form of round-to-nearest,
ties-away (qcs::tc::tf32_rna); this checks it against the hardware conversion cvt.rna.tf32.f32 on
every finite 32-bit pattern (tests/tf32_rounding_check.cu)."""
from __future__ import annotations

import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


@pytest.mark.gpu
def test_integer_rounding_matches_cvt_rna(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(nvcc).exists():
        pytest.skip("nvcc not found")
    exe = tmp_path / "tf32_rounding_check"
    subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17",
                    f"-I{ROOT / 'qcsim_gb300' / 'csrc'}", str(ROOT / "tests" / "tf32_rounding_check.cu"), "-o", str(exe)],
                   check=True, capture_output=True, text=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True, timeout=120).stdout.split()
    counts = dict(zip(out[0::2], map(int, out[1::2])))
    # every finite input below the overflow threshold (all amplitudes and their splits) rounds identically
    assert counts["differ_below_overflow"] == 0, counts
