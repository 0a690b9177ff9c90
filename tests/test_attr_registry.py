"""Per-device bookkeeping of kernel shared-memory limits (csrc/attr_registry.h),
checked on the CPU with a fake setter: a kernel is configured once per device,
again on another device, again for a larger size, and exactly once under
concurrent callers."""
import shutil
import subprocess
from pathlib import Path

import pytest

HERE = Path(__file__).resolve().parent
CSRC = HERE.parent / "fast_tensor_leverage_gb300" / "csrc"


def test_attr_registry_per_device(tmp_path):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    exe = tmp_path / "attr_registry_check"
    subprocess.run([gxx, "-std=c++17", "-O1", "-pthread", "-I", str(CSRC),
                    str(HERE / "native" / "attr_registry_check.cpp"), "-o", str(exe)], check=True)
    res = subprocess.run([str(exe)], capture_output=True, text=True)
    assert res.returncode == 0, res.stdout + res.stderr
    assert "attr_registry ok" in res.stdout
