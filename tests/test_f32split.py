"""The build's integer FP64 -> FP32 rounding (nemo_gb300/csrc/hc_f32split.h),
compiled as plain C on the host and checked against the host's IEEE
conversions (round to nearest, ties to even) on about ten million doubles."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def test_split_matches_ieee_conversions(tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no C compiler")
    exe = tmp_path / "f32split_check"
    subprocess.run([cc, "-O2", "-std=c11", "-o", str(exe), os.path.join(HERE, "native", "f32split_check.c"), "-lm"],
                   check=True)
    r = subprocess.run([str(exe), "1000000"], capture_output=True, text=True)
    print(r.stdout)
    assert r.returncode == 0, r.stdout
    assert "mismatches 0" in r.stdout
