"""The double-float arithmetic of the exact denoise rounding, compiled for
the host from the kernel's own header and checked against long double:
each operation within a few units of 2^-48 relative, the rounding of
values next to a half-integer exact."""
import shutil
import subprocess
from pathlib import Path

import pytest

HERE = Path(__file__).resolve().parent


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")
def test_dfloat_against_long_double(tmp_path):
    exe = tmp_path / "dfloat_check"
    subprocess.run(["g++", "-O2", "-ffp-contract=off", "-o", str(exe), str(HERE / "native" / "dfloat_check.cpp"),
                    "-lm"], check=True)
    out = subprocess.run([str(exe), "100000"], check=True, capture_output=True, text=True).stdout
    res = {k: float(v) for k, v in (line.split() for line in out.strip().splitlines())}
    # 2^-48 = 3.6e-15: one representation rounding of the result, a few at most.
    for op in ("exp", "sqrt", "div", "mul", "add", "sub"):
        assert res[op] < 2e-14, (op, res[op])
    assert res["rint_bad"] == 0
