"""GPU: the bounds-checked build (libcraw_bounds.so, every global index of
the develop, denoise, chroma and highlight kernels checked against its
buffer, a bad one recorded as CRAW_K_ERR_BOUNDS and skipped) develops the cases of
bounds_cases.py in a process of its own with no error bit set, and
gives the product build's outputs bit for bit."""
import os
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

import libcraw_gb300 as L

pytestmark = pytest.mark.gpu

HERE = Path(__file__).resolve().parent
BOUNDS = Path(L.__file__).resolve().parent / "_lib" / "libcraw_bounds.so"


def test_bounds_build_is_clean_and_equal(tmp_path):
    assert BOUNDS.exists(), "libcraw_bounds.so is built by libcraw_gb300.build.build()"
    sys.path.insert(0, str(HERE))
    import bounds_cases
    mine = bounds_cases.run_cases()
    out = tmp_path / "bounds.npz"
    env = dict(os.environ, CRAW_LIBRARY=str(BOUNDS))
    r = subprocess.run([sys.executable, str(HERE / "bounds_cases.py"), str(out)], env=env,
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-3000:]
    theirs = dict(np.load(out))
    assert set(theirs) == set(mine)
    for key in sorted(mine):
        if key.endswith("/errors"):
            assert int(theirs[key][0]) == 0, (key, int(theirs[key][0]))
            assert int(mine[key][0]) == 0, key
        else:
            assert np.array_equal(mine[key].view(np.uint8), theirs[key].view(np.uint8)), key
