"""Build recipe for the craw-gb300 shared libraries (no cmake, no setup.py).

Compiles, in parallel and in tree:

* ``libcraw_gb300/_lib/libcraw.so`` -- the product: the C23 host library
  (``csrc/host/*.c``, gcc ``-std=c2x``) and the sm_103a kernels
  (``csrc/kernels/*.cu``, nvcc ``-gencode arch=compute_103a,code=sm_103a``),
  linked with the static CUDA runtime. Its exported symbols are the
  ``craw_*`` C ABI declared in ``include/craw/*.h``.
* ``libcraw_gb300/_lib/libcraw_bounds.so`` -- the same library built with
  ``-DCRAW_DEBUG_BOUNDS=1``: its kernels check their indices against their
  buffers and report a bad one (CRAW_K_ERR_BOUNDS) instead of making the
  access (a stand-in for a memory checker; tests load it in a process of
  their own through ``CRAW_LIBRARY``).
* ``libcraw_gb300/_lib/libcraw_synth.so`` -- the seeded synthetic-frame
  generator used by the benchmark and the tests (OpenMP).
* ``oracle/_build/liboracle.so`` -- the CPU oracle (test infrastructure).
* ``oracle/_ref/`` -- the reference's own CPU code, only where the
  reference tree is present (``oracle/build_ref.sh``).

An object is rebuilt when its source or any header it may include is newer.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent
PKG = ROOT / "libcraw_gb300"
CSRC = PKG / "csrc"
LIB = PKG / "_lib"
OBJ = PKG / "_lib" / "obj"
ORACLE = ROOT / "oracle"
CUDA_HOME = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda"))
NVCC = str(CUDA_HOME / "bin" / "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
#: The reference's source tree, where present (it is not on every machine
#: that builds this project): CRAW_REFERENCE_DIR, else its usual checkout.
REFERENCE = Path(os.environ.get("CRAW_REFERENCE_DIR", "/root/reference"))

HOST_CFLAGS = ["-std=c2x", "-O2", "-fPIC", "-fvisibility=hidden", "-Wall", "-Wextra",
               "-Wno-unused-parameter", "-Wno-missing-field-initializers",
               f"-I{ROOT / 'include'}", f"-I{CUDA_HOME / 'include'}"]
NVCC_FLAGS = ["-std=c++17", "-O3", "-lineinfo", *ARCH, "-Xcompiler", "-fPIC",
              "-Xcompiler", "-fvisibility=hidden", f"-I{ROOT / 'include'}",
              "-diag-suppress", "177"]
# The highlight pass and the noise estimator restate host code whose
# float results they must reproduce: built like the reference's host code
# and the oracle, without multiply-add contraction.
NVCC_FILE_FLAGS = {"highlight": ["-fmad=false"], "noise": ["-fmad=false"]}


def _headers(*dirs: Path) -> float:
    t = 0.0
    for d in dirs:
        for p in d.rglob("*"):
            if p.suffix in (".h", ".cuh"):
                t = max(t, p.stat().st_mtime)
    return t


def _stale(out: Path, srcs: list[Path], hdr_time: float) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(s.stat().st_mtime > t for s in srcs) or hdr_time > t


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"command failed ({r.returncode}): {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")


def build(verbose: bool = False, with_reference: bool | None = None) -> dict[str, Path]:
    """Builds every library; returns their paths. Raises on a failed step."""
    LIB.mkdir(parents=True, exist_ok=True)
    (ORACLE / "_build").mkdir(parents=True, exist_ok=True)
    hdr = _headers(ROOT / "include", CSRC)

    # The product, and the bounds-checked variant (the host objects are the
    # same; the kernels are compiled again with the checks), in one pool.
    variants = {"libcraw.so": (OBJ, []), "libcraw_bounds.so": (LIB / "obj_bounds", ["-DCRAW_DEBUG_BOUNDS=1"])}
    jobs: list[tuple[Path, list[str], list[Path]]] = []
    objs: dict[str, list[Path]] = {}
    host: list[Path] = []
    for c in sorted((CSRC / "host").glob("*.c")):
        o = OBJ / (c.stem + ".o")
        host.append(o)
        jobs.append((o, ["gcc", *HOST_CFLAGS, "-c", str(c), "-o", str(o)], [c]))
    for name, (odir, extra) in variants.items():
        odir.mkdir(parents=True, exist_ok=True)
        objs[name] = list(host)
        for cu in sorted((CSRC / "kernels").glob("*.cu")):
            o = odir / (cu.stem + ".cu.o")
            objs[name].append(o)
            jobs.append((o, [NVCC, *NVCC_FLAGS, *extra, *NVCC_FILE_FLAGS.get(cu.stem, []), "-c", str(cu),
                             "-o", str(o)], [cu]))

    todo = [j for j in jobs if _stale(j[0], j[2], hdr)]
    workers = max(1, min(len(todo), os.cpu_count() or 4))
    if todo:
        with cf.ThreadPoolExecutor(workers) as ex:
            for f in cf.as_completed([ex.submit(_run, cmd) for _, cmd, _ in todo]):
                f.result()
        if verbose:
            print(f"compiled {len(todo)} objects", file=sys.stderr)

    for name in variants:
        so = LIB / name
        if _stale(so, objs[name], 0.0):
            _run([NVCC, "-shared", *ARCH, "-cudart", "static", "-o", str(so), *map(str, objs[name]),
                  "-Xlinker", "--exclude-libs,ALL", "-lm"])
    so = LIB / "libcraw.so"

    synth_src = CSRC / "synth" / "synth.c"
    synth = LIB / "libcraw_synth.so"
    if _stale(synth, [synth_src], _headers(CSRC / "synth")):
        _run(["gcc", "-std=c2x", "-O2", "-fPIC", "-fopenmp", "-shared", "-fvisibility=hidden",
              str(synth_src), "-o", str(synth), "-lm"])

    orc_src = ORACLE / "craw_oracle.c"
    orc = ORACLE / "_build" / "liboracle.so"
    if _stale(orc, [orc_src, ORACLE / "oracle_impl.h", ORACLE / "craw_oracle.h"], hdr):
        # -O3: the CPU baseline (bench.py) times this build; -ffp-contract=off
        # keeps its float results those of the reference's build on every host
        # (no -march=native: the same results on the x86 and Arm machines).
        _run(["gcc", "-std=c2x", "-O3", "-fPIC", "-ffp-contract=off", "-shared",
              "-fvisibility=hidden", f"-I{ROOT / 'include'}", f"-I{CUDA_HOME / 'include'}",
              str(orc_src), "-o", str(orc), "-lm"])

    out = {"craw": so, "craw_bounds": LIB / "libcraw_bounds.so", "synth": synth, "oracle": orc}
    if with_reference is None:
        with_reference = (REFERENCE / "lib" / "ref").is_dir()
    if with_reference and shutil.which("gcc"):
        ref_so = ORACLE / "_ref" / "libcraw_ref.so"
        if not ref_so.exists():
            _run(["sh", str(ORACLE / "build_ref.sh"), str(REFERENCE)])
        out["reference"] = ref_so
    return out


if __name__ == "__main__":
    for k, v in build(verbose=True).items():
        print(k, v)
