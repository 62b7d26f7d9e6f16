"""The C ABI: the library loads without a GPU, exports exactly what
include/craw/*.h declares, and its structs have the reference's layout."""
import ctypes as C
import re
import subprocess
from pathlib import Path

import pytest

import libcraw_gb300 as L
from libcraw_gb300.build import REFERENCE

ROOT = Path(__file__).resolve().parent.parent
REF_INCLUDE = REFERENCE / "include"


def declared_symbols():
    names = set()
    for h in (ROOT / "include" / "craw").glob("*.h"):
        text = h.read_text()
        for m in re.finditer(r"CRAW_API\s+[\w\s\*]+?\b(craw_\w+)\s*\(", text):
            names.add(m.group(1))
    return names


def test_exports_every_declared_symbol():
    lib = L.lib()
    declared = declared_symbols()
    assert len(declared) >= 25
    for name in declared:
        assert hasattr(lib, name), name
    assert declared == set(L.EXPORTS)


def test_exports_nothing_else():
    so = ROOT / "libcraw_gb300" / "_lib" / "libcraw.so"
    out = subprocess.run(["nm", "-D", "--defined-only", str(so)], capture_output=True, text=True).stdout
    syms = {line.split()[-1] for line in out.splitlines() if line.strip()}
    syms = {s for s in syms if not s.startswith("_")}
    assert syms == declared_symbols()


def test_version():
    assert L.version() == (0, 0, 1)


def test_struct_sizes():
    assert C.sizeof(L.PipelineParams) == 256
    assert C.sizeof(L.FrameParams) == 264
    assert C.sizeof(L.Profile) == 1264
    assert C.sizeof(L.ContextOptions) == 1024


def test_defaults():
    p = L.pipeline_params(64, 48)
    assert (p.debayer, p.out_space, p.out_format, p.nb_awb_slots, p.flags) == (
        L.DEBAYER_RCD, L.CS_XYZ_D65, L.FORMAT_RGBA16F, 1, 0)
    prof = L.profile_init()
    fp = L.frame_params(prof)
    assert fp.wb_mode == L.WB_AS_SHOT and fp.denoise_strength == 0 and not fp.out_space_set


def test_context_without_gpu_fails_cleanly():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(L.CrawError) as e:
        L.Context(0)
    assert e.value.code < 0


OFFSETS_C = r"""
#include <stdio.h>
#include <stddef.h>
#include <craw/pipeline.h>
#define F(T, f) printf(#T "." #f " %zu\n", offsetof(T, f));
int main(void) {
  F(CRAWFrameParams, profile) F(CRAWFrameParams, wb_mode) F(CRAWFrameParams, illuminant)
  F(CRAWFrameParams, exposure_stops) F(CRAWFrameParams, flags) F(CRAWFrameParams, out_space)
  F(CRAWFrameParams, out_space_set) F(CRAWFrameParams, denoise_strength)
  F(CRAWFrameParams, noise_override) F(CRAWFrameParams, false_color_passes)
  F(CRAWFrameParams, denoise_chroma_strength) F(CRAWFrameParams, lens)
  F(CRAWFrameParams, defringe_strength) F(CRAWFrameParams, denoise_temporal_strength)
  F(CRAWFrameParams, denoise_temporal_replay) F(CRAWFrameParams, sharpen_radius)
  F(CRAWFrameParams, rotation)
  F(CRAWPipelineParams, width) F(CRAWPipelineParams, debayer) F(CRAWPipelineParams, out_format)
  F(CRAWPipelineParams, flags) F(CRAWPipelineParams, nb_awb_slots)
  F(CRAWProfile, black_level) F(CRAWProfile, as_shot_matrix) F(CRAWProfile, wb_knots)
  F(CRAWProfile, matrix_knots) F(CRAWProfile, name) F(CRAWProfile, noise_knots)
  F(CRAWProfile, nb_noise_knots)
  printf("sizes %zu %zu %zu\n", sizeof(CRAWFrameParams), sizeof(CRAWPipelineParams), sizeof(CRAWProfile));
  return 0;
}
"""


@pytest.mark.skipif(not (REF_INCLUDE / "craw" / "pipeline.h").exists(), reason="reference headers absent")
def test_layout_matches_reference_headers(tmp_path):
    src = tmp_path / "off.c"
    src.write_text(OFFSETS_C)
    outs = []
    for inc in ([f"-I{ROOT / 'include'}", "-I/usr/local/cuda/include"],
                [f"-I{ROOT / 'oracle' / 'shim'}", f"-I{REF_INCLUDE}"]):
        exe = tmp_path / f"off{len(outs)}"
        subprocess.run(["gcc", "-std=c2x", *inc, str(src), "-o", str(exe)], check=True)
        outs.append(subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout)
    assert outs[0] == outs[1]
