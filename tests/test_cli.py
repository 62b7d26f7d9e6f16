"""The command-line front end (libcraw_gb300.cli): file formats on the CPU,
and on the GPU a dump developed through the CLI against the same frame
through craw_pipeline_record() directly."""
import numpy as np
import pytest

import libcraw_gb300 as L
from libcraw_gb300 import cli
from libcraw_gb300 import workloads as W


def test_pfm_round_trip(tmp_path):
    rng = np.random.default_rng(3)
    img = rng.standard_normal((7, 11, 4)).astype(np.float32)
    cli.write_pfm(tmp_path / "a.pfm", img)
    raw = (tmp_path / "a.pfm").read_bytes()
    assert raw.startswith(b"PF\n11 7\n-1.0\n")
    # Rows bottom to top: the first row in the file is the image's last.
    first = np.frombuffer(raw[len(b"PF\n11 7\n-1.0\n"):][:11 * 12], dtype="<f4").reshape(11, 3)
    assert np.array_equal(first, img[-1, :, :3])
    assert np.array_equal(cli.read_pfm(tmp_path / "a.pfm"), img[..., :3])


def test_raw_dump_and_synth(tmp_path):
    assert cli.main(["synth", str(tmp_path / "f.raw"), "--width", "64", "--height", "48", "--seed", "5"]) == 0
    m = cli.read_raw(tmp_path / "f.raw", 64, 48)
    assert m.dtype == np.uint16 and m.shape == (48, 64)
    assert np.array_equal(m, W.synth_frame(64, 48, 5, noise_a_dn=4.0, noise_b_dn=40.0))
    with pytest.raises(ValueError):
        cli.read_raw(tmp_path / "f.raw", 64, 50)


def test_help_lists_commands(capsys):
    with pytest.raises(SystemExit):
        cli.main(["--help"])
    out = capsys.readouterr().out
    for c in ("develop", "bench", "synth", "noise"):
        assert c in out


@pytest.mark.gpu
def test_cli_develop_matches_the_pipeline(tmp_path):
    import torch
    from gpu_util import develop

    w, h = 160, 96
    assert cli.main(["synth", str(tmp_path / "f.raw"), "--width", str(w), "--height", str(h)]) == 0
    assert cli.main(["develop", str(tmp_path / "f.raw"), str(tmp_path / "f.pfm"), "--width", str(w),
                     "--height", str(h), "--debayer", "rcd", "--space", "bt709", "--denoise", "1.0"]) == 0
    got = cli.read_pfm(tmp_path / "f.pfm")
    m = cli.read_raw(tmp_path / "f.raw", w, h)
    prof = W.make_profile()
    pp = L.pipeline_params(w, h, debayer=L.DEBAYER_RCD, out_space=L.CS_BT709, flags=L.FLAG_DENOISE,
                           out_format=L.FORMAT_RGBA32F)
    fp = L.frame_params(prof, denoise_strength=1.0, noise_override=W.noise_model(4.0, 40.0))
    with L.Context(0) as ctx, L.Pipeline(ctx, pp) as pipe:
        ref = develop(pipe, m, fp)
    assert np.array_equal(got, ref[..., :3])
    assert cli.main(["bench", "--width", str(w), "--height", str(h), "--frames", "3",
                     "--denoise", "1.0"]) == 0


@pytest.mark.gpu
def test_cli_highlights(tmp_path):
    from gpu_util import develop

    w, h = 128, 96
    m = W.highlight_frame(w, h, 77)
    m.tofile(tmp_path / "hl.raw")
    assert cli.main(["develop", str(tmp_path / "hl.raw"), str(tmp_path / "hl.pfm"), "--width", str(w),
                     "--height", str(h), "--space", "bt709", "--highlights"]) == 0
    got = cli.read_pfm(tmp_path / "hl.pfm")
    prof = W.make_profile()
    pp = L.pipeline_params(w, h, debayer=L.DEBAYER_RCD, out_space=L.CS_BT709,
                           flags=L.FLAG_HIGHLIGHT_RECONSTRUCTION, out_format=L.FORMAT_RGBA32F)
    fp = L.frame_params(prof, flags=L.FRAME_HIGHLIGHT_RECONSTRUCTION)
    with L.Context(0) as ctx, L.Pipeline(ctx, pp) as pipe:
        ref = develop(pipe, m, fp)
    assert np.array_equal(got, ref[..., :3])


@pytest.mark.gpu
def test_cli_noise(tmp_path, capsys):
    w, h = 1024, 768
    m = W.noise_ramp(w, h, 88, lo=0.0)
    m.tofile(tmp_path / "n.raw")
    assert cli.main(["noise", "--input", str(tmp_path / "n.raw"), "--width", str(w), "--height", str(h),
                     "--bins", "64", "--min-samples", "1000"]) == 0
    line = capsys.readouterr().out.strip().splitlines()[-1]
    est = L.noise_estimate(m, W.make_profile(), L.noise_estimate_params(nb_bins=64, min_bin_samples=1000))
    assert f"a {est.model.a:.4e} b {est.model.b:.4e}" in line and f"{est.nb_bins} bins" in line
