"""The FFVship-compatible command-line tool (vship_gb300/ffvship): argument handling, YUV4MPEG2
input (4:2:0 / 4:2:2 / 4:4:4, 8-16 bit, sitings), frame selection, JSON output (doc/FFVship.md
format) and agreement with the library's Y'CbCr entry points in the file's format (matrix by
height, as the reference guesses for files without one)."""
import json
import os
import subprocess

import numpy as np
import pytest

from vship_gb300 import synth

HERE = os.path.dirname(os.path.abspath(__file__))
CLI = os.path.join(os.path.dirname(HERE), "vship_gb300", "ffvship")


@pytest.fixture(scope="module")
def cli(vlib):
    assert os.path.exists(CLI)
    return CLI


def run(*args):
    return subprocess.run([CLI, *map(str, args)], capture_output=True, text=True, timeout=600)


def test_version(cli):
    r = run("--version")
    assert r.returncode == 0 and "ffvship" in r.stdout


def test_unknown_argument_fails(cli):
    r = run("--not-a-flag")
    assert r.returncode == 1 and "Unknown argument" in r.stderr


def test_missing_files_fail(cli):
    assert run("-s", "x.y4m").returncode == 1
    r = run("-s", "/nonexistent.y4m", "-e", "/nonexistent.y4m")
    assert r.returncode == 1 and "cannot open" in r.stderr


def test_rejects_unsupported_colorspace(cli, tmp_path):
    p = tmp_path / "a.y4m"
    p.write_bytes(b"YUV4MPEG2 W8 H8 F24:1 Cmono\nFRAME\n" + bytes(8 * 8))
    r = run("-s", p, "-e", p)
    assert r.returncode == 1 and "unsupported" in r.stderr


def test_rejects_differing_formats(cli, tmp_path):
    a, b = tmp_path / "a.y4m", tmp_path / "b.y4m"
    synth.write_y4m(str(a), [synth.yuv420p10_source(8, 8, 0, 1)], 8, 8)
    f = synth.yuv_frames(8, 8, 0, 10, 0, 0)[0]
    synth.write_y4m(str(b), [f], 8, 8, 10, chroma="444")
    r = run("-s", a, "-e", b)
    assert r.returncode == 1 and "differ" in r.stderr


def test_unknown_metric(cli, tmp_path):
    p = tmp_path / "a.y4m"
    synth.write_y4m(str(p), [synth.yuv420p10_source(8, 8, 0, 1)], 8, 8)
    r = run("-s", p, "-e", p, "-m", "PSNR")
    assert r.returncode == 1 and "Unknown metric" in r.stderr


def _clip(tmp_path, h, w, n, bits=10, chroma="420", siting=""):
    """n frame pairs written as .y4m, and the same planes as arrays of the file's sample type."""
    ssw, ssh = {"420": (1, 1), "422": (1, 0), "444": (0, 0)}[chroma]
    src, enc = [], []
    for t in range(n):
        r, d = synth.yuv_frames(h, w, t, bits, ssw, ssh, False, seed=13, distortion="dct")
        src.append(r)
        enc.append(d)
    ps, pe = tmp_path / f"src{bits}{chroma}.y4m", tmp_path / f"enc{bits}{chroma}.y4m"
    synth.write_y4m(str(ps), src, w, h, bits, chroma=chroma, siting=siting)
    synth.write_y4m(str(pe), enc, w, h, bits, chroma=chroma, siting=siting)
    dt = np.uint8 if bits == 8 else np.uint16
    arr = lambda f: [np.ascontiguousarray(np.asarray(p).astype(dt)) for p in f]
    return ps, pe, [arr(f) for f in src], [arr(f) for f in enc]


def _fmt(vlib, bits, chroma="420", loc=0):
    ss = {"420": (1, 1), "422": (1, 0), "444": (0, 0)}[chroma]
    return vlib.yuv_format(bits, ss, 2, False, loc)


@pytest.mark.gpu
@pytest.mark.parametrize("bits,chroma,siting,loc", [(10, "420", "", 0), (8, "420", "", 1), (8, "420", "mpeg2", 0),
                                                    (12, "422", "", 0), (16, "444", "", 0), (8, "420", "paldv", 2)])
def test_ssimu2_json_matches_library(cli, vlib, tmp_path, bits, chroma, siting, loc):
    h, w, n = 72, 96, 5
    ps, pe, src, enc = _clip(tmp_path, h, w, n, bits, chroma, siting)
    out = tmp_path / "s.json"
    r = run("-s", ps, "-e", pe, "-m", "SSIMULACRA2", "--json", out, "-g", 2, "-t", 2)
    assert r.returncode == 0, r.stderr
    got = json.loads(out.read_text())
    with vlib.SSIMU2Handler(w, h) as hd:
        hd.set_yuv_format(_fmt(vlib, bits, chroma, loc))
        want = [hd.compute_yuv(a, b) for a, b in zip(src, enc)]
    assert [len(x) for x in got] == [1] * n
    assert np.allclose([x[0] for x in got], want, atol=1e-5)
    assert "SSIMULACRA2" in r.stdout and "Average" in r.stdout


@pytest.mark.gpu
def test_butteraugli_selection_and_offset(cli, vlib, tmp_path):
    h, w, n = 64, 80, 6
    ps, pe, src, enc = _clip(tmp_path, h, w, n)
    out = tmp_path / "b.json"
    r = run("-s", ps, "-e", pe, "-m", "Butteraugli", "--qnorm", 3, "--intensity-target", 120, "--start", 1, "--end", 6,
            "--every", 2, "--encoded-offset", -1, "--json", out)
    assert r.returncode == 0, r.stderr
    got = json.loads(out.read_text())
    with vlib.ButteraugliHandler(w, h, 3, 120.0) as hd:
        hd.set_yuv_format(_fmt(vlib, 10))
        want = [hd.compute_yuv(src[s], enc[s - 1]) for s in (1, 3, 5)]
    assert len(got) == 3
    for g, wv in zip(got, want):
        assert np.allclose(g, wv, rtol=1e-5)
    assert "3-Norm" in r.stdout and "INF-Norm" in r.stdout


@pytest.mark.gpu
def test_crop_and_live_output(cli, vlib, tmp_path):
    h, w, n = 64, 80, 3
    ps, pe, src, enc = _clip(tmp_path, h, w, n)
    r = run("-s", ps, "-e", pe, "--cropTopSource", 8, "--cropTopEncoded", 8, "--cropLeftSource", 4,
            "--cropLeftEncoded", 4, "--live-score-output")
    assert r.returncode == 0, r.stderr
    lines = r.stdout.strip().splitlines()
    assert lines[0] == "3"
    got = dict((int(a), float(b)) for a, b in (ln.split() for ln in lines[1:]))
    crop = lambda f: [np.ascontiguousarray(f[0][8:, 4:]), np.ascontiguousarray(f[1][4:, 2:]),
                      np.ascontiguousarray(f[2][4:, 2:])]
    with vlib.SSIMU2Handler(w - 4, h - 8) as hd:
        hd.set_yuv_format(_fmt(vlib, 10))
        for i in range(n):
            assert abs(got[i] - hd.compute_yuv(crop(src[i]), crop(enc[i]))) < 1e-5
