"""The fz-gpu CLI: the reference's three output lines (fz.cu:207-209) and a file round
trip through -o / --decompress."""
import os
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_cli_prints_reference_lines_and_round_trips(fz, oracle, synth, tmp_path):
    data = synth.smooth2d(3600, 1800, seed=0)
    raw = tmp_path / "cesm-like-3600x1800.f32"
    data.tofile(raw)
    out = tmp_path / "s.fz"
    r = subprocess.run([fz.CLI_PATH, str(raw), "3600", "1800", "1", "1e-3", "-o", str(out)],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    want = oracle.compress(data, (3600, 1800, 1), 1e-3)
    nnz = oracle.parse_header(want)["nnz"]
    comp = 4 * ((2 * data.size + 511) // 512) + 16 * nnz
    lines = r.stdout.strip().splitlines()
    assert lines[0] == f"original size: {4 * data.size}"
    assert lines[1] == f"compressed size: {comp}"
    assert lines[2] == "compression ratio: %f" % np.float32(np.float32(4 * data.size) / np.float32(comp))
    st = np.fromfile(out, np.uint8)
    assert np.array_equal(st, want)
    rec = tmp_path / "r.f32"
    r = subprocess.run([fz.CLI_PATH, "--decompress", str(out), "-o", str(rec), "--verify", str(raw)],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    assert np.array_equal(np.fromfile(rec, np.float32).view(np.uint32), oracle.decompress(want).view(np.uint32))
    assert "PSNR" in r.stdout


def test_cli_missing_file_exits_nonzero(fz, tmp_path):
    r = subprocess.run([fz.CLI_PATH, str(tmp_path / "nope"), "10", "1", "1", "1e-3"],
                       capture_output=True, text=True, timeout=60)
    assert r.returncode == 1 and "fail to open" in r.stderr


def test_cli_reports_code_overflow(fz, tmp_path):
    """A delta beyond the 16-bit codes (the reference has no outlier channel, Q6) sets
    FZ_FLAG_CODE_OVERFLOW; both CLI directions warn on stderr, stdout keeps three lines."""
    data = np.zeros((64, 64), np.float32)
    data[10, 20] = 1.0e6  # relative eb 1e-6: |delta| ~ 5e5 codes
    raw = tmp_path / "spike.f32"
    data.tofile(raw)
    out = tmp_path / "spike.fz"
    r = subprocess.run([fz.CLI_PATH, str(raw), "64", "64", "1", "1e-6", "-o", str(out)],
                       capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    assert len(r.stdout.strip().splitlines()) == 3
    assert "FZ_FLAG_CODE_OVERFLOW" in r.stderr
    assert fz.parse_header(np.fromfile(out, np.uint8)[:64]).flags & 1
    r = subprocess.run([fz.CLI_PATH, "--decompress", str(out), "-o", str(tmp_path / "r.f32")],
                       capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and "FZ_FLAG_CODE_OVERFLOW" in r.stderr
    # a field that fits prints no warning
    ok = tmp_path / "ok.f32"
    np.linspace(0, 1, 4096, dtype=np.float32).tofile(ok)
    r = subprocess.run([fz.CLI_PATH, str(ok), "4096", "1", "1", "1e-3"], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and "FZ_FLAG_CODE_OVERFLOW" not in r.stderr
