"""The reference's C++ call sequence compiled against include/ahx_ahmed.hpp."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "dropin_sphere.cpp")
LIBDIR = os.path.join(ROOT, "ahmed_gb300")


def _build(tmp_path):
    exe = str(tmp_path / "dropin_sphere")
    subprocess.check_call(["g++", "-O2", "-std=c++14", "-I", os.path.join(ROOT, "include"), SRC,
                           "-L", LIBDIR, "-lahx", "-Wl,-rpath," + LIBDIR, "-o", exe])
    return exe


def test_dropin_compiles_and_builds_trees_on_host(tmp_path):
    exe = _build(tmp_path)
    out = subprocess.run([exe, "2048", "tree-only"], capture_output=True, text=True, check=True)
    assert out.stdout.startswith("leaves ")


@pytest.mark.gpu
def test_dropin_runs_on_gpu(tmp_path):
    exe = _build(tmp_path)
    out = subprocess.run([exe, "2048"], capture_output=True, text=True, timeout=300, cwd=str(tmp_path))
    assert out.returncode == 0, out.stdout + out.stderr
    assert "GMRes ret 0" in out.stdout
    assert "savembls/loadmbls round trip ok" in out.stdout
    assert "symmetric:" in out.stdout
    assert "helmholtz:" in out.stdout
    assert "helmholtz symmetric:" in out.stdout
    assert "helmholtz savembls/loadmbls round trip ok" in out.stdout
    assert "helmholtz agglH:" in out.stdout
    assert "single precision:" in out.stdout
