"""The division-free tsdf unpacking used by the kernels equals the
reference's IEEE division (float)t / 32766 for every int16 input."""
import os
import subprocess

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_unpack_matches_ieee_division_exhaustively(tmp_path):
    exe = str(tmp_path / "unpack_check")
    src = os.path.join(REPO, "tests", "unpack_check.cpp")
    inc = os.path.join(REPO, "marching_cube_gb300", "csrc")
    subprocess.run(["g++", "-O2", "-ffp-contract=off", "-I", inc, src, "-o", exe, "-lm"], check=True)
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout
    assert "0 mismatches" in r.stdout
