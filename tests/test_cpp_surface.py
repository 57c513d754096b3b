"""The C++ class surface (include/reconflow_gb300.hpp) compiles against the
C ABI and links with the library; on a GPU it runs the reference demo's call
order end to end."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _build(tmp_path):
    from reconflow_gb300 import _native

    _native.load()
    exe = tmp_path / "reconflow_demo"
    lib_dir = os.path.dirname(_native.LIB_PATH)
    cmd = ["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "cpp", "reconflow_demo.cpp"), "-o", str(exe),
           "-L", lib_dir, "-lrfgb300", f"-Wl,-rpath,{lib_dir}"]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return exe


def test_cpp_surface_compiles_and_links(tmp_path):
    exe = _build(tmp_path)
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    out = r.stdout.strip()
    # without a GPU the constructor path reports RF_ERR_NO_DEVICE cleanly
    assert out.startswith("ok") or out.startswith("error 6"), out


@pytest.mark.gpu
def test_cpp_demo_runs_on_gpu(tmp_path):
    exe = _build(tmp_path)
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    out = r.stdout.strip().split()
    assert r.returncode == 0 and out[0] == "ok", r.stdout + r.stderr
    med_u, med_z = float(out[1]), float(out[2])
    # one-pixel disparity, baseline 0.1, focal 125: depth 12.5
    assert abs(med_u - 1.0) < 0.2 and abs(med_z - 12.5) < 1.5, (med_u, med_z)
