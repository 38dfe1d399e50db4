"""include/sarbp_reference_shim.hpp: the reference's launchGenerateEcho /
launchBackProjection signatures on top of libsarbp.

CPU: the shim compiles into a program written against the reference's
interface and links to libsarbp.so.  GPU: that program runs the reference's
flow (echo generation, then back-projection) and its image focuses the
reference's brightest target (amplitude 1.5 at (Az0, Rg0), BPA_CUDA.cpp:31)
at pixel (Mslow/2, Nfast/2)."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "sar_cambrianaccelerationcard_gb300")


def build_flow(tmpdir):
    from sar_cambrianaccelerationcard_gb300 import build
    build.build()
    cuda_inc = "/usr/local/cuda/include"
    cuda_lib = "/usr/local/cuda/lib64"
    exe = os.path.join(tmpdir, "ref_flow")
    cmd = [shutil.which("g++") or "g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"), "-I", cuda_inc,
           os.path.join(ROOT, "tests", "shim", "ref_flow.cpp"), "-o", exe, "-L", PKG, "-lsarbp",
           f"-Wl,-rpath,{PKG}", "-L", cuda_lib, "-lcudart", f"-Wl,-rpath,{cuda_lib}"]
    subprocess.run(cmd, check=True)
    return exe


def test_shim_compiles_and_links(tmp_path):
    exe = build_flow(str(tmp_path))
    assert os.path.exists(exe)


@pytest.mark.gpu
def test_reference_flow_through_shim_focuses(tmp_path):
    exe = build_flow(str(tmp_path))
    out = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stdout + out.stderr
    _, i, j, v = out.stdout.split()
    assert abs(int(i) - 128) <= 1 and abs(int(j) - 4800) <= 1, out.stdout
    assert float(v) > 0
