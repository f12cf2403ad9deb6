"""The C++ host binding (pfem_gb300/host/pfem_host.hpp): the demo driver compiles against
include/pfem_gpu.h and links libpfemgpu.so (CPU), and runs PSPG and WC steps (GPU)."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _compile(tmp_path):
    from pfem_gb300 import build

    build.build()
    build.build_remesh()
    exe = str(tmp_path / "host_demo")
    lib_dir = os.path.join(ROOT, "pfem_gb300")
    cmd = ["g++", "-std=c++17", "-O2", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"),
           "-I", os.path.join(ROOT, "pfem_gb300", "host"), os.path.join(ROOT, "pfem_gb300", "host", "host_demo.cpp"),
           "-L", lib_dir, "-lpfemgpu", "-lpfemremesh", f"-Wl,-rpath,{lib_dir}", "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    return exe


def test_cpp_host_binding_compiles_and_links(tmp_path):
    assert os.path.exists(_compile(tmp_path))


def test_cpp_host_remesh_runs_on_cpu(tmp_path):
    """The C++ Remesher alone: alpha shape of a dam-break cloud, one remesh of the moved mesh."""
    exe = _compile(tmp_path)
    out = subprocess.run([exe, "remesh"], capture_output=True, text=True, timeout=300)
    print(out.stdout)
    assert out.returncode == 0, out.stdout + out.stderr
    assert "FAIL" not in out.stdout and out.stdout.count("ok ") == 5


@pytest.mark.gpu
def test_cpp_host_demo_runs(tmp_path, gpu_lib):
    exe = _compile(tmp_path)
    out = subprocess.run([exe], capture_output=True, text=True, timeout=600)
    print(out.stdout)
    assert out.returncode == 0, out.stdout + out.stderr
    assert "FAIL" not in out.stdout and out.stdout.count("ok ") == 15
