"""The C++ binding of INTEGRATION.md (tests/binding/dg_binding.cpp), written
against the reference's own types (reduced to their interfaces in
tests/binding/reference_stub.h), compiled with g++ against include/mgldg.h
and linked to libmgldg.so.  Without a GPU the program must compile, link and
report that no device exists; on the GPU it solves a small block problem
with the reference's default multigrid parameters and checks the residual.
"""
import os
import shutil
import subprocess

import pytest

import mgldg

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "multigrid-ldg_gb300")


def _build(tmp_path):
    if shutil.which("g++") is None:
        pytest.skip("no g++")
    mgldg.lib()                       # the library exists and loads
    exe = str(tmp_path / "dg_binding")
    cmd = ["g++", "-std=c++17", "-Wall", "-Werror", "-O1", "-I", os.path.join(ROOT, "include"),
           "-I", os.path.join(ROOT, "tests", "binding"), os.path.join(ROOT, "tests", "binding", "dg_binding.cpp"),
           "-L", PKG, "-lmgldg", f"-Wl,-rpath,{PKG}", "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def _has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except ImportError:
        return False


def test_binding_compiles_links_and_reports_no_device(tmp_path):
    exe = _build(tmp_path)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    if _has_gpu():
        assert r.returncode == 0, r.stdout + r.stderr
    else:
        assert r.returncode == 3, r.stdout + r.stderr
        assert "no CUDA device" in r.stdout


@pytest.mark.gpu
def test_binding_solves_on_gpu(tmp_path):
    exe = _build(tmp_path)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "relative residual" in r.stdout
