"""The C boundary from a plain C caller: tests/c_abi/check_abi.c is compiled
by gcc against include/wavefd.h and linked to the in-tree libwavefd.so, as a
cgo / JNI / N-API binding of the reference would link it.
  * layout: the C compiler's sizeof and field offsets of wfd_problem and
    wfd_batch_item equal those of the ctypes mirrors the Python side passes;
  * host: version, status texts, workspace sizes and argument checks, with no
    CUDA call (runs here);
  * gpu: the compute entry points on device 0 (the order-2 drop-ins against
    the update evaluated in double, the three forwards against each other,
    the misfit gradient's invariants, a two-item batch plan against the
    single call, a device-side position error).
"""
import ctypes
import glob
import os
import shutil
import subprocess

import pytest

from conftest import ROOT

SRC = os.path.join(ROOT, "tests", "c_abi", "check_abi.c")


def _cuda_home():
    nvcc = os.environ.get("NVCC") or shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))


@pytest.fixture(scope="module")
def check_abi(tmp_path_factory):
    gcc = shutil.which("gcc")
    if gcc is None:
        pytest.skip("gcc not found")
    from neuralmech_gb300 import _lib
    _lib.load()  # builds libwavefd.so in-tree if it is missing
    pkg = os.path.dirname(_lib.LIB_PATH)
    cuda = _cuda_home()
    libdirs = [d for d in [os.path.join(cuda, "lib64")] + glob.glob(os.path.join(cuda, "targets", "*", "lib"))
               if os.path.exists(os.path.join(d, "libcudart.so"))]
    if not libdirs:
        pytest.skip(f"libcudart.so not found under {cuda}")
    exe = str(tmp_path_factory.mktemp("c_abi") / "check_abi")
    cmd = [gcc, "-std=c11", "-O1", "-Wall", "-Wextra", "-Werror",
           "-I", os.path.join(ROOT, "include"), "-I", os.path.join(cuda, "include"), SRC,
           "-L", pkg, "-lwavefd", "-L", libdirs[0], "-lcudart", "-lm",
           f"-Wl,-rpath,{pkg}:{libdirs[0]}", "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def _run(exe, mode, timeout=60):
    return subprocess.run([exe, mode], capture_output=True, text=True, timeout=timeout)


def test_struct_layout_matches_ctypes(check_abi):
    from neuralmech_gb300 import _lib
    r = _run(check_abi, "layout")
    assert r.returncode == 0, r.stderr
    got = dict((k, int(v)) for k, v in (line.split() for line in r.stdout.splitlines()))
    item = {k[5:]: got.pop(k) for k in list(got) if k.startswith("item.")}
    assert got.pop("sizeof") == ctypes.sizeof(_lib.Problem)
    assert got == {name: getattr(_lib.Problem, name).offset for name, _ in _lib.Problem._fields_}
    assert item.pop("sizeof") == ctypes.sizeof(_lib.BatchItem)
    assert item == {name: getattr(_lib.BatchItem, name).offset for name, _ in _lib.BatchItem._fields_}


def test_host_calls_from_c(check_abi):
    r = _run(check_abi, "host")
    assert r.returncode == 0, r.stdout + r.stderr
    assert "ok (host)" in r.stdout


@pytest.mark.gpu
def test_compute_calls_from_c(check_abi):
    r = _run(check_abi, "gpu", timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "ok (gpu)" in r.stdout
