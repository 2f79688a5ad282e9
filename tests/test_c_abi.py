"""include/cpgpu.h is a plain C header: a C99 program compiles against it
with strict warnings, links with the device library, and runs (on a GPU) or
fails loudly with CPGPU_ERR_NO_DEVICE (without one)."""
import os
import platform
import subprocess

import pytest

import constraintphysics_gb300 as cg

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
# warnings are errors where the CPU suite runs (x86-64); elsewhere (the Arm GPU
# hosts, whose compiler adds target-specific notes) they are only reported
STRICT = ["-Wall", "-Wextra", "-pedantic"] + (["-Werror"] if platform.machine() in ("x86_64", "AMD64") else [])


def _build(tmp_path):
    exe = str(tmp_path / "c_abi_box_drop")
    lib_dir = os.path.dirname(cg.LIB_PATH)
    cmd = ["gcc", "-std=c99", *STRICT, "-I" + os.path.join(REPO, "include"),
           os.path.join(HERE, "c", "c_abi_box_drop.c"), "-L" + lib_dir, "-lcpgpu", "-Wl,-rpath," + lib_dir, "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_c_program_compiles_and_fails_loudly_without_gpu(tmp_path):
    exe = _build(tmp_path)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode in (0, 2), r.stdout + r.stderr
    if r.returncode == 2:
        assert "no CUDA device" in r.stdout


@pytest.mark.gpu
def test_c_program_drops_a_box_on_device(tmp_path):
    exe = _build(tmp_path)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
