"""The C ABI boundary: every entry point declared in include/cpgpu.h is
exported by the device library (and, with its own prefix, by both oracle
libraries); without a GPU the device library fails loudly instead of falling
back to a CPU path.  CPU only."""
import ctypes
import os
import re

import pytest

import constraintphysics_gb300 as cg

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "cpgpu.h")


def declared():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(cpgpu_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_the_api():
    names = declared()
    for n in ("cpgpu_world_create", "cpgpu_step", "cpgpu_body_hull", "cpgpu_get_contacts", "cpgpu_batch_step"):
        assert n in names


def test_device_library_exports_every_declared_symbol():
    lib = ctypes.CDLL(cg.LIB_PATH)
    missing = [n for n in declared() if not hasattr(lib, n)]
    assert not missing, missing


@pytest.mark.parametrize("which", ["ref", "port"])
def test_oracle_libraries_export_the_world_api(oracle_mod, which):
    abi = oracle_mod.ref_abi() if which == "ref" else oracle_mod.port_abi()
    prefix = "cpref_" if which == "ref" else "cport_"
    # batches, the allocation-free pair entry point and the FP64 audit exist
    # on the device path only
    batch_only = {n[len("cpgpu_"):] for n in declared()
                  if n.startswith(("cpgpu_batch_", "cpgpu_server_"))} | {"pairs_noalloc", "world_clone",
                                                                            "world_set_audit", "world_read_audit"}
    state_import = {"set_body_state", "set_contacts", "get_joint_state", "set_joint_state"}
    for n in declared():
        short = n[len("cpgpu_"):]
        if short in batch_only or (which == "ref" and short in state_import):
            continue
        assert hasattr(abi._lib, prefix + short), prefix + short


def _device_present():
    try:
        cuda = ctypes.CDLL("libcuda.so.1")
    except OSError:
        return False
    if cuda.cuInit(0) != 0:
        return False
    n = ctypes.c_int()
    return cuda.cuDeviceGetCount(ctypes.byref(n)) == 0 and n.value > 0


@pytest.mark.skipif(_device_present(), reason="a CUDA device is present")
def test_no_device_fails_loudly():
    with pytest.raises(cg.CPGPUError, match="status -8"):
        cg.world()


def test_invalid_arguments_are_rejected_without_a_device():
    abi = cg.lib()
    assert abi.world_destroy(None) == 0
    assert abi.step(None, 1) == -1
    assert b"null world" in abi.last_error()
