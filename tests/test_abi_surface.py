"""CPU checks of the drop-in boundary: libvship.so loads, exports every entry point that
include/VshipAPI.h declares (and the reference's 21 C functions), and its host-only behaviour
matches src/VshipLib.cpp without touching a GPU."""
import ctypes
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "VshipAPI.h")

# the reference's exported C functions (src/VshipAPI.h:32-148)
REFERENCE_FUNCTIONS = [
    "Vship_GetVersion", "Vship_GetDeviceCount", "Vship_SetDevice", "Vship_GetDeviceInfo", "Vship_GPUFullCheck",
    "Vship_GetErrorMessage", "Vship_PinnedMalloc", "Vship_PinnedFree", "Vship_SSIMU2Init", "Vship_SSIMU2Free",
    "Vship_ComputeSSIMU2Float", "Vship_ComputeSSIMU2Floatv2", "Vship_ComputeSSIMU2Uint16",
    "Vship_ComputeSSIMU2Uint16v2", "Vship_ButteraugliInit", "Vship_ButteraugliInitv2", "Vship_ButteraugliFree",
    "Vship_ComputeButteraugliFloat", "Vship_ComputeButteraugliFloatv2", "Vship_ComputeButteraugliUint16",
    "Vship_ComputeButteraugliUint16v2",
]


def declared_functions():
    with open(HEADER) as f:
        src = f.read()
    return sorted(set(re.findall(r"EXPORTPREPROCESS\s+[\w ]+?\s\**(Vship_\w+)\s*\(", src)))


def exported_symbols(lib):
    out = subprocess.run(["nm", "-D", "--defined-only", lib], capture_output=True, text=True, check=True).stdout
    return {ln.split()[-1] for ln in out.splitlines() if " T " in ln}


def test_header_declares_reference_surface():
    decl = declared_functions()
    for f in REFERENCE_FUNCTIONS:
        assert f in decl


def test_library_exports_every_declared_function(vlib):
    syms = exported_symbols(vlib.LIB_PATH)
    missing = [f for f in declared_functions() if f not in syms]
    assert not missing, missing
    # and nothing but the C ABI leaks out of the shared object
    assert all(s.startswith("Vship_") or s.startswith("VapourSynth") for s in syms), sorted(syms)


def test_python_signatures_cover_header(vlib):
    assert sorted(vlib.SIGNATURES) == declared_functions()


def test_version(vlib):
    assert vlib.version() == (3, 1, 0, "Cuda")


def test_error_message_contract(vlib):
    L = vlib.lib()
    for code in range(12):
        n = L.Vship_GetErrorMessage(code, None, 0)
        buf = ctypes.create_string_buffer(n)
        assert L.Vship_GetErrorMessage(code, buf, n) == n
        msg = buf.value.decode()
        assert len(msg) == n - 1
        assert msg.startswith(vlib.EXCEPTION_NAMES[code] + ":")
    # truncation: copies len-1 characters and NUL-terminates (src/VshipLib.cpp:122-128)
    buf = ctypes.create_string_buffer(b"\x01" * 16)
    need = L.Vship_GetErrorMessage(9, buf, 8)
    assert need > 8 and buf.raw[7] == 0 and len(buf.value) == 7


def test_bad_handler_without_gpu(vlib):
    L = vlib.lib()
    h = vlib.Handler(12345)
    assert L.Vship_SSIMU2Free(h) == vlib.BadHandler
    assert L.Vship_ButteraugliFree(h) == vlib.BadHandler
    score = ctypes.c_double()
    arr = (ctypes.c_void_p * 3)()
    assert L.Vship_ComputeSSIMU2Float(h, ctypes.byref(score), ctypes.cast(arr, vlib._PP),
                                      ctypes.cast(arr, vlib._PP), 16) == vlib.BadHandler


@pytest.mark.skipif(os.environ.get("CUDA_VISIBLE_DEVICES") is None and os.path.exists("/dev/nvidia0"),
                    reason="a GPU is visible")
def test_device_queries_report_errors_without_gpu(vlib):
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("GPU present")
    except Exception:
        pass
    L = vlib.lib()
    n = ctypes.c_int(-1)
    rc = L.Vship_GetDeviceCount(ctypes.byref(n))
    assert rc in (vlib.DeviceCountError, vlib.NoDeviceDetected)
    assert L.Vship_GPUFullCheck(0) in (vlib.DeviceCountError, vlib.NoDeviceDetected)
    h = vlib.Handler()
    assert L.Vship_SSIMU2Init(ctypes.byref(h), 64, 64) in (vlib.DeviceCountError, vlib.NoDeviceDetected)
