"""The C-ABI library loads and exports every entry point include/bcs.h declares
(no device work: these run without a GPU)."""
import ctypes as C
import os
import re
import subprocess

import bcs

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    text = open(os.path.join(REPO, "include", "bcs.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(bcs_[a-z_0-9]+)\s*\(", text)))


def test_header_and_python_agree():
    assert declared_functions() == sorted(bcs.EXPORTED)


def test_library_exports_every_declared_symbol(lib):
    out = subprocess.run(["nm", "-D", "--defined-only", bcs.LIB_PATH], capture_output=True, text=True).stdout
    exported = set(re.findall(r" T (bcs_\w+)", out))
    missing = [f for f in declared_functions() if f not in exported]
    assert not missing, missing
    for f in declared_functions():
        assert getattr(lib, f) is not None


def test_status_strings_and_version(lib):
    assert lib.bcs_abi_version() == 1
    assert lib.bcs_status_string(0) == b"ok"
    assert lib.bcs_status_string(3) == b"out of device memory"


def test_invalid_arguments_rejected_before_device_work(lib):
    h = C.c_void_p()
    assert lib.bcs_create(None, None, C.byref(h)) == 1
    d = bcs.SceneDesc()
    d.type_count = 0
    assert lib.bcs_create(C.byref(d), None, C.byref(h)) == 1
    assert not h.value
    assert lib.bcs_step(None, 1) == 1
