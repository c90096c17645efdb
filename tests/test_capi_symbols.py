"""The C-ABI library loads and exports every symbol include/paraprobe_gb300.h declares."""
import os
import re
import subprocess

from paraprobe_gb300 import native

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared(header):
    src = open(os.path.join(ROOT, "include", header)).read()
    return sorted(set(re.findall(r"^\s*(?:int|void|const char\*)\s+(pp_\w+)\s*\(", src, re.M)))


def test_library_exports_all_declared_symbols(native_lib):
    out = subprocess.run(["nm", "-D", "--defined-only", native.LIB_PATH], capture_output=True, text=True).stdout
    exported = set(re.findall(r"\sT\s(pp_\w+)$", out, re.M))
    for name in _declared("paraprobe_gb300.h"):
        assert name in exported, name
    assert set(native.EXPORTS) <= exported


def test_strerror_without_gpu(native_lib):
    assert native_lib.pp_strerror(0) == b"ok"
    assert native_lib.pp_strerror(-4) == b"unsupported"
