"""CPU-side checks of the C-ABI library: it builds for sm_103a, loads, and
exports every entry point include/newt_gpu.h declares.  No GPU calls."""
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    names = []
    for f in os.listdir(os.path.join(ROOT, "include")):
        if f.endswith(".h"):
            src = open(os.path.join(ROOT, "include", f)).read()
            names += re.findall(r"NEWT_API\s+[\w\s\*]+?\b(newt_gpu_\w+)\s*\(", src)
    return sorted(set(names))


@pytest.fixture(scope="module")
def lib_path():
    from tooling_gb300 import build as B
    return B.build()


def test_header_declares_entry_points():
    names = _declared()
    assert "newt_gpu_step" in names and "newt_gpu_create" in names
    assert len(names) >= 20


def test_library_exports_every_declared_symbol(lib_path):
    out = subprocess.run(["nm", "-D", "--defined-only", lib_path], capture_output=True, text=True).stdout
    exported = set(re.findall(r"\bT (newt_gpu_\w+)", out))
    missing = [n for n in _declared() if n not in exported]
    assert not missing, missing


def test_library_loads_and_python_binding_matches_header(lib_path):
    from tooling_gb300 import api
    L = api.load_library(lib_path)
    for n in _declared():
        assert hasattr(L, n)
    assert sorted(api.EXPORTED) == _declared()


def test_build_targets_sm_103a_only():
    from tooling_gb300 import build as B
    assert B.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]
