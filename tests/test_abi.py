"""The C ABI library loads and exports every entry point include/cacg.h declares.
No compute call is made (this suite runs without a GPU)."""
import ctypes
import os
import re

import cases  # noqa: F401  (sys.path set by conftest)

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared():
    src = open(os.path.join(ROOT, "include", "cacg.h")).read()
    return sorted(set(re.findall(r"\b(cacg_[a-z0-9_]+)\s*\(", src)))


def test_header_and_binding_agree(cacg_lib):
    assert declared() == sorted(cacg_lib.EXPORTED)


def test_library_exports_all_symbols(cacg_lib):
    lib = ctypes.CDLL(cacg_lib._build.LIB)
    for name in declared():
        assert hasattr(lib, name), name


def test_version_string(cacg_lib):
    lib = cacg_lib.load()
    assert b"sm_103a" in lib.cacg_version()


def test_create_without_gpu_fails_cleanly(cacg_lib):
    # on a host without a GPU the ABI reports a CUDA status instead of crashing
    import subprocess, sys
    code = ("import ctypes,sys; sys.path.insert(0,%r);"
            "from cac_code_gb300 import cacg; lib=cacg.load();"
            "h=ctypes.c_void_p(); rc=lib.cacg_create(ctypes.byref(h),0);"
            "print(rc)") % ROOT
    env = dict(os.environ, CUDA_VISIBLE_DEVICES="")
    p = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, env=env)
    assert p.returncode == 0, p.stderr
    assert int(p.stdout.strip().splitlines()[-1]) == -3
