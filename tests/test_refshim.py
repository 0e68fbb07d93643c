"""The reference-side plug-ins (cac_code_gb300/refshim: PairLJCutGPU,
PairEAMGPU, NeighborGPU, FixNVEGPU and their shared handle) compile against
the reference's headers (pair.h:82-105, neighbor.h:74-76, fix_nve.h) with the
reference's flags and link, with the reference's own objects, the single-rank
MPI stand-in and libcacg.so, into a program that runs.  Compile and link only:
no GPU call.  Skipped where the reference tree is absent."""
import glob
import os
import subprocess
import tempfile

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SHIM = os.path.join(ROOT, "cac_code_gb300", "refshim")


def test_plugins_compile_and_link(cacg_lib):
    from oracle import oracle as O
    if not os.path.isdir(O.REF_TREE):
        pytest.skip("reference tree absent")
    O.build(ref=True)
    objs = sorted(o for o in glob.glob(os.path.join(ROOT, "oracle", "_ref", "obj", "*.o"))
                  if not o.endswith("harness.o"))
    assert objs
    wd = tempfile.mkdtemp(prefix="refshim_")
    flags = ["-std=gnu++98", "-fpermissive", "-w", "-O1", "-I" + O.REF_TREE,
             "-I" + os.path.join(ROOT, "oracle", "ref"), "-I" + os.path.join(ROOT, "include"),
             "-I" + SHIM]
    srcs = sorted(glob.glob(os.path.join(SHIM, "*.cpp"))) + [
        os.path.join(ROOT, "tests", "refshim_link_main.cpp")]
    out = []
    for src in srcs:
        o = os.path.join(wd, os.path.basename(src) + ".o")
        p = subprocess.run(["g++"] + flags + ["-c", src, "-o", o], capture_output=True, text=True)
        assert p.returncode == 0, p.stderr[-3000:]
        out.append(o)
    libdir = os.path.dirname(cacg_lib._build.LIB)
    exe = os.path.join(wd, "refshim_link")
    p = subprocess.run(["g++", "-o", exe] + out + objs +
                       ["-L" + libdir, "-lcacg", "-Wl,-rpath," + libdir, "-lm"],
                       capture_output=True, text=True)
    assert p.returncode == 0, p.stderr[-3000:]
    p = subprocess.run([exe], capture_output=True, text=True)
    assert p.returncode == 0, p.stderr
