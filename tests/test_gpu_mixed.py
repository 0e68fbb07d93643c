"""Mixed precision (FP32 pair terms, FP64 accumulation, embedding derivative and
integration) against the reference's FP64 forces: relative force error <= 1e-4.

Errors are measured two ways on every atom and node: RMS of |df| over RMS of |f|
and max |df| over max |f|.  The neighbor lists are the FP64 lists (identical).
"""
import numpy as np
import pytest

import cases as C
from cac_code_gb300 import cacg

pytestmark = pytest.mark.gpu

TOL = 1e-4


def rel_err(f, ref):
    f = np.asarray(f, dtype=np.float64).reshape(-1, 3)
    ref = np.asarray(ref, dtype=np.float64).reshape(-1, 3)
    d = np.linalg.norm(f - ref, axis=1)
    n = np.linalg.norm(ref, axis=1)
    return float(np.sqrt((d ** 2).mean() / (n ** 2).mean())), float(d.max() / n.max())


@pytest.mark.parametrize("name", ["lj_atoms", "lj_cac", "eam_cac", "eam_atoms"])
def test_mixed_forces_within_1e4(cacg_lib, name):
    from gpu_runner import run_gpu
    cfg, z = C.load_golden(name)
    m = C.model_from_arrays(z)
    out = run_gpu(cfg, m, cacg.MIXED, steps=0)
    for k in ("atom_f", "nodef"):
        if k in out:
            rms, mx = rel_err(out[k], z["ref_" + k])
            assert rms <= TOL and mx <= TOL, (k, rms, mx)


def test_mixed_trajectory_close_to_fp64(cacg_lib):
    """Ten NVE steps in mixed precision stay close to the FP64 trajectory."""
    from gpu_runner import run_gpu
    cfg, z = C.load_golden("eam_cac")
    m = C.model_from_arrays(z)
    a = run_gpu(cfg, m, cacg.MIXED, steps=10)
    b = run_gpu(cfg, m, cacg.FP64, steps=10)
    assert np.abs(a["s1_x"] - b["s1_x"]).max() < 1e-6
    assert np.abs(a["s1_nodex"] - b["s1_nodex"]).max() < 1e-6
