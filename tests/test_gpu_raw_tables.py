"""Pair tables handed over as the reference built them (cacg_set_lj,
cacg_set_eam): a reference-side Pair subclass whose base class already read
the potential passes its tables instead of a file.  With the reference's own
tables, dumped by its harness into the golden fixtures, the bit-exact mode
reproduces the golden lists, forces and trajectory bit for bit."""
import numpy as np
import pytest

import cases as C
from cac_code_gb300 import cacg

pytestmark = pytest.mark.gpu

KEYS = ("atom_neigh", "atom_f", "nodef", "s1_x", "s1_v", "s1_nodex", "s1_nodev")


def bits_equal(a, b):
    a, b = np.asarray(a, dtype=np.float64), np.asarray(b, dtype=np.float64)
    return a.shape == b.shape and np.array_equal(a.view(np.int64), b.view(np.int64))


@pytest.mark.parametrize("name", ["lj_cac", "eam_cac"])
def test_reference_tables_give_golden_outputs(cacg_lib, name):
    from gpu_runner import run_gpu
    cfg, z = C.load_golden(name)
    m = C.model_from_arrays(z)
    kw = C.settings_kwargs(cfg)
    if cfg["pair"] == "eam":
        sc = z["ref_eam_scalars"]
        lines = ["pair_style eam"]

        def hand_over(s):
            s.set_eam(int(sc[0]), sc[1], int(sc[2]), sc[3], z["ref_eam_frho"], z["ref_eam_rhor"],
                      z["ref_eam_z2r"], sc[4], sc[5])
    else:
        lines = [f"pair_style lj/cut {kw['lj'][2]!r}"]

        def hand_over(s):
            s.set_lj(z["ref_lj_lj1"], z["ref_lj_lj2"], z["ref_lj_cutsq"])
    out = run_gpu(cfg, m, cacg.FP64_EXACT, pair_lines=lines, before_init=hand_over)
    for k in KEYS:
        if "ref_" + k in z.files and k in out:
            assert bits_equal(out[k], z["ref_" + k]), k


def test_tables_refused_before_pair_style(cacg_lib):
    s = cacg.System(0)
    try:
        with pytest.raises(cacg.CacgError):
            s.set_lj(np.zeros(4), np.zeros(4), np.ones(4))
    finally:
        s.close()
