"""GPU path (libcacg, sm_103a) against the reference.

* FP64_EXACT: neighbor lists identical entry for entry, forces and Verlet
  trajectories bit-identical to the reference's golden outputs and to the CPU
  restatement run on the same host.
* FP64 (fused multiply-add): lists identical; forces within 1e-12 of the force
  scale (max |f| of the reference) -- the FP64 tolerance of the path.
"""
import numpy as np
import pytest

import cases as C
from cac_code_gb300 import cacg

pytestmark = pytest.mark.gpu

NAMES = list(C.CASES)
FP64_TOL = 1e-12   # relative to the force scale


def bits_equal(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    if a.dtype.kind == "f":
        return a.shape == b.shape and np.array_equal(a.astype(np.float64).view(np.int64),
                                                     b.astype(np.float64).view(np.int64))
    return a.shape == b.shape and np.array_equal(a, b)


@pytest.mark.parametrize("name", NAMES)
def test_exact_mode_matches_reference_golden(cacg_lib, name):
    from gpu_runner import run_gpu
    cfg, z = C.load_golden(name)
    m = C.model_from_arrays(z)
    out = run_gpu(cfg, m, cacg.FP64_EXACT)
    for k, v in out.items():
        if k.startswith("_"):
            continue
        assert bits_equal(v, z["ref_" + k]), k


@pytest.mark.parametrize("name", ["lj_cac", "eam_atoms"])
def test_input_script_path_matches_golden(cacg_lib, name):
    """Same case driven by pair_style/pair_coeff/neighbor/fix commands and read_data."""
    from gpu_runner import run_gpu
    cfg, z = C.load_golden(name)
    m = C.model_from_arrays(z)
    out = run_gpu(cfg, m, cacg.FP64_EXACT, via_files=True)
    for k in ("atom_neigh", "atom_f", "s1_x", "s1_v"):
        assert bits_equal(out[k], z["ref_" + k]), k
    if m.nelements:
        for k in ("ip_neigh_site", "nodef", "s1_nodex"):
            assert bits_equal(out[k], z["ref_" + k]), k


@pytest.mark.parametrize("name", ["lj_cac", "eam_cac", "eam_atoms"])
def test_fma_mode_within_fp64_tolerance(cacg_lib, name):
    from gpu_runner import run_gpu
    cfg, z = C.load_golden(name)
    m = C.model_from_arrays(z)
    out = run_gpu(cfg, m, cacg.FP64, steps=0)
    for k in ("atom_numneigh", "atom_neigh", "ip_numneigh", "ip_neigh_elem", "ip_neigh_site"):
        if k in out:
            assert bits_equal(out[k], z["ref_" + k]), k
    for k in ("atom_f", "nodef"):
        if k in out:
            ref = z["ref_" + k]
            scale = np.abs(ref).max()
            assert np.abs(out[k] - ref).max() <= FP64_TOL * scale, k


def test_exact_mode_matches_oracle_larger_slab(cacg_lib, oracle_lib):
    """A larger LJ CAC slab than the fixtures, oracle run on this host."""
    from gpu_runner import run_gpu
    cfg = dict(C.CASES["lj_cac"])
    cfg.update(cells=(6, 16, 16), nae=8, layers=2, seed=21, steps=3, check=True, every=1)
    m = C.build_model(cfg)
    out = run_gpu(cfg, m, cacg.FP64_EXACT)
    o = oracle_lib.Oracle(m, **C.settings_kwargs(cfg))
    o.setup()
    num, nb = o.atom_list()
    assert bits_equal(out["atom_numneigh"], num) and bits_equal(out["atom_neigh"], nb)
    assert bits_equal(out["atom_f"], o.atom_forces().reshape(-1))
    enum, eneigh, ipn, ipj, ipnj = o.elem_lists()
    assert bits_equal(out["ip_numneigh"], ipn) and bits_equal(out["ip_neigh_site"], ipnj)
    assert bits_equal(out["nodef"], o.elem_forces().reshape(-1))
    o.run(cfg["steps"])
    assert bits_equal(out["s1_x"], o.atoms()["x"].reshape(-1))
    assert bits_equal(out["s1_nodex"], o.elements()["nodex"].reshape(-1))


def test_fma_mode_large_coordinates(cacg_lib, oracle_lib):
    """Elements far from the origin (|x| up to ~200 A): the fast FP64 mode must
    still agree with the reference arithmetic within 1e-12 of the force scale."""
    from cac_code_gb300 import workloads as W
    import os
    import tempfile
    eam = W.write_eam(os.path.join(tempfile.mkdtemp(), "Cu.eam"), n=2000)
    m, cfg = W.c2_sample(seed=9)
    s = cacg.System(0)
    try:
        W.configure_system(s, m, cfg, eam)
        s.set_precision(cacg.FP64)
        s.init()
        s.setup()
        s.neighbor_build()
        s.neighbor_ebuild()
        s.neighbor_nbuild()
        s.pair_compute()
        s.pair_ecompute()
        f = s.atoms()["f"]
        nf = s.elements()["nodef"]
    finally:
        s.close()
    o = oracle_lib.Oracle(m, **W.oracle_kwargs(cfg, eam))
    o.setup()
    o.atom_list()
    fr = o.atom_forces()
    o.elem_lists()
    nfr = o.elem_forces()
    assert np.abs(f - fr).max() <= FP64_TOL * np.abs(fr).max()
    assert np.abs(nf - nfr).max() <= FP64_TOL * np.abs(nfr).max()
