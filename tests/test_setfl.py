"""The setfl (eam/alloy) reader: a one-element setfl file with the golden
funcfl file's grids gives the same tables, hence the reference's outputs bit
for bit."""
import numpy as np
import pytest

import cases as C
from cac_code_gb300 import lattice as L


def _numbers(path, skip):
    with open(path) as f:
        lines = f.read().splitlines()[skip:]
    return np.array([float(v) for line in lines for v in line.split()])


def test_funcfl_to_setfl_keeps_the_numbers(tmp_path):
    path = str(tmp_path / "Cu.setfl")
    L.funcfl_to_setfl(C.EAM_FILE, path)
    assert np.array_equal(_numbers(C.EAM_FILE, 3), _numbers(path, 6))


def test_setfl_and_funcfl_tables_agree(tmp_path):
    pot = L.AnalyticEAM()
    f1, f2 = str(tmp_path / "a.eam"), str(tmp_path / "a.setfl")
    L.write_eam_funcfl(pot, f1, nrho=800, nr=800)
    L.write_eam_setfl(pot, f2, nrho=800, nr=800)
    a = _numbers(f1, 3)
    b = _numbers(f2, 6)
    assert a.shape == b.shape and np.array_equal(a, b)
    h1 = open(f1).read().splitlines()[2].split()
    h2 = open(f2).read().splitlines()[4].split()
    assert h1 == h2


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["eam_cac", "eam_atoms"])
def test_eam_alloy_matches_reference_golden(cacg_lib, tmp_path, name):
    from gpu_runner import run_gpu
    # the committed funcfl file's own numbers (tables computed on another
    # host could differ in the last bit)
    path = str(tmp_path / "Cu.setfl")
    L.funcfl_to_setfl(C.EAM_FILE, path)
    cfg, z = C.load_golden(name)
    m = C.model_from_arrays(z)
    out = run_gpu(cfg, m, cacg_lib.FP64_EXACT,
                  pair_lines=["pair_style eam/alloy", f"pair_coeff * * {path} Cu"])
    for k, v in out.items():
        if k.startswith("_"):
            continue
        ref = z["ref_" + k]
        assert np.array_equal(np.asarray(v).view(np.uint8), np.asarray(ref, dtype=v.dtype).view(np.uint8)), k


@pytest.mark.gpu
def test_eam_alloy_rejects_unknown_element(cacg_lib, tmp_path):
    path = str(tmp_path / "Cu.setfl")
    L.write_eam_setfl(L.AnalyticEAM(), path, nrho=800, nr=800)
    s = cacg_lib.System(0)
    try:
        s.command("units metal")
        s.command("boundary p p p")
        cfg, z = C.load_golden("eam_atoms")
        s.load_model(C.model_from_arrays(z))
        s.command("pair_style eam/alloy")
        with pytest.raises(cacg_lib.CacgError):
            s.command(f"pair_coeff * * {path} Ni")
    finally:
        s.close()
