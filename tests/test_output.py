"""The reference's outputs written from device state: the xyz dump of
centro-symmetry defects and the Tecplot element dump."""
import os

import numpy as np
import pytest

import cases as C


def _system(cacg, name):
    from gpu_runner import configure
    cfg, z = C.load_golden(name)
    m = C.model_from_arrays(z)
    s = cacg.System(0)
    configure(s, cfg, m)
    s.set_precision(cacg.FP64_EXACT)
    s.init()
    s.setup()
    s.neighbor_build()
    if m.nelements:
        s.neighbor_ebuild()
        s.neighbor_nbuild()
    return s, z


@pytest.mark.gpu
def test_xyz_dump_lists_the_centro_defects(cacg_lib, tmp_path):
    s, z = _system(cacg_lib, "eam_cac")
    try:
        path = str(tmp_path / "defects.xyz")
        s.dump_xyz(path)
        c = s.centro()
        x = s.atoms()["x"]
    finally:
        s.close()
    assert np.array_equal(c, z["ref_centro"])
    sel = (c > 1) & (c < 10)
    lines = open(path).read().splitlines()
    assert lines[0] == str(int(sel.sum())) and lines[1] == "XYZ"
    want = ["Cu %g %g %g %g" % (x[i, 0], x[i, 1], x[i, 2], c[i]) for i in np.nonzero(sel)[0]]
    assert lines[2:] == want


@pytest.mark.gpu
def test_element_dump_zone(cacg_lib, tmp_path):
    s, _ = _system(cacg_lib, "lj_cac")
    try:
        s.pair_ecompute()
        e = s.elements()
        path = str(tmp_path / "elements.dat")
        s.dump_elements(path)
        s.dump_elements(path, append=True)
    finally:
        s.close()
    ne = e["nodex"].shape[0]
    lines = open(path).read().splitlines()
    zone = 3 + 8 * ne + ne
    assert len(lines) == 2 * zone
    assert lines[0] == 'title="results for cac"'
    assert lines[2] == f'zone t="load step 0", n=  {8 * ne} e =  {ne} datapacking=point, zonetype=febrick'
    node = [" ".join("%g" % v for v in np.concatenate([e["nodex"][i, k], e["nodev"][i, k],
                                                       e["nodef"][i, k]]))
            for i in range(ne) for k in range(8)]
    assert lines[3:3 + 8 * ne] == node
    assert lines[3 + 8 * ne] == "1 2 3 4 5 6 7 8"
    assert lines[zone - 1] == " ".join(str(8 * (ne - 1) + k) for k in range(1, 9))
