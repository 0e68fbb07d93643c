"""The CPU restatement (oracle/) against the reference's own outputs.

Golden fixtures come from the unmodified reference sources run through the
oracle harness (tests/golden/make_golden.py).  Every comparison is exact:
lists entry for entry, forces and trajectories bit for bit.
"""
import numpy as np
import pytest

import cases as C

NAMES = list(C.CASES)


def run_oracle(O, name):
    cfg, z = C.load_golden(name)
    m = C.model_from_arrays(z)
    o = O.Oracle(m, **C.settings_kwargs(cfg))
    am, em, fixes = C.fix_setup(cfg, m)
    if fixes:
        o.set_masks(am, em)
        for kind, bit, arg in fixes:
            if kind == "setforce":
                o.add_setforce(bit, arg)
            else:
                o.add_viscous(bit, arg)
    o.setup()
    out = {}
    if m.natoms:
        out["atom_numneigh"], out["atom_neigh"] = o.atom_list()
        a = o.atoms(all_=True)
        out["atom_tag_all"], out["atom_x_all"] = a["tag"], a["x"].reshape(-1)
        out["centro"] = o.centro()
        out["atom_f"] = o.atom_forces().reshape(-1)
    if m.nelements:
        enum, eneigh, ipn, ipj, ipnj = o.elem_lists()
        out.update(elem_numneigh=enum, elem_neigh=eneigh, ip_numneigh=ipn,
                   ip_neigh_elem=ipj, ip_neigh_site=ipnj, elem_cuts=o.cuts())
        out["nodef"] = o.elem_forces().reshape(-1)
    o.run(cfg["steps"])
    a = o.atoms()
    e = o.elements()
    out.update(s1_x=a["x"].reshape(-1), s1_v=a["v"].reshape(-1), s1_f=a["f"].reshape(-1),
               s1_nodex=e["nodex"].reshape(-1), s1_nodev=e["nodev"].reshape(-1),
               s1_nodef=e["nodef"].reshape(-1), s1_elem_x=e["x"].reshape(-1),
               rebuilds=np.array([o.size(8)]))
    return cfg, z, out


@pytest.mark.parametrize("name", NAMES)
def test_oracle_matches_reference(oracle_lib, name):
    cfg, z, out = run_oracle(oracle_lib, name)
    for k, v in out.items():
        ref = z["ref_" + k]
        assert v.shape == ref.shape, (k, v.shape, ref.shape)
        if v.dtype.kind == "f":
            assert np.array_equal(v.view(np.int64), ref.astype(np.float64).view(np.int64)), k
        else:
            assert np.array_equal(v, ref), k


def test_rebuilds_happened():
    # the forced-rebuild cases exercise pbc + borders + all three builders
    for name in ("lj_cac", "eam_atoms", "lj_cac_bigbins", "lj_cac_fixes"):
        cfg, z = C.load_golden(name)
        assert int(z["ref_rebuilds"][0]) >= 1, name
