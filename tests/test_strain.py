"""Uniaxial strain ramp (fix deform, x erate): the box grows as
L(t) = L0 (1 + R t) about its centre with affine remaps of the positions.
The reference has no box deformation, so the oracle's restatement is the
reference here (parity unpinned against the reference itself)."""
import numpy as np
import pytest

import cases as C

ERATE = 0.02  # per time unit: large, so that the remaps force neighbor rebuilds


def _oracle_run(O, name, steps):
    cfg, z = C.load_golden(name)
    m = C.model_from_arrays(z)
    o = O.Oracle(m, **C.settings_kwargs(cfg))
    o.setup()
    if m.natoms:
        o.atom_list()
        o.atom_forces()
    if m.nelements:
        o.elem_lists()
        o.elem_forces()
    o.set_deform([ERATE, 0.0, 0.0])
    lo0, hi0 = o.box()
    o.run(steps)
    return cfg, m, o, lo0, hi0


def test_oracle_box_follows_the_ramp(oracle_lib):
    steps = 40
    cfg, m, o, lo0, hi0 = _oracle_run(oracle_lib, "lj_cac", steps)
    lo, hi = o.box()
    dt = 0.005
    L = (hi0[0] - lo0[0]) * (1 + ERATE * steps * dt)
    assert abs((hi[0] - lo[0]) - L) <= 1e-12 * L
    assert abs(0.5 * (lo[0] + hi[0]) - 0.5 * (lo0[0] + hi0[0])) <= 1e-12 * L
    assert np.array_equal(lo[1:], lo0[1:]) and np.array_equal(hi[1:], hi0[1:])
    assert o.size(8) >= 1  # the remaps forced neighbor rebuilds


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["lj_cac", "eam_cac"])
def test_gpu_strain_ramp_matches_oracle(oracle_lib, cacg_lib, name):
    from gpu_runner import configure
    steps = 30
    cfg, m, o, _, _ = _oracle_run(oracle_lib, name, steps)
    s = cacg_lib.System(0)
    try:
        configure(s, cfg, m)
        s.command(f"fix 9 all deform 1 x erate {ERATE!r}")
        s.set_precision(cacg_lib.FP64_EXACT)
        s.init()
        s.setup()
        if m.natoms:
            s.neighbor_build()
            s.pair_compute()
        s.neighbor_ebuild()
        s.neighbor_nbuild()
        s.pair_ecompute()
        s.run(steps)
        lo, hi = s.box()
        olo, ohi = o.box()
        assert np.array_equal(lo, olo) and np.array_equal(hi, ohi)
        a, oa = s.atoms(), o.atoms()
        e, oe = s.elements(), o.elements()
        for k in ("x", "v", "f"):
            assert np.array_equal(a[k], oa[k]), k
        for k in ("nodex", "nodev", "nodef"):
            assert np.array_equal(e[k], oe[k]), k
        assert s.counts()["rebuilds"] == o.size(8)
        if name == "lj_cac":
            assert o.size(8) >= 1  # the remaps forced rebuilds (pbc, borders, bins)
    finally:
        s.close()


@pytest.mark.gpu
def test_mixed_error_along_the_ramp(oracle_lib, cacg_lib):
    """Mixed precision along a strain ramp: every 10 steps its configuration is
    evaluated in bit-exact FP64 by a second handle; forces, energy and virial
    agree within the mixed mode's tolerance."""
    from gpu_runner import configure
    cfg, z = C.load_golden("eam_cac")
    m = C.model_from_arrays(z)
    hs = []
    try:
        for mode in (cacg_lib.MIXED, cacg_lib.FP64_EXACT):
            s = cacg_lib.System(0)
            hs.append(s)
            configure(s, cfg, m)
            s.command(f"fix 9 all deform 1 x erate {ERATE!r}")
            s.set_precision(mode)
            s.init()
            s.setup()
            s.neighbor_build()
            s.neighbor_ebuild()
            s.neighbor_nbuild()
            s.pair_compute()
            s.pair_ecompute()
        mx, ex = hs
        for block in range(3):
            mx.run(10)
            ex.run(10)  # same box schedule
            a, e = mx.atoms(), mx.elements()
            assert np.array_equal(mx.box()[0], ex.box()[0])
            ex.put_atoms(a["x"], a["v"])
            ex.put_nodes(e["nodex"], e["nodev"])
            ex.setup()  # ghosts and bins for the positions just put
            ex.neighbor_build()
            ex.neighbor_ebuild()
            ex.neighbor_nbuild()
            for h in (mx, ex):
                h.pair_compute()
                h.pair_ecompute()
            fa, fe = mx.atoms()["f"], ex.atoms()["f"]
            na, ne = mx.elements()["nodef"], ex.elements()["nodef"]
            assert np.sqrt(((fa - fe) ** 2).sum() / (fe ** 2).sum()) < 1e-4, block
            assert np.sqrt(((na - ne) ** 2).sum() / (ne ** 2).sum()) < 1e-4, block
            tm, te = mx.thermo(), ex.thermo()
            pe_m, pe_e = tm["pe_atoms"] + tm["pe_elements"], te["pe_atoms"] + te["pe_elements"]
            assert abs(pe_m - pe_e) <= 1e-12 * abs(pe_e)  # energies are FP64 in every mode
            assert np.allclose(tm["virial"], te["virial"], rtol=1e-12, atol=0)
    finally:
        for h in hs:
            h.close()
