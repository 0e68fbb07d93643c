"""Parity at the configurations' own sizes, against the CPU restatement of the
reference (the oracle) run on the same host.

* C1 in full (LJ, 16,384 atoms + 64 elements of 8 sites per edge), bit-exact
  FP64: the atom, element and integration-point lists entry for entry, atom
  and nodal forces bit for bit, and 200 Verlet steps through 20 full rebuilds
  (neigh_modify every 10 check no) bit for bit, atoms and nodes.  (Under the
  reference's element force the nodes' kinetic energy grows without bound;
  by step 260 the bin grid, sized from the elements' extent, no longer holds
  the atoms and the reference's algorithm stops: C1 cannot run its 1,000
  steps.)
* A C2-structured EAM slab of 100,672 atoms + 256 elements of 11 sites per
  edge (the element shape of C2, C3 and C5): the lists entry for entry and
  forces within 1e-12 of the force scale in FP64, within 1e-4 (RMS and max
  relative, atoms and nodes) in mixed precision.
"""
import os
import tempfile

import numpy as np
import pytest

from cac_code_gb300 import cacg
from cac_code_gb300 import workloads as W

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12
MIXED_TOL = 1e-4


def bits_equal(a, b):
    a, b = np.asarray(a), np.asarray(b)
    if a.dtype.kind == "f":
        return a.shape == b.shape and np.array_equal(a.astype(np.float64).view(np.int64),
                                                     b.astype(np.float64).view(np.int64))
    return a.shape == b.shape and np.array_equal(a, b)


def rel_err(f, ref):
    f = np.asarray(f, dtype=np.float64).reshape(-1, 3)
    ref = np.asarray(ref, dtype=np.float64).reshape(-1, 3)
    d = np.linalg.norm(f - ref, axis=1)
    n = np.linalg.norm(ref, axis=1)
    return float(np.sqrt((d ** 2).mean() / (n ** 2).mean())), float(d.max() / n.max())


def _system(m, cfg, eam, mode, commands=()):
    s = cacg.System(0)
    W.configure_system(s, m, cfg, eam)
    for c in commands:
        s.command(c)
    s.set_precision(mode)
    s.init()
    s.setup()
    s.neighbor_build()
    s.neighbor_ebuild()
    s.neighbor_nbuild()
    s.pair_compute()
    s.pair_ecompute()
    return s


def test_c1_full_bit_exact(cacg_lib, oracle_lib):
    m, cfg = W.c1_lj()
    cfg = dict(cfg, every=10, check=False)
    o = oracle_lib.Oracle(m, **W.oracle_kwargs(cfg))
    o.setup()
    num, nb = o.atom_list()
    enum, eneigh, ipn, ipj, ipnj = o.elem_lists()
    fa = o.atom_forces()
    fe = o.elem_forces()
    s = _system(m, cfg, "", cacg.FP64_EXACT,
                [f"neigh_modify every {cfg['every']} delay 0 check no"])
    try:
        gnum, gnb = s.atom_list()
        assert bits_equal(gnum, num) and bits_equal(gnb, nb)
        genum, geneigh, gipn, gipj, gipnj = s.elem_lists()
        assert bits_equal(genum, enum) and bits_equal(geneigh, eneigh)
        assert bits_equal(gipn, ipn) and bits_equal(gipj, ipj) and bits_equal(gipnj, ipnj)
        assert bits_equal(s.atoms()["f"], fa)
        assert bits_equal(s.elements()["nodef"], fe)
        o.run(200)
        s.run(200)
        assert s.counts()["rebuilds"] == 20
        a, e = s.atoms(), s.elements()
        ao, eo = o.atoms(), o.elements()
        for k in ("x", "v", "f"):
            assert bits_equal(a[k], ao[k]), k
        for k in ("nodex", "nodev", "nodef"):
            assert bits_equal(e[k], eo[k]), k
    finally:
        s.close()


@pytest.fixture(scope="module")
def c2_slab(oracle_lib):
    eam = W.write_eam(os.path.join(tempfile.mkdtemp(), "Cu_analytic_2000.eam"))
    m, cfg = W.c2_eam(cells=(13, 44, 44), layers=4, seed=17)
    o = oracle_lib.Oracle(m, **W.oracle_kwargs(cfg, eam))
    o.setup()
    lists = o.atom_list() + o.elem_lists()
    fa = o.atom_forces()
    fe = o.elem_forces()
    return m, cfg, eam, lists, fa, fe


def test_c2_slab_fp64_within_1e12(cacg_lib, c2_slab):
    m, cfg, eam, lists, fa, fe = c2_slab
    assert m.natoms >= 100000 and m.etypes[0].nae == (11, 11, 11)
    s = _system(m, cfg, eam, cacg.FP64)
    try:
        got = s.atom_list() + s.elem_lists()
        for g, r in zip(got, lists):
            assert bits_equal(g, r)
        f, nf = s.atoms()["f"], s.elements()["nodef"]
    finally:
        s.close()
    assert np.abs(f - fa).max() <= FP64_TOL * np.abs(fa).max()
    assert np.abs(nf - fe).max() <= FP64_TOL * np.abs(fe).max()


def test_c2_slab_mixed_within_1e4(cacg_lib, c2_slab):
    m, cfg, eam, lists, fa, fe = c2_slab
    s = _system(m, cfg, eam, cacg.MIXED)
    try:
        f, nf = s.atoms()["f"], s.elements()["nodef"]
    finally:
        s.close()
    for got, ref in ((f, fa), (nf, fe)):
        rms, mx = rel_err(got, ref)
        assert rms <= MIXED_TOL and mx <= MIXED_TOL, (rms, mx)
