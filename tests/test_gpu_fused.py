"""Fused element passes (one warp per element: lattice lines as FP32 offsets
from the element's centre in shared memory, guard-band pairs decided in FP64)
against the unfused passes and against bit-exact FP64 forces.

The fused path runs when every integration-point list entry references its
row's own element; the C2 sample's elements (11 sites per edge) are such
elements, since the reference's element lists find no other element centre
within their neighbor stencil (element_neighbor.cpp:11-75).
"""
import os
import tempfile

import numpy as np
import pytest

from cac_code_gb300 import cacg
from cac_code_gb300 import workloads as W

pytestmark = pytest.mark.gpu

TOL = 1e-4


def rel_err(f, ref):
    f = np.asarray(f, dtype=np.float64).reshape(-1, 3)
    ref = np.asarray(ref, dtype=np.float64).reshape(-1, 3)
    d = np.linalg.norm(f - ref, axis=1)
    n = np.linalg.norm(ref, axis=1)
    return float(np.sqrt((d ** 2).mean() / (n ** 2).mean())), float(d.max() / n.max())


def _run(mode, fused, steps, vscale, eam):
    m, cfg = W.c2_sample(seed=13)
    m.atom_v = m.atom_v * vscale
    m.nodev = m.nodev * vscale
    s = cacg.System(0)
    try:
        W.configure_system(s, m, cfg, eam)
        s.set_precision(mode)
        s.command(f"tune fused {'yes' if fused else 'no'}")
        s.init()
        s.setup()
        s.neighbor_build()
        s.neighbor_ebuild()
        s.neighbor_nbuild()
        s.pair_compute()
        s.pair_ecompute()
        c = s.counts()
        first = (s.atoms()["f"].copy(), s.elements()["nodef"].copy(), c["elem_fused"])
        s.run(steps)
        return first, s.atoms(), s.elements(), s.counts()
    finally:
        s.close()


@pytest.fixture(scope="module")
def eam_file():
    return W.write_eam(os.path.join(tempfile.mkdtemp(), "Cu_analytic_2000.eam"))


@pytest.mark.parametrize("vscale", [1.0, 40.0])
def test_fused_passes_match_unfused_and_fp64(cacg_lib, eam_file, vscale):
    """Nodal forces of one evaluation within 1e-5 of the unfused passes and
    within 1e-4 of bit-exact FP64; 25 steps (a rebuild decision, and at 40x
    the thermal speeds list reorders) stay within 1e-6 A of the unfused run."""
    f0, a0, e0, c0 = _run(cacg.MIXED, False, 25, vscale, eam_file)
    f1, a1, e1, c1 = _run(cacg.MIXED, True, 25, vscale, eam_file)
    fx, _, _, _ = _run(cacg.FP64_EXACT, False, 0, vscale, eam_file)
    assert f0[2] == 0 and f1[2] == 1, "the fused path must run only where asked"
    assert np.array_equal(f0[0], f1[0])  # atom passes untouched
    rms, mx = rel_err(f1[1], f0[1])
    assert rms <= 1e-5 and mx <= 1e-5, (rms, mx)
    rms, mx = rel_err(f1[1], fx[1])
    assert rms <= TOL and mx <= TOL, (rms, mx)
    assert np.abs(e1["nodex"] - e0["nodex"]).max() < 1e-6
    assert np.abs(a1["x"] - a0["x"]).max() < 1e-6
    if vscale > 1.0:
        assert c1["ip_reorders"] >= 2, c1["ip_reorders"]


def test_fused_passes_off_for_foreign_entries(cacg_lib):
    """Lists whose rows reference other elements' sites (a bin size that
    covers the element cutoff) keep the unfused passes."""
    import cases as C
    from gpu_runner import run_gpu
    cfg, z = C.load_golden("lj_cac_bigbins")
    m = C.model_from_arrays(z)
    out = run_gpu(cfg, m, cacg.MIXED, steps=0)
    assert out["_counts"]["elem_fused"] == 0


def test_fused_variants_bit_identical(cacg_lib, eam_file):
    """The three kernel arrangements of the fused passes (coefficients in
    registers, in shared memory, two entries in flight) give the same bits."""
    m, cfg = W.c2_sample(seed=13)
    s = cacg.System(0)
    try:
        W.configure_system(s, m, cfg, eam_file)
        s.set_precision(cacg.MIXED)
        s.init()
        s.setup()
        s.neighbor_build()
        s.neighbor_ebuild()
        s.neighbor_nbuild()
        out = []
        for v in (0, 1, 2):
            s.command(f"tune fused_variant {v}")
            s.pair_ecompute()
            assert s.counts()["elem_fused"] == 1
            out.append(s.elements()["nodef"].copy())
    finally:
        s.close()
    for o in out[1:]:
        assert np.array_equal(o.view(np.int64), out[0].view(np.int64))


def _band_run(m, cfg, eam_file, band, variant, steps=8, cull=True):
    s = cacg.System(0)
    try:
        W.configure_system(s, m, cfg, eam_file)
        s.set_precision(cacg.MIXED)
        s.command(f"tune fused_variant {variant}")
        s.command(f"tune cull {'yes' if cull else 'no'}")
        if band is not None:
            s.command(f"tune band {band}")
        s.init()
        s.setup()
        s.neighbor_build()
        s.neighbor_ebuild()
        s.neighbor_nbuild()
        s.pair_compute()
        s.pair_ecompute()
        s.run(steps)
        return s.atoms(), s.elements(), s.counts()
    finally:
        s.close()


def _lj_sample():
    """LJ elements of 11 sites per edge; the skin (2.8) is the whole list
    cutoff (Neighbor::init sets cutneighmax = skin, neighbor.cpp:297-374), as
    in C1; no element sees another's sites, so the fused LJ pass runs."""
    from cac_code_gb300 import lattice as L
    m = L.make_slab_model(W.A_LJ, 1.0, (6, 22, 22), 11, 4, L.gauss_intp(11, False))
    L.thermalize(m, 0.1, W.KB["lj"], W.MVV2E["lj"], 5)
    L.remap_into_box(m)
    cfg = dict(units="lj", boundary="f p p", pair="lj/cut", lj=(1.0, 1.0, 2.5), skin=2.8,
               every=4, delay=0, check=True, dt=0.005, gauss_per_element=8)
    return m, cfg


@pytest.mark.parametrize("pot,variant", [("eam", 0), ("eam", 1), ("eam", 2), ("lj", 1)])
def test_guard_band_reruns_are_exact(cacg_lib, eam_file, pot, variant):
    """A pair of an element whose FP32 distance falls in the guard band has
    the element re-run by the exact pass (FP64 decisions).  Widened to
    cutsq (1 +- 0.1), the band holds a lattice shell (EAM Cu: the sixth at
    +8 %; LJ: the fifth at +0.8 %, scanned with the displacement culling off),
    so every element is re-run at every pass; decisions outside the default
    band agree in FP32 and FP64, so positions and forces stay bit-identical to
    the default band's over 8 steps."""
    if pot == "eam":
        m, cfg = W.c2_sample(seed=13)
    else:
        m, cfg = _lj_sample()
    cull = pot == "eam"
    a0, e0, c0 = _band_run(m, cfg, eam_file, None, 1, cull=cull)
    a1, e1, c1 = _band_run(m, cfg, eam_file, 0.1, variant, cull=cull)
    assert c0["elem_fused"] == 1 and c1["elem_fused"] == 1
    passes = (2 if pot == "eam" else 1) * (1 + 8)
    assert c1["band_reruns"] >= passes * c1["enlocal"], (c1["band_reruns"], c1["enlocal"])
    assert c0["band_reruns"] < c1["band_reruns"]
    for k in ("x", "v", "f"):
        assert np.array_equal(a0[k], a1[k]), k
    for k in ("nodex", "nodev", "nodef"):
        assert np.array_equal(e0[k], e1[k]), k
