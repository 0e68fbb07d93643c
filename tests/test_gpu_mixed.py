"""Mixed precision against the reference's FP64 forces: relative force error
<= 1e-4.  Mixed mode evaluates pair terms in FP32; F'(rho) of atoms from the
FP64 spline at the FP64 density ("tune fprime fp64", the default; "fp32" takes
the FP32 spline), of integration points from the FP64 spline arithmetic carried
out in double-single, of element sites in FP32; it sums chunks of 8 pairs in
FP32 and the chunks as FP32 double-single pairs, and integrates in FP64.

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


def _run_cull(cacg, cfg, m, cull, steps, tune=(), graphs=True):
    from gpu_runner import configure
    s = cacg.System(0)
    try:
        configure(s, cfg, m)
        s.set_precision(cacg.MIXED)
        s.command(f"tune cull {cull}")
        for t in tune:
            s.command(f"tune {t}")
        s.set_graphs(graphs)
        s.init()
        s.setup()
        s.neighbor_build()
        s.pair_compute()
        if m.nelements:
            s.neighbor_ebuild()
            s.neighbor_nbuild()
            s.pair_ecompute()
        s.run(steps)
        return s.atoms(), s.elements(), s.counts()
    finally:
        s.close()


@pytest.mark.parametrize("case", ["eam_atoms", "eam_cac"])
@pytest.mark.parametrize("vscale", [1.0, 5.0, 40.0])
def test_displacement_culling_is_bit_identical(cacg_lib, case, vscale):
    """The density pass skips atom-list entries beyond r_c + 1 A at the list
    reorder, and both integration-point passes skip such entries of their rows
    (their sites are not even computed), while no atom (node) has moved 0.495 A
    since: the skipped entries are provably out of range, so the trajectory
    equals the unculled one bit for bit, with thermal motion (culling engaged
    throughout), faster motion (lists reordered again on the device between
    builds) and motion fast enough to force rebuilds."""
    cfg, z = C.load_golden(case)
    cfg = dict(cfg, every=10, check=True)
    m = C.model_from_arrays(z)
    m.atom_v = m.atom_v * vscale
    if m.nelements:
        m.nodev = m.nodev * vscale
    a0, e0, c0 = _run_cull(cacg_lib, cfg, m, "no", 40)
    a1, e1, c1 = _run_cull(cacg_lib, cfg, m, "yes", 40)
    assert c0["rebuilds"] == c1["rebuilds"]
    for k in ("x", "v", "f"):
        assert np.array_equal(a0[k], a1[k]), k
    for k in ("nodex", "nodev", "nodef"):
        assert np.array_equal(e0[k], e1[k]), k


@pytest.mark.parametrize("graphs", [True, False])
def test_two_stream_step_is_bit_identical(cacg_lib, graphs):
    """A mixed step runs its atom chain and its element chain on two streams
    (they do not interact); the trajectory equals the one-stream trajectory bit
    for bit, in graph replays and eager steps, across device-side list
    reorders and rebuilds."""
    cfg, z = C.load_golden("eam_cac")
    cfg = dict(cfg, every=10, check=True)
    m = C.model_from_arrays(z)
    m.atom_v = m.atom_v * 5.0
    m.nodev = m.nodev * 5.0
    a0, e0, c0 = _run_cull(cacg_lib, cfg, m, "yes", 40, tune=("streams no",), graphs=graphs)
    a1, e1, c1 = _run_cull(cacg_lib, cfg, m, "yes", 40, tune=("streams yes",), graphs=graphs)
    assert c0["rebuilds"] == c1["rebuilds"]
    for k in ("x", "v", "f"):
        assert np.array_equal(a0[k], a1[k]), k
    for k in ("nodex", "nodev", "nodef"):
        assert np.array_equal(e0[k], e1[k]), k


def _prepared(cacg, cfg, m, precision):
    from gpu_runner import configure
    s = cacg.System(0)
    configure(s, cfg, m)
    s.set_precision(precision)
    s.init()
    s.setup()
    s.neighbor_build()
    s.pair_compute()
    s.neighbor_ebuild()
    s.neighbor_nbuild()
    s.pair_ecompute()
    return s


def _host_array(a, pinned):
    if not pinned:
        return np.ascontiguousarray(a, dtype=np.float64)
    import torch
    h = torch.empty(a.shape, dtype=torch.float64).pin_memory().numpy()
    h[...] = a
    return h


@pytest.mark.parametrize("precision,pinned,vscale", [("MIXED", False, 5.0), ("MIXED", True, 5.0),
                                                     ("FP64", False, 5.0), ("MIXED", True, 20.0)])
def test_run_host_matches_device_resident_run(cacg_lib, precision, pinned, vscale):
    """cacg_run_host (state copied in from host buffers, stepped, copied back,
    with the last step's copies overlapping its computation in mixed precision,
    and on reused pinned buffers the whole call replayed as one graph) gives
    the device-resident trajectory bit for bit: one step per call across
    rebuild decisions, then several steps per call.  At 20x the velocities a
    decision step rebuilds (the atom chain that ran ahead of the decision is
    discarded and the step redone on the new lists)."""
    cfg, z = C.load_golden("eam_cac")
    cfg = dict(cfg, every=10, check=True)
    m = C.model_from_arrays(z)
    m.atom_v = m.atom_v * vscale
    m.nodev = m.nodev * vscale
    prec = getattr(cacg_lib, precision)
    a = _prepared(cacg_lib, cfg, m, prec)
    b = _prepared(cacg_lib, cfg, m, prec)
    try:
        x0 = a.atoms()
        e0 = a.elements()
        hx = _host_array(x0["x"], pinned)
        hv = _host_array(x0["v"], pinned)
        hnx = _host_array(e0["nodex"], pinned)
        hnv = _host_array(e0["nodev"], pinned)
        for _ in range(23):
            a.run_host(1, hx, hv, hnx, hnv)
        single_graph_steps = a.counts()["graph_steps"]
        a.run_host(7, hx, hv, hnx, hnv)
        b.run(30)
        xb, eb = b.atoms(), b.elements()
        assert np.array_equal(hx, xb["x"])
        assert np.array_equal(hv, xb["v"])
        assert np.array_equal(hnx, eb["nodex"])
        assert np.array_equal(hnv, eb["nodev"])
        ca = a.counts()
        assert ca["rebuilds"] == b.counts()["rebuilds"]
        if vscale > 10.0:
            assert ca["rebuilds"] >= 1
        if pinned:  # single-step calls replayed the whole-call graph
            assert single_graph_steps > 0
    finally:
        a.close()
        b.close()


@pytest.mark.parametrize("parts", [1, 3])
def test_run_host_element_heavy_state(cacg_lib, tmp_path, parts):
    """As above with more node state than atom state (a slab of two cells
    between forty element layers a side, the C5 proportions): the atom state
    goes in first and the atoms' velocities go out while the elements run;
    with "tune out_parts 3" the element force pass runs in three parts whose
    node velocities are integrated and copied out part by part.  The
    trajectory is still the device-resident one bit for bit."""
    from cac_code_gb300 import workloads as W
    eam = W.write_eam(str(tmp_path / "Cu.eam"))
    m, cfg = W.c2_eam(cells=(2, 22, 22), layers=40, seed=7)
    cfg = dict(cfg, every=10, check=True)
    assert m.nelements * 192 > m.natoms * 24

    def prepared():
        s = cacg_lib.System(0)
        W.configure_system(s, m, cfg, eam)
        s.set_precision(cacg_lib.MIXED)
        s.command(f"tune out_parts {parts}")
        s.init()
        s.setup()
        s.neighbor_build()
        s.pair_compute()
        s.neighbor_ebuild()
        s.neighbor_nbuild()
        s.pair_ecompute()
        return s

    a, b = prepared(), prepared()
    try:
        x0, e0 = a.atoms(), a.elements()
        hx, hv = _host_array(x0["x"], True), _host_array(x0["v"], True)
        hnx, hnv = _host_array(e0["nodex"], True), _host_array(e0["nodev"], True)
        for _ in range(23):
            a.run_host(1, hx, hv, hnx, hnv)
        a.run_host(7, hx, hv, hnx, hnv)
        b.run(30)
        xb, eb = b.atoms(), b.elements()
        assert np.array_equal(hx, xb["x"])
        assert np.array_equal(hv, xb["v"])
        assert np.array_equal(hnx, eb["nodex"])
        assert np.array_equal(hnv, eb["nodev"])
        assert a.counts()["rebuilds"] == b.counts()["rebuilds"]
    finally:
        a.close()
        b.close()


def test_union_variant_agrees_with_direct_passes(cacg_lib):
    """`tune union yes` stages each warp's neighbor union in shared memory and
    walks the build-order lists (the direct passes walk the reordered ones, so
    the FP32 sums differ in order only): forces agree to FP32 rounding, and a
    short trajectory stays together."""
    cfg, z = C.load_golden("eam_atoms")
    m = C.model_from_arrays(z)
    out = []
    for u in ("no", "yes"):
        a, e, c = _run_cull(cacg_lib, cfg, m, "yes", 10, tune=(f"union {u}",))
        out.append(a)
    f0, f1 = out[0]["f"], out[1]["f"]
    scale = np.abs(f0).max()
    assert np.abs(f0 - f1).max() <= 1e-5 * scale
    assert np.abs(out[0]["x"] - out[1]["x"]).max() <= 1e-8


def test_ip_group_sizes_agree(cacg_lib):
    """The integration-point passes split each row's entries over 4, 8 or 16
    lanes (`tune ip_group`); the lane sums meet in a fixed order, so the nodal
    forces of the three widths agree to FP32 rounding."""
    cfg, z = C.load_golden("eam_cac")
    m = C.model_from_arrays(z)
    nodef = []
    for gsz in (4, 8, 16):
        a, e, c = _run_cull(cacg_lib, cfg, m, "yes", 0, tune=(f"ip_group {gsz}",))
        nodef.append(e["nodef"])
    scale = np.abs(nodef[0]).max()
    for other in nodef[1:]:
        assert np.abs(nodef[0] - other).max() <= 1e-5 * scale
