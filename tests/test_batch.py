"""Batched replicas (cac_code_gb300.batch): the draw, the packing that keeps
replicas independent, and a short batched run with the autotuner."""
import os
import tempfile

import numpy as np
import pytest

from cac_code_gb300 import batch as B


def test_draw_is_seeded_and_in_range():
    a = B.draw_replicas(256, seed=4)
    b = B.draw_replicas(256, seed=4)
    assert [r.sites for r in a] == [r.sites for r in b]
    s = np.array([r.sites for r in a])
    assert s.min() >= 2000 and s.max() <= 60000
    assert 10000 < s.mean() < 25000  # log-uniform mean ~ 17,000
    f = np.array([r.atom_fraction for r in a])
    assert f.min() >= 0.2 and f.max() <= 0.8
    assert {r.pair for r in a} == {"lj", "eam"}


def test_packing_keeps_gaps():
    reps = [r for r in B.draw_replicas(16, seed=9) if r.pair == "eam"][:3]
    models = [B.replica_model(r, 1) for r in reps]
    big, ca, ce, spans = B.pack(models, B.STYLE["eam"]["gap"])
    assert big.natoms == sum(m.natoms for m, _, _ in models)
    assert big.nelements == sum(m.nelements for m, _, _ in models)
    for (a0, a1), (b0, b1) in zip(spans, spans[1:]):
        assert b0 - a1 >= B.STYLE["eam"]["gap"] - 1e-9
    assert ce.sum() > 0


def _forces(cacg, model, cfg, eam, cla=None, cle=None):
    from cac_code_gb300 import workloads as W
    s = cacg.System(0)
    try:
        W.configure_system(s, model, cfg, eam)
        s.set_precision(cacg.FP64)
        s.init()
        s.setup()
        s.neighbor_build()
        s.neighbor_ebuild()
        s.neighbor_nbuild()
        s.pair_compute()
        s.pair_ecompute()
        return s.atoms()["f"], s.elements()["nodef"]
    finally:
        s.close()


@pytest.mark.gpu
def test_replicas_in_a_batch_do_not_interact(cacg_lib):
    from cac_code_gb300 import workloads as W
    eam = W.write_eam(os.path.join(tempfile.gettempdir(), "cacg_batch_Cu2000.eam"))
    reps = [r for r in B.draw_replicas(20, seed=5) if r.pair == "eam"][:3]
    for r in reps:
        r.sites = 2500
    models = [B.replica_model(r, 1) for r in reps]
    big, _, _, _ = B.pack(models, B.STYLE["eam"]["gap"])
    cfg = B.class_config("eam")
    fa, fn = _forces(cacg_lib, big, cfg, eam)
    import dataclasses
    oa = on = 0
    for m, _, _ in models:
        # the replica alone, at its coordinates in the batch and in the same box
        alone = dataclasses.replace(
            big, atom_x=big.atom_x[oa:oa + m.natoms], atom_v=big.atom_v[oa:oa + m.natoms],
            nodex=big.nodex[on:on + m.nelements], nodev=big.nodev[on:on + m.nelements],
            elem_type=big.elem_type[on:on + m.nelements])
        a, n = _forces(cacg_lib, alone, cfg, eam)
        sc = max(np.abs(a).max(), np.abs(n).max())
        assert np.abs(fa[oa:oa + m.natoms] - a).max() <= 1e-12 * sc
        assert np.abs(fn[on:on + m.nelements] - n).max() <= 1e-12 * sc
        oa += m.natoms
        on += m.nelements


@pytest.mark.gpu
def test_small_batched_run_with_autotuner(cacg_lib):
    from cac_code_gb300 import workloads as W
    eam = W.write_eam(os.path.join(tempfile.gettempdir(), "cacg_batch_Cu2000.eam"))
    res = B.run_batch(eam, n=6, steps=30, seed=7, tune=True)
    assert res["replicas"] == 6 and len(res["classes"]) >= 2 and res["schedule"] == "graph"
    assert np.isfinite(res["site_steps_per_s"]) and res["site_steps_per_s"] > 0
    for c in res["classes"]:
        # every step but the rebuilds and the eager step after each ran inside
        # a device-loop graph launch, and no rebuild decision was taken on the host
        assert c["graph_steps"] >= 30 - 2 * c["rebuilds"] - 1
        assert c["host_decisions"] == 0 and 1 <= c["loop_launches"] <= c["rebuilds"] + 1
        assert c["autotune"]["chosen"]["block"] in (128, 256, 512)
        assert len(c["autotune"]["trials"]) >= 8


@pytest.mark.gpu
def test_schedules_agree(cacg_lib):
    """One graph for all classes, one host thread per class, and one class
    after another give the same per-class rebuilds and steps."""
    from cac_code_gb300 import workloads as W
    eam = W.write_eam(os.path.join(tempfile.gettempdir(), "cacg_batch_Cu2000.eam"))
    runs = [B.run_batch(eam, n=6, steps=40, seed=7, tune=False, schedule=sch)
            for sch in ("graph", "threads", "sequential")]
    for cs in zip(*(r["classes"] for r in runs)):
        assert len({(c["pair"], c["sites"], c["rebuilds"]) for c in cs}) == 1
