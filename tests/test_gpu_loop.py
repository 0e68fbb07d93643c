"""The device step loop ("tune loop device"): one CUDA graph launch runs steps
back to back with Neighbor::decide (neighbor.cpp:1150-1163) taken on the
device, and hands a step that needs a rebuild to the host; after set-up and
after each rebuild one step runs eagerly before the loop is captured again.
The trajectory is bit-identical to the host loop's (eager decision steps), in
every precision mode, with and without the distance check, with post-force
fixes, and the rebuilds happen at the same steps."""
import numpy as np
import pytest

import cases as C
from cac_code_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _run(cacg, cfg, m, mode, loop, steps, chunks=1, workload=False):
    from gpu_runner import configure
    s = cacg.System(0)
    try:
        if workload:
            W.configure_system(s, m, cfg)
        else:
            configure(s, cfg, m)
        s.set_precision(mode)
        s.command(f"tune loop {loop}")
        s.init()
        s.setup()
        s.neighbor_build()
        s.pair_compute()
        if m.nelements:
            s.neighbor_ebuild()
            s.neighbor_nbuild()
            s.pair_ecompute()
        for _ in range(chunks):
            s.run(steps // chunks)
        a, e = s.atoms(), s.elements()
        return a, e, s.counts()
    finally:
        s.close()


def _same(r0, r1):
    (a0, e0, c0), (a1, e1, c1) = r0, r1
    for k in ("x", "v", "f"):
        assert np.array_equal(a0[k], a1[k]), k
    for k in ("nodex", "nodev", "nodef"):
        assert np.array_equal(e0[k], e1[k]), k
    assert c0["rebuilds"] == c1["rebuilds"]
    assert c0["step"] == c1["step"]


@pytest.mark.parametrize("mode", ["FP64_EXACT", "FP64", "MIXED"])
@pytest.mark.parametrize("check", [True, False])
def test_device_loop_is_bit_identical(cacg_lib, mode, check):
    cfg, z = C.load_golden("eam_cac")
    cfg = dict(cfg, every=5, check=check)
    m = C.model_from_arrays(z)
    code = getattr(cacg_lib, mode)
    host = _run(cacg_lib, cfg, m, code, "host", 60)
    dev = _run(cacg_lib, cfg, m, code, "device", 60)
    _same(host, dev)
    c0, c1 = host[2], dev[2]
    assert c0["loop_launches"] == 0 and c0["host_decisions"] == 12
    assert c1["host_decisions"] == 0
    # every step but the rebuild steps and the eager step after set-up and
    # after each rebuild ran inside the loop; a launch ends at each rebuild
    r = c1["rebuilds"]
    assert 60 - 2 * r - 1 <= c1["graph_steps"] <= 60 - r
    assert r <= c1["loop_launches"] <= r + 1
    if not check:  # rebuilds at steps 5, 10, ..., 60; stretches 2-4, 7-9, ...
        assert r == 12 and c1["loop_launches"] == 12 and c1["graph_steps"] == 36


def test_device_loop_with_fixes(cacg_lib):
    cfg, z = C.load_golden("lj_cac_fixes")
    cfg = dict(cfg, every=4, check=True)
    m = C.model_from_arrays(z)
    host = _run(cacg_lib, cfg, m, cacg_lib.MIXED, "host", 40)
    dev = _run(cacg_lib, cfg, m, cacg_lib.MIXED, "device", 40, chunks=4)
    _same(host, dev)
    assert dev[2]["host_decisions"] == 0


def test_device_loop_c1_full(cacg_lib):
    """C1 in full (16,384 atoms + 64 elements), FP64 bit for bit, a rebuild
    every 10 steps without the check: 5 rebuilds in 50 steps, each handed
    to the host by its own loop launch (the last at the last step); steps 1,
    11, ..., 41 run eagerly."""
    m, cfg = W.c1_lj()
    cfg = dict(cfg, every=10, check=False)
    host = _run(cacg_lib, cfg, m, cacg_lib.FP64_EXACT, "host", 50, workload=True)
    dev = _run(cacg_lib, cfg, m, cacg_lib.FP64_EXACT, "device", 50, workload=True)
    _same(host, dev)
    assert dev[2]["rebuilds"] == host[2]["rebuilds"] == 5
    assert dev[2]["loop_launches"] == 5
    assert dev[2]["graph_steps"] == 40


def test_batch_graph_equals_separate_runs(cacg_lib):
    """cacg_run_batch: several handles' step loops as branches of one CUDA
    graph give the same trajectories, bit for bit, as each handle's own run,
    across rebuilds (handed to the host) and with post-force fixes."""
    from gpu_runner import configure
    names = ["eam_cac", "lj_cac_fixes", "lj_cac"]
    cases = []
    for nm in names:
        cfg, z = C.load_golden(nm)
        cases.append((dict(cfg, every=3, check=True), C.model_from_arrays(z)))

    def make():
        out = []
        for cfg, m in cases:
            s = cacg_lib.System(0)
            configure(s, cfg, m)
            s.set_precision(cacg_lib.MIXED)
            s.command("tune loop device")
            s.init()
            s.setup()
            s.neighbor_build()
            s.pair_compute()
            if m.nelements:
                s.neighbor_ebuild()
                s.neighbor_nbuild()
                s.pair_ecompute()
            out.append(s)
        return out

    alone, batch = make(), make()
    try:
        for s in alone:
            s.run(45)
        cacg_lib.run_batch(batch, 45)
        for a, b in zip(alone, batch):
            ca, cb = a.counts(), b.counts()
            assert ca["step"] == cb["step"] and ca["rebuilds"] == cb["rebuilds"]
            assert cb["host_decisions"] == 0
            for k in ("x", "v", "f"):
                assert np.array_equal(a.atoms()[k], b.atoms()[k]), k
            for k in ("nodex", "nodev", "nodef"):
                assert np.array_equal(a.elements()[k], b.elements()[k]), k
    finally:
        for s in alone + batch:
            s.close()
