"""Steps without a rebuild decision replay a captured CUDA graph: the
trajectory is bit-identical to the eager one, in every precision mode."""
import numpy as np
import pytest

import cases as C


def _run(cacg, cfg, m, mode, graphs, steps):
    from gpu_runner import configure
    s = cacg.System(0)
    try:
        configure(s, cfg, m)
        s.set_precision(mode)
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
        a, e = s.atoms(), s.elements()
        return a, e, s.counts()
    finally:
        s.close()


@pytest.mark.gpu
@pytest.mark.parametrize("mode", ["FP64_EXACT", "FP64", "MIXED"])
def test_graph_replay_is_bit_identical(cacg_lib, mode):
    cfg, z = C.load_golden("eam_cac")
    cfg = dict(cfg, every=10, check=True)
    m = C.model_from_arrays(z)
    code = getattr(cacg_lib, mode)
    a0, e0, c0 = _run(cacg_lib, cfg, m, code, False, 40)
    a1, e1, c1 = _run(cacg_lib, cfg, m, code, True, 40)
    assert c0["graph_steps"] == 0 and c1["graph_steps"] >= 30
    for k in ("x", "v", "f"):
        assert np.array_equal(a0[k], a1[k]), k
    for k in ("nodex", "nodev", "nodef"):
        assert np.array_equal(e0[k], e1[k]), k
    assert c0["rebuilds"] == c1["rebuilds"]
