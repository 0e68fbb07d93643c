"""Edge cases of the path: a system of elements only, an empty system, a
neighbor list that overflows its per-atom capacity, and bad arguments."""
import numpy as np
import pytest

import cases as C


def _elements_only():
    from cac_code_gb300 import surrogate as S
    m = S.element_box(4, 4, 1, 1)  # 2 x 1 x 1 x 4 = 8 elements, periodic, no atoms
    rng = np.random.default_rng(3)
    m.nodex = m.nodex + rng.normal(0.0, 0.03, m.nodex.shape)
    m.nodev = rng.normal(0.0, 1.0, m.nodev.shape)
    return m, dict(S.BOX_CFG)


def test_oracle_runs_elements_only(oracle_lib):
    from cac_code_gb300 import workloads as W
    m, cfg = _elements_only()
    o = oracle_lib.Oracle(m, **W.oracle_kwargs(cfg, C.EAM_FILE))
    o.setup()
    o.elem_lists()
    o.elem_forces()
    o.run(4)
    assert np.isfinite(o.elements()["nodef"]).all()


@pytest.mark.gpu
def test_elements_only_matches_oracle(oracle_lib, cacg_lib):
    from cac_code_gb300 import workloads as W
    m, cfg = _elements_only()
    o = oracle_lib.Oracle(m, **W.oracle_kwargs(cfg, C.EAM_FILE))
    o.setup()
    o.elem_lists()
    o.elem_forces()
    o.run(4)
    s = cacg_lib.System(0)
    try:
        W.configure_system(s, m, cfg, C.EAM_FILE)
        s.set_precision(cacg_lib.FP64_EXACT)
        s.init()
        s.setup()
        s.neighbor_ebuild()
        s.neighbor_nbuild()
        s.pair_ecompute()
        s.run(4)
        e, oe = s.elements(), o.elements()
        for k in ("nodex", "nodev", "nodef"):
            assert np.array_equal(e[k], oe[k]), k
        assert s.counts()["nlocal"] == 0
    finally:
        s.close()


@pytest.mark.gpu
def test_empty_system_runs(cacg_lib):
    s = cacg_lib.System(0)
    try:
        s.command("units lj")
        s.command("boundary p p p")
        s.set_box([0, 0, 0], [10, 10, 10], (True, True, True))
        s.set_masses([1.0])
        s.set_atoms(np.zeros((0, 3)), np.zeros((0, 3)), np.zeros(0, dtype=np.int32))
        s.command("pair_style lj/cut 2.5")
        s.command("pair_coeff 1 1 1.0 1.0")
        s.command("neighbor 0.3 bin")
        s.command("fix 1 all nve")
        s.init()
        s.setup()
        s.run(3)
        c = s.counts()
        assert c["nlocal"] == 0 and c["enlocal"] == 0 and c["step"] == 3
        assert s.thermo()["etotal"] == 0.0
    finally:
        s.close()


@pytest.mark.gpu
def test_neighbor_overflow_is_reported(cacg_lib):
    from gpu_runner import configure
    cfg, z = C.load_golden("lj_atoms")
    m = C.model_from_arrays(z)
    s = cacg_lib.System(0)
    try:
        configure(s, cfg, m)
        s.command("neigh_modify one 8")
        s.init()
        s.setup()
        with pytest.raises(cacg_lib.CacgError) as e:
            s.neighbor_build()
        assert e.value.status == -4
    finally:
        s.close()


@pytest.mark.gpu
def test_bad_arguments_are_refused(cacg_lib):
    s = cacg_lib.System(0)
    try:
        for bad in ("pair_style nosuch", "units furlongs", "boundary p q p", "fix 1 all nvt"):
            with pytest.raises(cacg_lib.CacgError):
                s.command(bad)
        with pytest.raises(cacg_lib.CacgError):
            s.run(1)  # no box, no pair style
    finally:
        s.close()
