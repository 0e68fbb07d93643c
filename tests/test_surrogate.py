"""The nodal-force surrogate in the step: its training samples against the
oracle, what the trained ensemble gains over simpler predictors, and the
fallback to the plain quadrature."""
import os
import tempfile

import numpy as np
import pytest

import cases as C


def _eam_file():
    from cac_code_gb300 import workloads as W
    d = os.path.join(tempfile.gettempdir(), "cacg_sur_eam")
    os.makedirs(d, exist_ok=True)
    return W.write_eam(os.path.join(d, "Cu2000.eam"))


@pytest.mark.gpu
def test_samples_match_oracle(oracle_lib, cacg_lib):
    from gpu_runner import configure
    cfg, z = C.load_golden("eam_cac")
    m = C.model_from_arrays(z)
    x0 = m.nodex.copy()
    o = oracle_lib.Oracle(m, **C.settings_kwargs(cfg))
    o.setup()
    o.atom_list()
    o.elem_lists()
    nodef = o.elem_forces()
    n = o.size(0) + o.size(1)
    rho, fp = np.zeros(n), np.zeros(n)
    erho = np.zeros(8 * (o.size(3) + o.size(4)))
    o._L.orc_get_eam_scratch(o.h, oracle_lib._d(rho), oracle_lib._d(fp), oracle_lib._d(erho))
    s = cacg_lib.System(0)
    try:
        configure(s, cfg, m)
        s.set_precision(cacg_lib.FP64_EXACT)
        s.init()
        s.setup()
        s.neighbor_build()
        s.neighbor_ebuild()
        s.neighbor_nbuild()
        s.surrogate_reference(x0)
        x, t = s.surrogate_samples()
    finally:
        s.close()
    ne = m.nelements
    assert np.array_equal(t, nodef.reshape(ne, 24).astype(np.float32))
    u = m.nodex - x0
    u = u - u.mean(axis=1, keepdims=True)
    assert np.abs(x[:, :24] - u.reshape(ne, 24)).max() <= 1e-6 * max(1.0, np.abs(u).max())
    assert np.array_equal(x[:, 24:], erho[:8 * ne].reshape(ne, 8).astype(np.float32))


@pytest.mark.gpu
def test_trained_ensemble_beats_simpler_predictors(cacg_lib):
    from cac_code_gb300 import surrogate as S
    eam = _eam_file()
    # many strain states matter more than many thermal snapshots per state
    x, t, info = S.generate(eam, 65536, seed=1, planes=8, ny=8, nz=8, snapshots=4)
    xv, tv, _ = S.generate(eam, 8192, seed=2, planes=8, ny=8, nz=8, snapshots=4)
    assert info["samples"] == 65536 and np.isfinite(t).all()
    net, loss = S.train(x, t, members=4, epochs=8, batch=1024, lr=2e-3)
    try:
        mean, spread = net.predict(xv)
        e_net = S.force_errors(mean, tv)["rms_rel"]
        e_zero = S.force_errors(np.zeros_like(tv), tv)["rms_rel"]
        a = np.hstack([x, np.ones((x.shape[0], 1))]).astype(np.float64)
        coef, *_ = np.linalg.lstsq(a, t.astype(np.float64), rcond=None)
        lin = np.hstack([xv, np.ones((xv.shape[0], 1))]) @ coef
        e_lin = S.force_errors(lin, tv)["rms_rel"]
        assert e_net < 0.05 * e_zero, (e_net, e_zero)
        assert e_net < 0.75 * e_lin, (e_net, e_lin)
        assert np.all(spread >= 0) and np.median(spread) > 0
    finally:
        net.close()


@pytest.mark.gpu
def test_fallback_and_acceptance_in_the_step(cacg_lib):
    from cac_code_gb300 import surrogate as S
    from cac_code_gb300 import workloads as W
    eam = _eam_file()
    x, t, _ = S.generate(eam, 16384, seed=3, planes=8, ny=8, nz=8, snapshots=4)
    net, _ = S.train(x, t, members=4, epochs=2, batch=1024, lr=2e-3)
    m, cfg = W.c2_sample()
    s = cacg_lib.System(0)
    try:
        W.configure_system(s, m, cfg, eam)
        s.set_precision(cacg_lib.FP64)
        s.init()
        with pytest.raises(cacg_lib.CacgError):
            s.setup()
            s.neighbor_build()
            s.neighbor_ebuild()
            s.neighbor_nbuild()
            s.surrogate_attach(net, tol=1.0, dist=11.0)  # FP64 modes: refused
        s.set_precision(cacg_lib.MIXED)
        s.surrogate_reference(m.nodex)
        s.pair_ecompute()
        plain = s.elements()["nodef"].copy()
        feats, _ = s.surrogate_samples()
        # tolerance 0: every far element falls back, forces bit-identical
        s.surrogate_attach(net, tol=0.0, dist=11.0)
        s.pair_ecompute()
        c = s.counts()
        assert c["surrogate_elements"] > 0 and c["surrogate_accepted"] == 0
        assert np.array_equal(s.elements()["nodef"], plain)
        # tolerance inf: every far element takes the ensemble mean
        s.surrogate_attach(net, tol=1e30, dist=11.0)
        s.pair_ecompute()
        c = s.counts()
        nf = s.elements()["nodef"]
        assert c["surrogate_accepted"] == c["surrogate_elements"]
        pred, _ = net.predict(feats)
        changed = np.any(nf != plain, axis=(1, 2))
        assert changed.sum() == c["surrogate_elements"]
        np.testing.assert_allclose(nf[changed].reshape(-1, 24), pred[changed], rtol=0,
                                   atol=2e-2 * np.abs(pred).max())
        assert np.array_equal(nf[~changed], plain[~changed])
        # the step runs with it and stays finite
        s.run(5)
        assert np.isfinite(s.elements()["nodef"]).all()
        s.surrogate_attach(None)
        assert s.counts()["surrogate_elements"] == 0
    finally:
        s.close()
        net.close()


@pytest.mark.gpu
def test_rejected_elements_back_off(cacg_lib):
    """An element the ensemble rejects is re-tested after 1, 3, 7, 15, 31, 63,
    then 127 steps: with every far element rejected (tolerance 0), 64 steps
    test each 6 times (steps 0, 2, 6, 14, 30, 62), and the trajectory equals
    the one without the surrogate bit for bit (rejected elements take the
    quadrature)."""
    from cac_code_gb300 import surrogate as S
    from cac_code_gb300 import workloads as W
    eam = _eam_file()
    x, t, _ = S.generate(eam, 8192, seed=4, planes=8, ny=8, nz=8, snapshots=4)
    net, _ = S.train(x, t, members=2, epochs=1, batch=1024, lr=2e-3)
    m, cfg = W.c2_sample(seed=5)
    out = []
    try:
        for attach in (True, False):
            s = cacg_lib.System(0)
            try:
                W.configure_system(s, m, cfg, eam)
                s.set_precision(cacg_lib.MIXED)
                s.init()
                s.setup()
                s.neighbor_build()
                s.neighbor_ebuild()
                s.neighbor_nbuild()
                if attach:
                    s.surrogate_reference(m.nodex)
                    s.surrogate_attach(net, tol=0.0, dist=11.0)
                c0 = s.counts()
                s.run(64)
                c1 = s.counts()
                out.append((s.elements()["nodex"], c1["surrogate_evaluated"] - c0["surrogate_evaluated"],
                            c1["surrogate_elements"], c1["surrogate_accepted"]))
            finally:
                s.close()
    finally:
        net.close()
    (nx_s, ev, far, acc), (nx_p, _, _, _) = out
    assert far > 0 and acc == 0
    assert ev == 6 * far, (ev, far)
    assert np.array_equal(nx_s.view(np.int64), nx_p.view(np.int64))
