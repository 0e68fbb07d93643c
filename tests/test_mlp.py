"""The surrogate MLP: its CPU restatement pinned by finite differences, then
the tensor-core GEMM, the device loss/gradient and prediction against it, and
training."""
import numpy as np
import pytest

from oracle import mlp_oracle as MO


def _data(n, seed):
    # one fixed target function; the seed draws the inputs
    w = np.random.default_rng(0).normal(size=(MO.NIN, MO.NOUT)) / np.sqrt(MO.NIN)
    rng = np.random.default_rng(seed)
    x = rng.normal(size=(n, MO.NIN)).astype(np.float32)
    t = (np.tanh(x @ w) + 0.1 * np.sin(3 * x[:, :MO.NOUT])).astype(np.float32)
    return x, t


def _params(seed, scale=1.0):
    rng = np.random.default_rng(seed)
    d = {}
    for name, shp in MO.SHAPES:
        fan = shp[1] if len(shp) == 2 else 1
        d[name] = (rng.uniform(-1, 1, size=shp) * scale * np.sqrt(3.0 / fan)).astype(np.float32)
        if name.startswith("b"):
            d[name] *= 0.1
    return MO.pack(d).astype(np.float32)


def test_oracle_backward_matches_finite_differences():
    x, t = _data(16, 1)
    p = _params(2).astype(np.float64)
    _, g = MO.loss_grad(p, x.astype(np.float64), t.astype(np.float64), exact=True)
    rng = np.random.default_rng(3)
    offs = np.cumsum([0] + [int(np.prod(s)) for _, s in MO.SHAPES])
    for b in range(len(MO.SHAPES)):
        for i in rng.integers(offs[b], offs[b + 1], size=4):
            h = 1e-6
            pp, pm = p.copy(), p.copy()
            pp[i] += h
            pm[i] -= h
            lp, _ = MO.loss_grad(pp, x, t, exact=True)
            lm, _ = MO.loss_grad(pm, x, t, exact=True)
            fd = (lp - lm) / (2 * h)
            assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(g[i])) + 1e-9, (MO.SHAPES[b][0], i, fd, g[i])


def test_bf16_rounding_is_nearest_even():
    v = np.array([1.0, 1.00390625, 1.005859375, 3.0e-41, -2.5], dtype=np.float32)
    r = MO.bf16(v)
    assert r[0] == 1.0 and r[1] == 1.0  # tie -> even
    assert r[2] == np.float32(1.0078125)
    assert r[4] == -2.5


@pytest.mark.gpu
@pytest.mark.parametrize("m,n,k", [(128, 256, 64), (300, 24, 256), (1000, 1024, 64),
                                   (257, 64, 4096), (4096, 256, 256), (24, 256, 1024)])
def test_gemm_bf16_matches_numpy(cacg_lib, m, n, k):
    import ctypes
    import torch
    L = cacg_lib.load()
    dev = torch.device("cuda", 0)
    g = torch.Generator().manual_seed(m * 7 + n + k)
    a = torch.randn(m, k, generator=g).to(torch.bfloat16)
    b = torch.randn(n, k, generator=g).to(torch.bfloat16)
    ref = a.float().double() @ b.float().double().T
    da, db = a.to(dev), b.to(dev)
    dc = torch.full((m, n), float("nan"), dtype=torch.float32, device=dev)
    err = torch.zeros(1, dtype=torch.int32, device=dev)
    st = ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
    rc = L.cacg_gemm_bf16_tn(ctypes.c_void_p(da.data_ptr()), k, ctypes.c_void_p(db.data_ptr()), k,
                             ctypes.c_void_p(dc.data_ptr()), n, m, n, k,
                             ctypes.c_void_p(err.data_ptr()), st)
    assert rc == 0
    torch.cuda.synchronize(dev)
    assert int(err.item()) == 0
    c = dc.cpu().double()
    rel = (c - ref).abs().max().item() / ref.abs().max().item()
    assert rel < 1e-5, rel


@pytest.mark.gpu
def test_device_loss_grad_matches_oracle(cacg_lib):
    x, t = _data(500, 4)
    net = cacg_lib.Mlp(0, members=2, seed=11)
    try:
        net.fit_normalization(x, t)
        im, isd, om, osd, _ = net.normalization()
        xn, tn = MO.normalize(x, t, (im, isd, om, osd))
        for k in range(2):
            p = net.params(k)
            loss, g = net.loss_grad(k, x, t)
            l_ref, g_ref = MO.loss_grad(p.astype(np.float64), xn, tn)
            assert abs(loss - l_ref) <= 1e-3 * l_ref, (loss, l_ref)
            offs = np.cumsum([0] + [int(np.prod(s)) for _, s in MO.SHAPES])
            for b, (name, _) in enumerate(MO.SHAPES):
                gd, gr = g[offs[b]:offs[b + 1]], g_ref[offs[b]:offs[b + 1]]
                rel = np.linalg.norm(gd - gr) / max(np.linalg.norm(gr), 1e-30)
                assert rel < 2e-2, (k, name, rel)
    finally:
        net.close()


def _oracle_ensemble(net, x, norm):
    ys = []
    for k in range(net.members):
        xn, _ = MO.normalize(x, None, norm)
        y, _ = MO.forward(net.params(k).astype(np.float64), xn)
        ys.append(y * norm[3] + norm[2])
    ys = np.array(ys)
    return ys.mean(axis=0), ys.std(axis=0).max(axis=1)


@pytest.mark.gpu
def test_device_prediction_and_training(cacg_lib):
    x, t = _data(32768, 5)
    xv, tv = _data(1024, 6)
    net = cacg_lib.Mlp(0, members=4, seed=3)
    try:
        net.fit_normalization(x, t)
        norm = net.normalization()[:4]
        # the fused ensemble kernel against the oracle forward, untrained
        mean, spread = net.predict(xv)
        m_ref, s_ref = _oracle_ensemble(net, xv, norm)
        assert np.abs(mean - m_ref).max() <= 2e-2 * np.abs(m_ref).max()
        assert np.abs(spread - s_ref).max() <= 5e-2 * s_ref.max() + 1e-6
        before = float(((mean - tv) ** 2).mean())
        loss = net.train(x, t, epochs=10, batch=1024, lr=2e-3)
        mean, spread = net.predict(xv)
        # and trained
        m_ref, s_ref = _oracle_ensemble(net, xv, norm)
        assert np.abs(mean - m_ref).max() <= 2e-2 * np.abs(m_ref).max()
        after = float(((mean - tv) ** 2).mean())
        assert loss < 0.1, loss
        assert after < 0.3 * before, (before, after)
    finally:
        net.close()
