"""cacg_kinetic_noalloc (kinetic sums kept in a fixed device array) against
the handle-based cacg_compute_thermo on the same state, two calls in a row.

Collected last so that it also runs after every other test has used the
library on the same device."""
import ctypes

import numpy as np
import pytest

import cases as C

MVV2E = {"lj": 1.0, "metal": 1.0364269e-4}


@pytest.mark.gpu
def test_kinetic_noalloc_matches_thermo(cacg_lib):
    import torch
    from gpu_runner import configure
    cfg, z = C.load_golden("eam_cac")
    m = C.model_from_arrays(z)
    s = cacg_lib.System(0)
    try:
        configure(s, cfg, m)
        s.set_precision(cacg_lib.FP64)
        s.init()
        s.setup()
        s.neighbor_build()
        s.neighbor_ebuild()
        s.neighbor_nbuild()
        s.run(3)
        ref = s.thermo()
        a, e = s.atoms(), s.elements()
    finally:
        s.close()
    L = cacg_lib.load()
    dev = torch.device("cuda", 0)
    mvv2e = MVV2E[cfg["units"]]
    emass = float(np.prod(m.etypes[0].nae)) * m.mass
    items = {
        "atoms": (a["v"], np.ones(len(a["v"]), np.int32), [0.0, m.mass], 1, 1.0),
        "nodes": (e["nodev"].reshape(-1, 3), np.ones(len(e["nodev"]), np.int32),
                  [0.0, emass], 8, 1.0 / 8),
    }
    stream = ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
    bufs = {}
    for k, (v, t, mass, per, sc) in items.items():
        bufs[k] = (torch.tensor(np.ascontiguousarray(v), dtype=torch.float64, device=dev),
                   torch.tensor(t, dtype=torch.int32, device=dev),
                   torch.tensor(mass, dtype=torch.float64, device=dev), per, sc)
    results = []
    for call in range(2):
        got = {}
        for k, (v, t, mass, per, sc) in bufs.items():
            out = torch.full((7,), float("nan"), dtype=torch.float64, device=dev)
            rc = L.cacg_kinetic_noalloc(ctypes.c_void_p(v.data_ptr()), ctypes.c_void_p(t.data_ptr()),
                                        ctypes.c_void_p(mass.data_ptr()), v.shape[0], per, sc,
                                        mvv2e, ctypes.c_void_p(out.data_ptr()), stream)
            assert rc == 0, rc
            torch.cuda.synchronize(dev)
            got[k] = out.cpu().numpy()
        tol = 1e-12
        assert abs(got["atoms"][0] - ref["ke_atoms"]) <= tol * abs(ref["ke_atoms"]), (call, got, ref)
        assert abs(got["nodes"][0] - ref["ke_nodes"]) <= tol * abs(ref["ke_nodes"]), (call, got, ref)
        tens = got["atoms"][1:] + got["nodes"][1:]
        sc = np.abs(ref["kinetic_tensor"]).max()
        assert np.abs(tens - ref["kinetic_tensor"]).max() <= tol * sc, (call, tens, ref)
        results.append(got)
    for k in bufs:
        assert np.array_equal(results[0][k], results[1][k]), k
    # a request beyond the fixed scratch array is refused before any launch
    big = (8192 * 256) + 1
    v, t, mass, per, sc = bufs["atoms"]
    out = torch.zeros(7, dtype=torch.float64, device=dev)
    rc = L.cacg_kinetic_noalloc(ctypes.c_void_p(v.data_ptr()), ctypes.c_void_p(t.data_ptr()),
                                ctypes.c_void_p(mass.data_ptr()), big, 1, 1.0, 1.0,
                                ctypes.c_void_p(out.data_ptr()), stream)
    assert rc == -8
