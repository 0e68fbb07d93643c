"""Training samples, training and evaluation of the nodal-force surrogate.

The surrogate (``cacg.Mlp``: an ensemble of MLPs 32 -> 256 -> 256 -> 256 -> 24,
SiLU, tensor-core BF16 with FP32 accumulation) predicts an element's 24 nodal
forces from its 24 nodal displacements about their mean, relative to the ideal
lattice, and its 8 nodal densities.  The reference has no counterpart.

Samples come from the plain method itself: a fully periodic box of elements
(no atoms, so no element is near an interface) is strained affinely along
x, y and z (each normal strain uniform in [-3 %, +3 %]; the box stays
orthogonal, as the reference's domain is), its nodes are displaced by
Gaussian thermal noise of a temperature drawn uniformly in [0, 500] K, and the
FP64 quadrature gives the nodal forces (``System.surrogate_samples``).  Many
noise snapshots share one strained box and its neighbor lists: the noise stays
far below half the skin, so the lists stay valid.
"""
from __future__ import annotations

import math
from typing import Dict, Optional, Tuple

import numpy as np

from . import cacg
from . import lattice as L
from . import workloads as W

# rms thermal displacement of a node at 300 K (Cu, harmonic estimate)
SIGMA_300K = 0.1


def element_box(nae: int, planes: int, ny: int, nz: int, a: float = W.A_CU,
                mass: float = L.AnalyticEAM().mass) -> L.Model:
    """A periodic box filled with elements only: ``planes`` (even) element planes
    along x, ``ny`` x ``nz`` element periods in y and z; 2*ny*nz*planes elements
    with the C2 element type (8 near-Gauss points plus the 8 nodes)."""
    if planes % 2:
        raise ValueError("planes must be even for an x-periodic element superlattice")
    per = nae * a
    ly, lz = ny * per, nz * per
    origins = L.tile_elements(nae, a, 0.0, planes, +1, ly, lz)
    nodex = L.elements_nodes(origins, nae, a).reshape(-1, 8, 3)
    ip, w = L.gauss_intp(nae, True)
    m = L.Model(boxlo=np.zeros(3), boxhi=np.array([planes // 2 * per, ly, lz]),
                periodic=(True, True, True), mass=mass, atom_x=np.zeros((0, 3)),
                atom_v=np.zeros((0, 3)), etypes=[L.ElementType((nae, nae, nae), ip, w)],
                elem_type=np.ones(nodex.shape[0], dtype=np.int64), nodex=nodex,
                nodev=np.zeros_like(nodex), lattice_a=a)
    L.remap_into_box(m)
    return m


def _strained(m: L.Model, eps: np.ndarray) -> L.Model:
    s = L.Model(**{k: getattr(m, k) for k in m.__dataclass_fields__})
    f = 1.0 + eps
    s.boxhi = m.boxlo + (m.boxhi - m.boxlo) * f
    s.nodex = m.boxlo + (m.nodex - m.boxlo) * f
    s.nodev = np.zeros_like(m.nodex)
    return s


BOX_CFG = dict(units="metal", boundary="p p p", pair="eam", skin=7.5, every=10, delay=0,
               check=True, dt=0.001)


def generate(eam_file: str, n_samples: int, seed: int = 1, nae: int = 11, planes: int = 8,
             ny: int = 8, nz: int = 8, snapshots: int = 16, strain: float = 0.03,
             t_max: float = 500.0, device: int = 0) -> Tuple[np.ndarray, np.ndarray, Dict]:
    """At least ``n_samples`` (features, nodal forces) pairs from the plain FP64
    quadrature under random normal strains and thermal noise."""
    rng = np.random.default_rng(seed)
    base = element_box(nae, planes, ny, nz)
    xs, ts, got, configs = [], [], 0, 0
    while got < n_samples:
        eps = rng.uniform(-strain, strain, size=3)
        m = _strained(base, eps)
        s = cacg.System(device)
        try:
            W.configure_system(s, m, BOX_CFG, eam_file)
            s.set_precision(cacg.FP64)
            s.init()
            s.setup()
            s.neighbor_ebuild()
            s.neighbor_nbuild()
            s.surrogate_reference(base.nodex)
            zeros = np.zeros_like(m.nodex)
            for _ in range(snapshots):
                temp = rng.uniform(0.0, t_max)
                sig = SIGMA_300K * math.sqrt(temp / 300.0)
                s.put_nodes(m.nodex + rng.normal(scale=sig, size=m.nodex.shape), zeros)
                x, t = s.surrogate_samples()
                xs.append(x)
                ts.append(t)
                got += x.shape[0]
                if got >= n_samples:
                    break
        finally:
            s.close()
        configs += 1
    x = np.concatenate(xs)[:n_samples]
    t = np.concatenate(ts)[:n_samples]
    info = {"samples": int(x.shape[0]), "strain_configs": configs,
            "elements_per_config": int(base.nelements), "snapshots_per_config": snapshots,
            "strain": strain, "t_max_K": t_max, "nae": nae}
    return x, t, info


def train(x: np.ndarray, t: np.ndarray, members: int = 4, epochs: int = 20, batch: int = 2048,
          lr: float = 2e-3, seed: int = 5, device: int = 0) -> Tuple[cacg.Mlp, float]:
    net = cacg.Mlp(device, members=members, seed=seed)
    net.fit_normalization(x, t)
    loss = net.train(x, t, epochs=epochs, batch=batch, lr=lr, seed=seed + 1)
    return net, loss


def force_errors(pred: np.ndarray, ref: np.ndarray) -> Dict[str, float]:
    """Relative nodal-force errors: rms over nodes of |df| / rms |f|, and the
    largest |df| / largest |f|."""
    d = np.linalg.norm((pred - ref).reshape(-1, 3), axis=1)
    n = np.linalg.norm(ref.reshape(-1, 3), axis=1)
    return {"rms_rel": float(np.sqrt((d ** 2).mean() / max((n ** 2).mean(), 1e-300))),
            "max_rel": float(d.max() / max(n.max(), 1e-300))}
