"""Batched independent CAC replicas on one GPU.

Replicas of uneven size (sites drawn log-uniform in [2k, 60k], atom fraction
uniform in [0.2, 0.8]), temperature (uniform in [10, 600] K; in LJ units
T* = kB T / 0.4 eV) and applied shear (uniform in [0, 4 %], an affine displacement held by
clamped boundary slabs under fix setforce) are grouped by pair style and size
class.  The replicas of a class share one handle: they sit side by side along
the non-periodic x axis, each a slab with the class's periodic y-z cross
section, separated by gaps wider than the element neighbor cutoff, so that no
list ever crosses from one replica into another.  Every kernel of a step then
covers all replicas of the class at once, and steps without a rebuild
decision replay one captured CUDA graph.

Per class an autotuner times the candidate bin sizes (the reference's default
r_n / 2 and r_n) and thread-block sizes of the persistent mixed-precision
kernels (256, 512) on a few steps and keeps the fastest.

The reference runs one system per process; it has no batching.
"""
from __future__ import annotations

import dataclasses
import math
import time
from typing import Dict, List, Tuple

import numpy as np

from . import cacg
from . import lattice as L
from . import workloads as W

A_LJ = (4.0 / 1.0) ** (1.0 / 3.0)  # FCC at rho* = 1.0

# per pair style: lattice, element size (sites per edge), cross sections (in
# element periods) of the size classes, gap between replicas, reference commands
STYLE = {
    "eam": dict(a=W.A_CU, nae=10, units="metal", skin=7.5, gap=70.0, kb=W.KB["metal"],
                mvv2e=W.MVV2E["metal"], t_scale=1.0, dt=0.001),
    # LJ temperatures: T* = kB T / eps with eps = 0.4 eV (a Cu-like well), so
    # 10-600 K maps to T* = 0.002-0.13, below the LJ melting point
    "lj": dict(a=A_LJ, nae=8, units="lj", skin=2.8, gap=20.0, kb=1.0, mvv2e=1.0,
               t_scale=8.617343e-5 / 0.4, dt=0.005),
}
SIZE_CLASSES = [(2000, 8000, 1), (8000, 20000, 2), (20000, 60001, 3)]  # sites lo, hi, periods


@dataclasses.dataclass
class Replica:
    index: int
    pair: str
    sites: int
    atom_fraction: float
    temperature: float  # K (EAM) or the LJ equivalent temperature x t_scale
    shear: float
    seed: int


def draw_replicas(n: int = 256, seed: int = 4) -> List[Replica]:
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        out.append(Replica(i, "lj" if i % 2 else "eam",
                           int(round(math.exp(rng.uniform(math.log(2000), math.log(60000))))),
                           float(rng.uniform(0.2, 0.8)), float(rng.uniform(10.0, 600.0)),
                           float(rng.uniform(0.0, 0.04)), int(rng.integers(1 << 30))))
    return out


def size_class(sites: int) -> int:
    for k, (lo, hi, _) in enumerate(SIZE_CLASSES):
        if lo <= sites < hi:
            return k
    return len(SIZE_CLASSES) - 1


def replica_model(r: Replica, periods: int) -> Tuple[L.Model, np.ndarray, np.ndarray]:
    """The replica's slab and its clamp flags (outermost element plane per side)."""
    st = STYLE[r.pair]
    a, nae = st["a"], st["nae"]
    c = nae * periods  # cells across y and z: whole element periods
    per_cell = 4 * c * c
    ip_per_layer = 2 * (2 * periods * periods) * 8  # both sides, 2 p^2 elements per plane
    ax = max(2, int(round(r.atom_fraction * r.sites / per_cell)))
    layers = max(2, int(round((1 - r.atom_fraction) * r.sites / ip_per_layer)))
    mass = L.AnalyticEAM().mass if r.pair == "eam" else 1.0
    m = L.make_slab_model(a, mass, (ax, c, c), nae, layers, L.gauss_intp(nae, r.pair == "eam"))
    L.thermalize(m, r.temperature * st["t_scale"], st["kb"], st["mvv2e"], r.seed)
    # simple shear u_y = g (x - x_mid), held by the clamped outer planes
    xs = np.concatenate([m.atom_x[:, 0], m.nodex[:, :, 0].ravel()])
    xmid = 0.5 * (xs.min() + xs.max())
    m.atom_x[:, 1] += r.shear * (m.atom_x[:, 0] - xmid)
    m.nodex[:, :, 1] += r.shear * (m.nodex[:, :, 0] - xmid)
    cen = m.element_centres()[:, 0]
    half = 0.5 * nae * a
    clamp_e = (cen <= cen.min() + 0.25 * half) | (cen >= cen.max() - 0.25 * half)
    m.nodev[clamp_e] = 0.0
    clamp_a = np.zeros(m.natoms, dtype=np.int32)
    L.remap_into_box(m)  # the shear moved sites across the periodic y faces
    L.wrap_elements(m)
    return m, clamp_a, clamp_e.astype(np.int32)


def pack(models: List[Tuple[L.Model, np.ndarray, np.ndarray]], gap: float) -> Tuple[L.Model, np.ndarray, np.ndarray, List[Tuple[float, float]]]:
    """Replicas side by side along x, gaps of `gap`; one periodic y-z cross section."""
    xs, vs, nx, nv, et, ca, ce, spans = [], [], [], [], [], [], [], []
    x = 0.0
    for m, cla, cle in models:
        lo = min(m.atom_x[:, 0].min() if m.natoms else np.inf, m.nodex[:, :, 0].min())
        hi = max(m.atom_x[:, 0].max() if m.natoms else -np.inf, m.nodex[:, :, 0].max())
        shift = x - lo
        xa = m.atom_x.copy()
        xa[:, 0] += shift
        xn = m.nodex.copy()
        xn[:, :, 0] += shift
        xs.append(xa)
        vs.append(m.atom_v)
        nx.append(xn)
        nv.append(m.nodev)
        et.append(m.elem_type)
        ca.append(cla)
        ce.append(cle)
        spans.append((x, x + hi - lo))
        x += (hi - lo) + gap
    m0 = models[0][0]
    big = L.Model(boxlo=np.array([-0.5 * gap, m0.boxlo[1], m0.boxlo[2]]),
                  boxhi=np.array([x - 0.5 * gap, m0.boxhi[1], m0.boxhi[2]]),
                  periodic=(False, True, True), mass=m0.mass, atom_x=np.concatenate(xs),
                  atom_v=np.concatenate(vs), etypes=m0.etypes, elem_type=np.concatenate(et),
                  nodex=np.concatenate(nx), nodev=np.concatenate(nv), lattice_a=m0.lattice_a)
    return big, np.concatenate(ca), np.concatenate(ce), spans


def class_config(pair: str) -> dict:
    st = STYLE[pair]
    cfg = dict(units=st["units"], boundary="f p p", pair="eam" if pair == "eam" else "lj/cut",
               skin=st["skin"], every=10, delay=0, check=True, dt=st["dt"], gauss_per_element=8)
    if pair == "lj":
        cfg["lj"] = (1.0, 1.0, 2.5)
    return cfg


def _prepare(s: cacg.System):
    s.setup()
    s.neighbor_build()
    s.neighbor_ebuild()
    s.neighbor_nbuild()
    s.pair_compute()
    s.pair_ecompute()


def _snapshot(s: cacg.System):
    a, e = s.atoms(), s.elements()
    return a["x"].copy(), a["v"].copy(), e["nodex"].copy(), e["nodev"].copy()


def _restore(s: cacg.System, snap):
    s.put_atoms(snap[0], snap[1])
    s.put_nodes(snap[2], snap[3])


def autotune(s: cacg.System, skin: float, steps: int = 20) -> Dict:
    """Fastest (bin size, block size) of the candidates on `steps` steps, each
    trial from the same starting state."""
    best, trials = None, []
    snap = _snapshot(s)
    for binsize in (0.0, skin):  # 0: the reference's default r_n / 2
        for block in (256, 512):
            s.command(f"neigh_modify binsize {binsize!r}" if binsize else "neigh_modify binsize 0.0")
            s.command(f"tune block {block}")
            _restore(s, snap)
            _prepare(s)
            s.run(3)
            s.run(steps)
            ms = s.timing()[0] / steps
            trials.append({"binsize": binsize or "default", "block": block, "ms_per_step": ms})
            if best is None or ms < best[0]:
                best = (ms, binsize, block)
    s.command(f"neigh_modify binsize {best[1]!r}" if best[1] else "neigh_modify binsize 0.0")
    s.command(f"tune block {best[2]}")
    _restore(s, snap)
    _prepare(s)
    return {"chosen": {"binsize": best[1] or "default", "block": best[2]}, "trials": trials}


def run_batch(eam_file: str, n: int = 256, steps: int = 2000, seed: int = 4, tune: bool = True,
              device: int = 0, mode: int = cacg.MIXED) -> Dict:
    """All replicas, class by class; returns per-class and whole-batch site-steps/s."""
    reps = draw_replicas(n, seed)
    classes: Dict[Tuple[str, int], List[Replica]] = {}
    for r in reps:
        classes.setdefault((r.pair, size_class(r.sites)), []).append(r)
    out, tot_sites_steps, tot_ms = [], 0.0, 0.0
    for (pair, k), rs in sorted(classes.items()):
        periods = SIZE_CLASSES[k][2]
        t0 = time.perf_counter()
        big, cla, cle, spans = pack([replica_model(r, periods) for r in rs], STYLE[pair]["gap"])
        t_build = time.perf_counter() - t0
        cfg = class_config(pair)
        s = cacg.System(device)
        try:
            W.configure_system(s, big, cfg, eam_file)
            s.set_group("clamp", cla, cle)
            s.command("fix 2 clamp setforce 0.0 0.0 0.0")
            s.set_precision(mode)
            s.init()
            _prepare(s)
            tuned = autotune(s, cfg["skin"]) if tune else None
            sites = W.metric_sites(big, cfg)
            s.run(3)
            c0 = s.counts()
            s.run(steps)
            ms = s.timing()[0]
            c1 = s.counts()
            out.append({"pair": pair, "size_class": list(SIZE_CLASSES[k][:2]), "replicas": len(rs),
                         "sites": sites, "atoms": big.natoms, "elements": big.nelements,
                         "cross_section_periods": periods, "steps": steps, "ms": ms,
                         "site_steps_per_s": sites * steps / (ms * 1e-3),
                         "graph_steps": c1["graph_steps"] - c0["graph_steps"],
                         "rebuilds": c1["rebuilds"] - c0["rebuilds"], "build_s": round(t_build, 2),
                         "autotune": tuned})
            tot_sites_steps += sites * steps
            tot_ms += ms
        finally:
            s.close()
    return {"replicas": n, "classes": out, "site_steps_per_s": tot_sites_steps / (tot_ms * 1e-3),
            "total_sites": int(sum(c["sites"] for c in out)), "steps": steps}
