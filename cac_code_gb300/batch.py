"""Batched independent CAC replicas on one GPU.

Replicas of uneven size (sites drawn log-uniform in [2k, 60k], atom fraction
uniform in [0.2, 0.8]), temperature (uniform in [10, 600] K; in LJ units
T* = kB T / 0.4 eV) and applied shear (uniform in [0, 4 %], an affine displacement held by
clamped boundary slabs under fix setforce) are grouped by pair style and size
class.  The replicas of a class share one handle: they sit side by side along
the non-periodic x axis, each a slab with the class's periodic y-z cross
section, separated by gaps wider than the element neighbor cutoff, so that no
list ever crosses from one replica into another.  Every kernel of a step then
covers all replicas of the class at once.

Each class runs its steps through the device step loop ("tune loop device"):
step after step inside a CUDA graph, the rebuild decision (Neighbor::decide,
neighbor.cpp:1150-1163) taken on the device, back to the host only for a step
that needs a rebuild.  All classes' loops are the branches of one graph
(cacg_run_batch): one launch runs every replica until each class is done or
needs a rebuild; the host performs those rebuilds and launches again.  (The
alternatives: each handle's loop from its own host thread, or one class after
another.)

The nodes are damped (fix viscous): under the reference's element force the
elements of these slabs gain kinetic energy without bound over some hundreds
of steps, and the damping keeps 2,000 steps of every replica bounded.

Per class an autotuner searches, on a few steps from the same starting state
each, the bin size (the reference's default r_n / 2, or r_n) and the threads
per block of the persistent mixed-precision kernels (128, 256, 512), then, on
the best of those, one stream or two (atom and element chains) and the
arrangement of the fused element kernel (coefficients in registers, in shared
memory, or in shared memory with two entries in flight per lane), and keeps
the fastest.

The reference runs one system per process; it has no batching.
"""
from __future__ import annotations

import dataclasses
import math
import threading
import time
from typing import Dict, List, Tuple

import numpy as np

from . import cacg
from . import lattice as L
from . import workloads as W

A_LJ = (4.0 / 1.0) ** (1.0 / 3.0)  # FCC at rho* = 1.0

# per pair style: lattice, element size (sites per edge), cross sections (in
# element periods) of the size classes, gap between replicas, reference commands
# (damp: fix viscous gamma of the nodes, relaxation times m / gamma of about 8
# steps for EAM nodes of 1000 / 8 Cu masses and 1.3 steps for LJ nodes of
# 512 / 8 masses; in the oracle the hottest replica of the smallest class runs
# 2,000 steps bounded with these, while LJ nodes under gamma 1000 or 5000 gain
# energy again after 1,000-2,000 steps)
STYLE = {
    "eam": dict(a=W.A_CU, nae=10, units="metal", skin=7.5, gap=70.0, kb=W.KB["metal"],
                mvv2e=W.MVV2E["metal"], t_scale=1.0, dt=0.001, damp=100.0),
    # LJ temperatures: T* = kB T / eps with eps = 0.4 eV (a Cu-like well), so
    # 10-600 K maps to T* = 0.002-0.13, below the LJ melting point
    "lj": dict(a=A_LJ, nae=8, units="lj", skin=2.8, gap=20.0, kb=1.0, mvv2e=1.0,
               t_scale=8.617343e-5 / 0.4, dt=0.005, damp=10000.0),
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


def _apply(s: cacg.System, opts: Dict) -> None:
    b = opts["binsize"]
    s.command(f"neigh_modify binsize {b!r}" if b else "neigh_modify binsize 0.0")
    s.command(f"tune block {opts['block']}")
    if "streams" in opts:
        s.command(f"tune streams {opts['streams']}")
    if "fused_variant" in opts:
        s.command(f"tune fused_variant {opts['fused_variant']}")


def autotune(s: cacg.System, skin: float, steps: int = 12) -> Dict:
    """Fastest options on `steps` steps, each trial from the same starting
    state: bin size x block size, then streams x fused-kernel arrangement on
    the best of those (the arrangements only when the element passes run
    fused)."""
    trials = []
    snap = _snapshot(s)

    def trial(opts):
        _apply(s, opts)
        _restore(s, snap)
        _prepare(s)
        s.run(3)
        s.run(steps)
        ms = s.timing()[0] / steps
        trials.append(dict(opts, binsize=opts["binsize"] or "default", ms_per_step=ms))
        return ms

    stage1 = [{"binsize": b, "block": k} for b in (0.0, skin) for k in (128, 256, 512)]
    best = min(stage1, key=trial)
    fused = s.counts()["elem_fused"] == 1
    stage2 = [dict(best, streams=st, fused_variant=v)
              for st in ("yes", "no") for v in ((0, 1, 2) if fused else (1,))]
    best = min(stage2, key=trial)
    _apply(s, best)
    _restore(s, snap)
    _prepare(s)
    chosen = dict(best, binsize=best["binsize"] or "default")
    return {"chosen": chosen, "trials": trials}


@dataclasses.dataclass
class _Class:
    pair: str
    k: int
    reps: List[Replica]
    system: cacg.System
    sites: int
    atoms: int
    elements: int
    build_s: float
    tuned: Dict = None
    ms: float = 0.0
    wall_s: float = 0.0
    c0: Dict = None
    c1: Dict = None
    error: BaseException = None


def _prepare_class(pair: str, k: int, rs: List[Replica], eam_file: str, device: int, mode: int,
                   tune: bool, loop: str) -> _Class:
    periods = SIZE_CLASSES[k][2]
    st = STYLE[pair]
    t0 = time.perf_counter()
    big, cla, cle, spans = pack([replica_model(r, periods) for r in rs], st["gap"])
    t_build = time.perf_counter() - t0
    cfg = class_config(pair)
    s = cacg.System(device)
    try:
        W.configure_system(s, big, cfg, eam_file)
        s.set_group("clamp", cla, cle)
        s.command("fix 2 clamp setforce 0.0 0.0 0.0")
        if big.nelements:
            s.set_group("nodes", None, np.ones(big.nelements, dtype=np.int32))
            s.command(f"fix 3 nodes viscous {st['damp']!r}")
        s.set_precision(mode)
        s.command(f"tune loop {loop}")
        s.init()
        _prepare(s)
        c = _Class(pair, k, rs, s, W.metric_sites(big, cfg), big.natoms, big.nelements,
                   round(t_build, 2))
        c.tuned = autotune(s, cfg["skin"]) if tune else None
        s.run(3)
        return c
    except BaseException:
        s.close()
        raise


def _run_class(c: _Class, steps: int) -> None:
    try:
        c.c0 = c.system.counts()
        t0 = time.perf_counter()
        c.system.run(steps)
        c.wall_s = time.perf_counter() - t0
        c.ms = c.system.timing()[0]
        c.c1 = c.system.counts()
    except BaseException as ex:  # re-raised by the caller
        c.error = ex


def run_batch(eam_file: str, n: int = 256, steps: int = 2000, seed: int = 4, tune: bool = True,
              device: int = 0, mode: int = cacg.MIXED, loop: str = "device",
              schedule: str = "graph") -> Dict:
    """All replicas: the classes prepared (and autotuned) one after another,
    then timed together: schedule "graph" runs every class's loop as a branch
    of one CUDA graph (cacg_run_batch), "threads" each class from its own host
    thread on its own stream, "sequential" one class after another.  Returns
    per-class counts and the whole batch's site-steps/s (the total site-steps
    over the wall time of the timed run; per class also site-steps/s over its
    own run where the class runs alone)."""
    reps = draw_replicas(n, seed)
    groups: Dict[Tuple[str, int], List[Replica]] = {}
    for r in reps:
        groups.setdefault((r.pair, size_class(r.sites)), []).append(r)
    classes: List[_Class] = []
    try:
        for (pair, k), rs in sorted(groups.items()):
            classes.append(_prepare_class(pair, k, rs, eam_file, device, mode, tune, loop))
        t0 = time.perf_counter()
        if schedule == "graph":
            for c in classes:
                c.c0 = c.system.counts()
            cacg.run_batch([c.system for c in classes], steps)
            for c in classes:
                c.c1 = c.system.counts()
                c.ms = float("nan")
        elif schedule == "threads":
            threads = [threading.Thread(target=_run_class, args=(c, steps)) for c in classes]
            for t in threads:
                t.start()
            for t in threads:
                t.join()
        else:
            for c in classes:
                _run_class(c, steps)
        wall = time.perf_counter() - t0
        for c in classes:
            if c.error is not None:
                raise c.error
        out = []
        for c in classes:
            c0, c1 = c.c0, c.c1
            out.append({"pair": c.pair, "size_class": list(SIZE_CLASSES[c.k][:2]),
                        "replicas": len(c.reps), "sites": c.sites, "atoms": c.atoms,
                        "elements": c.elements, "cross_section_periods": SIZE_CLASSES[c.k][2],
                        "steps": steps, "ms": c.ms if schedule != "graph" else None,
                        "site_steps_per_s": (c.sites * steps / (c.ms * 1e-3)
                                             if schedule != "graph" else None),
                        "graph_steps": c1["graph_steps"] - c0["graph_steps"],
                        "rebuilds": c1["rebuilds"] - c0["rebuilds"],
                        "loop_launches": c1["loop_launches"] - c0["loop_launches"],
                        "host_decisions": c1["host_decisions"] - c0["host_decisions"],
                        "build_s": c.build_s, "autotune": c.tuned})
        tot = sum(c.sites for c in classes) * steps
        return {"replicas": n, "classes": out, "steps": steps,
                "total_sites": int(sum(c.sites for c in classes)),
                "site_steps_per_s": tot / wall, "wall_s": round(wall, 3),
                "schedule": schedule, "loop": loop}
    finally:
        for c in classes:
            c.system.close()
