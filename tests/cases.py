"""Parity cases shared by the tests and tests/golden/make_golden.py.

Each case is a seeded CAC configuration plus the reference commands and the
harness directives that produce its golden outputs.  Inputs are stored in the
fixture file itself (positions, velocities, tables), so nothing depends on a
random generator or libm being identical across hosts.
"""
from __future__ import annotations

import json
import os
from typing import Dict

import numpy as np

from cac_code_gb300 import lattice as L

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")
EAM_FILE = os.path.join(GOLDEN, "Cu_analytic.eam")
A_LJ = 1.587401   # FCC at rho* = 1.0: a = (4/rho*)^(1/3)
A_CU = 3.615

# name -> settings; "steps" steps after the single-shot outputs
CASES: Dict[str, dict] = {
    # atoms only, periodic, LJ: list + forces + 5 steps with a rebuild check every step
    "lj_atoms": dict(kind="atoms", units="lj", pair="lj/cut", skin=2.8, boundary="p p p",
                     every=1, delay=0, check=True, binsize=0.0, nsplit=2, dt=None,
                     cells=(4, 4, 4), jitter=0.05, temp=0.5, seed=11, steps=5),
    # LJ CAC slab: atoms + 2 planes of nae=4 elements per side, rebuild every step
    "lj_cac": dict(kind="slab", units="lj", pair="lj/cut", skin=2.8, boundary="f p p",
                   every=1, delay=0, check=False, binsize=0.0, nsplit=2, dt=None,
                   cells=(4, 8, 8), nae=4, layers=2, nodes_as_ip=False, jitter=0.03,
                   temp=0.1, seed=12, steps=4),
    # same with a user bin size large enough that the element list sees all
    # neighbors within cut_all (the default r_n/2 bins miss them)
    "lj_cac_bigbins": dict(kind="slab", units="lj", pair="lj/cut", skin=2.8,
                           boundary="f p p", every=1, delay=0, check=False, binsize=11.5,
                           nsplit=2, dt=None, cells=(4, 8, 8), nae=4, layers=2,
                           nodes_as_ip=False, jitter=0.03, temp=0.1, seed=13, steps=2),
    # EAM CAC slab, metal units, nodes are integration points (EAM nodal density)
    "eam_cac": dict(kind="slab", units="metal", pair="eam", skin=7.5, boundary="f p p",
                    every=2, delay=0, check=True, binsize=0.0, nsplit=2, dt=None,
                    cells=(4, 8, 8), nae=4, layers=2, nodes_as_ip=True, jitter=0.05,
                    temp=300.0, seed=14, steps=6),
    # lj_cac with regions, groups and the post-force fixes setforce / viscous
    "lj_cac_fixes": dict(kind="slab", units="lj", pair="lj/cut", skin=2.8, boundary="f p p",
                         every=1, delay=0, check=False, binsize=0.0, nsplit=2, dt=None,
                         cells=(4, 8, 8), nae=4, layers=2, nodes_as_ip=False, jitter=0.03,
                         temp=0.1, seed=16, steps=6, fixes=True),
    # EAM atoms only, periodic, forced rebuild every step
    "eam_atoms": dict(kind="atoms", units="metal", pair="eam", skin=7.5, boundary="p p p",
                      every=1, delay=0, check=False, binsize=0.0, nsplit=2, dt=None,
                      cells=(5, 5, 5), jitter=0.08, temp=600.0, seed=15, steps=3),
}

KB = {"lj": 1.0, "metal": 8.617343e-5}
MVV2E = {"lj": 1.0, "metal": 1.0364269e-4}


def build_model(cfg: dict) -> L.Model:
    """Deterministic-in-this-process model for a case (fixtures store the result)."""
    a = A_LJ if cfg["units"] == "lj" else A_CU
    mass = 1.0 if cfg["units"] == "lj" else L.AnalyticEAM().mass
    rng = np.random.default_rng(cfg["seed"])
    if cfg["kind"] == "atoms":
        m = L.make_slab_model(a, mass, cfg["cells"], 0, 0, (None, None))
        m.periodic = (True, True, True)
        m.boxlo = np.zeros(3)
        m.boxhi = np.array(cfg["cells"], dtype=np.float64) * a
    else:
        ip = L.gauss_intp(cfg["nae"], cfg["nodes_as_ip"])
        m = L.make_slab_model(a, mass, cfg["cells"], cfg["nae"], cfg["layers"], ip)
    m.atom_x = m.atom_x + rng.normal(0.0, cfg["jitter"], m.atom_x.shape)
    if m.nelements:
        m.nodex = m.nodex + rng.normal(0.0, cfg["jitter"], m.nodex.shape)
    L.thermalize(m, cfg["temp"], KB[cfg["units"]], MVV2E[cfg["units"]], cfg["seed"] + 1000)
    L.remap_into_box(m)
    return m


def _fix_bounds(m: L.Model):
    lo, hi = float(m.boxlo[0]), float(m.boxhi[0])
    return lo + 0.3 * (hi - lo), lo + 0.7 * (hi - lo)


def fix_lines(cfg: dict, m: L.Model) -> list:
    """Reference commands of a case's regions, groups and post-force fixes."""
    if not cfg.get("fixes"):
        return []
    x1, x2 = _fix_bounds(m)
    return [f"region lo block INF {x1!r} INF INF INF INF",
            f"region hi block {x2!r} INF INF INF INF INF",
            "group lo region lo",
            "group hi region hi",
            "group mid subtract all lo hi",
            "fix 2 lo setforce 0.0 0.0 NULL",
            "fix 3 hi viscous 0.5",
            "fix 4 mid viscous 0.05"]


def fix_setup(cfg: dict, m: L.Model):
    """The same groups as masks (bit 1 all, 2 lo, 4 hi, 8 mid: region block
    bounds inclusive, atoms by position, elements by centre) and the fixes in
    order, for the oracle."""
    if not cfg.get("fixes"):
        return None, None, []
    x1, x2 = _fix_bounds(m)

    def masks(x):
        mk = np.ones(len(x), dtype=np.int32)
        lo = x[:, 0] <= x1
        hi = x[:, 0] >= x2
        mk[lo] |= 2
        mk[hi] |= 4
        mk[~lo & ~hi] |= 8
        return mk
    am = masks(m.atom_x)
    em = masks(m.element_centres()) if m.nelements else np.zeros(0, np.int32)
    return am, em, [("setforce", 2, (0.0, 0.0, None)), ("viscous", 4, 0.5),
                    ("viscous", 8, 0.05)]


def settings_kwargs(cfg: dict, eam_file: str = EAM_FILE) -> dict:
    kw = dict(units=cfg["units"], pair=cfg["pair"], skin=cfg["skin"], every=cfg["every"],
              delay=cfg["delay"], check=cfg["check"], binsize=cfg["binsize"],
              nsplit=cfg["nsplit"], dt=cfg["dt"])
    if cfg["pair"] == "eam":
        kw["eam_file"] = eam_file
    else:
        kw["lj"] = (1.0, 1.0, 2.5)
    return kw


def model_to_arrays(m: L.Model) -> dict:
    out = dict(boxlo=m.boxlo, boxhi=m.boxhi, periodic=np.array(m.periodic, dtype=np.int32),
               mass=np.array([m.mass]), atom_x=m.atom_x, atom_v=m.atom_v,
               nodex=m.nodex, nodev=m.nodev, elem_type=m.elem_type.astype(np.int32),
               elem_centre=m.element_centres())
    if m.nelements:
        et = m.etypes[0]
        out.update(nae=np.array(et.nae, dtype=np.int32), intp=et.intp.astype(np.int32),
                   weight=et.weight)
    return out


def model_from_arrays(z) -> L.Model:
    etypes = []
    if z["nodex"].shape[0]:
        etypes = [L.ElementType(tuple(int(v) for v in z["nae"]), z["intp"].astype(np.int64),
                                z["weight"].astype(np.float64))]
    m = L.Model(boxlo=z["boxlo"].copy(), boxhi=z["boxhi"].copy(),
                periodic=tuple(bool(v) for v in z["periodic"]), mass=float(z["mass"][0]),
                atom_x=z["atom_x"].copy(), atom_v=z["atom_v"].copy(), etypes=etypes,
                elem_type=z["elem_type"].astype(np.int64), nodex=z["nodex"].copy(),
                nodev=z["nodev"].copy())
    return m


def load_golden(name: str):
    path = os.path.join(GOLDEN, name + ".npz")
    z = np.load(path)
    cfg = json.loads(str(z["settings"]))
    return cfg, z


def neighbor_pairs(num, neigh, tag_all, x_all, owner_x, box_prd):
    """Rows as sorted (owner tag, image shift) tuples: set comparison across
    different ghost numberings."""
    rows = []
    o = 0
    for i in range(len(num)):
        js = neigh[o:o + num[i]]
        o += num[i]
        t = tag_all[js]
        shift = np.rint((x_all[js] - owner_x[t - 1]) / box_prd).astype(np.int64)
        rows.append(sorted(zip(t.tolist(), map(tuple, shift.tolist()))))
    return rows
