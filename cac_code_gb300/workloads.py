"""The synthetic benchmark configurations, as seeded models plus input commands.

C1  LJ CAC slab (reduced units): 16x16x16-cell atom slab (16,384 atoms) between
    32+32 rhombohedral elements with 8 sites per edge, 2x2x2 Gauss points,
    periodic y,z, T* = 0.1, dt = 0.005, neighbor 2.8 bin.
C2  EAM Cu CAC slab (metal units): 25x100x100-cell atom slab (1,000,000 atoms)
    between 10,000+10,000 elements with 10 sites per edge (1,000 sites each);
    integration points = 8 Gauss points + the 8 nodes (weight 0, needed for the
    EAM nodal densities); periodic y,z, 300 K, dt = 1 fs, neighbor 7.5 bin.

"Edge of N spacings" in the configuration text is realised as N lattice sites
per element edge, so the element period (N lattice constants) divides the
atom slab's y,z extent and elements tile the FCC lattice without shared sites.
The site-steps/s metric counts atoms plus Gauss integration points; node
density rows and interpolated neighbor sites are work, not sites.
"""
from __future__ import annotations

import os
from typing import Tuple

import numpy as np

from . import lattice as L

KB = {"lj": 1.0, "metal": 8.617343e-5}
MVV2E = {"lj": 1.0, "metal": 1.0364269e-4}
A_LJ = 1.587401
A_CU = 3.615


def c1_lj(seed: int = 1) -> Tuple[L.Model, dict]:
    m = L.make_slab_model(A_LJ, 1.0, (16, 16, 16), 8, 4, L.gauss_intp(8, False))
    L.thermalize(m, 0.1, KB["lj"], MVV2E["lj"], seed)
    L.remap_into_box(m)
    cfg = dict(units="lj", boundary="f p p", pair="lj/cut", lj=(1.0, 1.0, 2.5), skin=2.8,
               every=10, delay=0, check=True, dt=0.005, gauss_per_element=8)
    return m, cfg


def c2_eam(cells=(25, 100, 100), layers: int = 50, nae: int = 10, seed: int = 2,
           temperature: float = 300.0) -> Tuple[L.Model, dict]:
    m = L.make_slab_model(A_CU, L.AnalyticEAM().mass, cells, nae, layers,
                          L.gauss_intp(nae, True))
    L.thermalize(m, temperature, KB["metal"], MVV2E["metal"], seed)
    L.remap_into_box(m)
    cfg = dict(units="metal", boundary="f p p", pair="eam", skin=7.5, every=10, delay=0,
               check=True, dt=0.001, gauss_per_element=8)
    return m, cfg


def c2_sample(seed: int = 3) -> Tuple[L.Model, dict]:
    """A small replica with C2's structure and atom:element ratio (50:1), used for
    the bounded CPU samples: 8,000 atoms + 160 elements."""
    return c2_eam(cells=(5, 20, 20), layers=10, seed=seed)


def metric_sites(m: L.Model, cfg: dict) -> int:
    return m.natoms + cfg["gauss_per_element"] * m.nelements


def write_eam(path: str, n: int = 2000) -> str:
    """Analytic EAM Cu tabulated with Nr = Nrho = n (the C2/C3 configuration)."""
    if not os.path.exists(path):
        L.write_eam_funcfl(L.AnalyticEAM(), path, nrho=n, nr=n)
    return path


def commands(cfg: dict, eam_file: str = "") -> list:
    out = [f"units {cfg['units']}", f"boundary {cfg['boundary']}"]
    return out


def pair_commands(cfg: dict, eam_file: str = "") -> list:
    if cfg["pair"] == "lj/cut":
        e, s, c = cfg["lj"]
        out = [f"pair_style lj/cut {c!r}", f"pair_coeff 1 1 {e!r} {s!r}"]
    else:
        out = ["pair_style eam", f"pair_coeff 1 1 {eam_file}"]
    out += [f"neighbor {cfg['skin']!r} bin",
            f"neigh_modify every {cfg['every']} delay {cfg['delay']} "
            f"check {'yes' if cfg['check'] else 'no'}",
            f"timestep {cfg['dt']!r}", "fix 1 all nve"]
    return out


def configure_system(sys_, m: L.Model, cfg: dict, eam_file: str = "") -> None:
    """Drive a cacg.System through the reference-style commands and upload ``m``."""
    for c in commands(cfg):
        sys_.command(c)
    sys_.load_model(m)
    for c in pair_commands(cfg, eam_file):
        sys_.command(c)


def oracle_kwargs(cfg: dict, eam_file: str = "") -> dict:
    kw = dict(units=cfg["units"], pair=cfg["pair"], skin=cfg["skin"], every=cfg["every"],
              delay=cfg["delay"], check=cfg["check"], dt=cfg["dt"])
    if cfg["pair"] == "eam":
        kw["eam_file"] = eam_file
    else:
        kw["lj"] = cfg["lj"]
    return kw
