"""The synthetic benchmark configurations, as seeded models plus input commands.

"An edge of N primitive spacings" is realised as N + 1 lattice sites per
element edge where the element period then divides the atom slab's y,z extent;
elements tile the FCC lattice with no shared sites.

C1  LJ CAC slab (reduced units): 16x16x16-cell atom slab (16,384 atoms) between
    32+32 rhombohedral elements with 8 sites per edge (7 spacings: a period of
    9 sites does not divide the 16-cell slab), 2x2x2 Gauss points, periodic
    y,z, T* = 0.1, dt = 0.005, neighbor 2.8 bin.
C2  EAM Cu CAC slab (metal units): 21x110x110-cell atom slab (1,016,400 atoms)
    between 10,000+10,000 elements with 11 sites per edge (10 spacings, 1,331
    sites each); integration points = 8 Gauss points + the 8 nodes (weight 0,
    needed for the EAM nodal densities); periodic y,z, 300 K, dt = 1 fs,
    neighbor 7.5 bin.
C3  the C2 model at 83x110x110 cells (4,017,200 atoms) + 500+500 element planes
    (200,000 elements, 11 sites per edge), for the strain ramp.
C5  the surrogate configuration: 16x176x176 cells (1,982,464 atoms) + 488+488
    element planes of 512 (499,712 elements, 11 sites per edge; 3,997,696 Gauss
    points).

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


def c2_eam(cells=(21, 110, 110), layers: int = 50, nae: int = 11, seed: int = 2,
           temperature: float = 300.0) -> Tuple[L.Model, dict]:
    m = L.make_slab_model(A_CU, L.AnalyticEAM().mass, cells, nae, layers,
                          L.gauss_intp(nae, True))
    L.thermalize(m, temperature, KB["metal"], MVV2E["metal"], seed)
    L.remap_into_box(m)
    cfg = dict(units="metal", boundary="f p p", pair="eam", skin=7.5, every=10, delay=0,
               check=True, dt=0.001, gauss_per_element=8)
    return m, cfg


def c2_sample(seed: int = 3) -> Tuple[L.Model, dict]:
    """A small replica with C2's structure and about its atom:element ratio
    (61:1 against 51:1): 9,680 atoms + 160 elements, 11 sites per edge."""
    return c2_eam(cells=(5, 22, 22), layers=10, seed=seed)


def c3_eam(seed: int = 4) -> Tuple[L.Model, dict]:
    """C3: 4,017,200 atoms + 200,000 elements (11 sites per edge)."""
    return c2_eam(cells=(83, 110, 110), layers=500, seed=seed)


def c5_eam(seed: int = 6) -> Tuple[L.Model, dict]:
    """C5: 1,982,464 atoms + 499,712 elements (11 sites per edge), the
    surrogate configuration."""
    return c2_eam(cells=(16, 176, 176), layers=488, seed=seed)


def c2_medium(seed: int = 2) -> Tuple[L.Model, dict]:
    """C2's structure at profiling size: 266,200 atoms + 7,200 elements."""
    return c2_eam(cells=(22, 55, 55), layers=72, seed=seed)


def c5_medium(seed: int = 6) -> Tuple[L.Model, dict]:
    """C5's structure at profiling size: 247,808 atoms + 64,000 elements."""
    return c2_eam(cells=(8, 88, 88), layers=250, seed=seed)


def c5_sample(seed: int = 7) -> Tuple[L.Model, dict]:
    """A small replica with C5's structure and atom:element ratio (about 4:1):
    7,744 atoms + 1,936 elements, 11 sites per edge."""
    return c2_eam(cells=(4, 22, 22), layers=121, seed=seed)


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
