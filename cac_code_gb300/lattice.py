"""Synthetic CAC models: FCC atoms, rhombohedral 8-node elements, potentials.

Everything here is seeded and deterministic.  It writes the reference's own
input formats so the same files drive both this library and the reference:

* data files as parsed by ReadData (read_data.cpp:166-211): header counts and box,
  ``Masses``, ``NAAE`` (``type nx ny nz``), ``Numint`` (``type n``), ``Intp``
  (``type idx i j k w``, integer lattice indices, element.cpp:1144-1166),
  ``Atoms`` (``id type x y z``), ``Elements`` (``id type xc yc zc``) and
  ``Nodes`` (``eid k x y z ntag`` or the 9-word form with velocities,
  element.cpp:478-540);
* the EAM potential file variant PairEAM::read_file reads (pair_eam.cpp:197-248):
  comment line, ``int mass``, ``nrho drho nr dr cut``, then F(rho), rho(r) and
  r*phi(r) (stored directly as z2r, pair_eam.cpp:487).

Element geometry.  An element of type t with ``n`` lattice sites per edge spans
``n-1`` primitive FCC spacings along a1=(0,1,1)a/2, a2=(1,0,1)a/2, a3=(1,1,0)a/2.
Node k sits at the parent-space corner listed in ``NODE_PARENT`` (the reference's
node order, element.cpp:1340-1347), so interior site (i,j,k) is exactly the
lattice site R + i*a1 + j*a2 + k*a3.  Elements tile the lattice with period
``n`` spacings along each ai, so no two elements (and no element and the atom
slab) share a lattice site.
"""
from __future__ import annotations

import dataclasses
import math
from typing import List, Optional, Sequence, Tuple

import numpy as np

# parent-space corner of node k (element.cpp:1340-1347 / 1403-1410 ordering)
NODE_PARENT = np.array(
    [[-1, -1, -1], [1, -1, -1], [1, 1, -1], [-1, 1, -1],
     [-1, -1, 1], [1, -1, 1], [1, 1, 1], [-1, 1, 1]], dtype=np.int64)

FCC_BASIS = np.array([[0.0, 0.0, 0.0], [0.0, 0.5, 0.5], [0.5, 0.0, 0.5], [0.5, 0.5, 0.0]])
PRIMITIVE = np.array([[0.0, 0.5, 0.5], [0.5, 0.0, 0.5], [0.5, 0.5, 0.0]])


@dataclasses.dataclass
class ElementType:
    nae: Tuple[int, int, int]
    intp: np.ndarray          # (numint, 3) integer lattice indices
    weight: np.ndarray        # (numint,)


@dataclasses.dataclass
class Model:
    """A CAC configuration in the reference's data-file terms."""
    boxlo: np.ndarray
    boxhi: np.ndarray
    periodic: Tuple[bool, bool, bool]
    mass: float
    atom_x: np.ndarray                 # (na, 3)
    atom_v: np.ndarray                 # (na, 3)
    etypes: List[ElementType]
    elem_type: np.ndarray              # (ne,) 1-based
    nodex: np.ndarray                  # (ne, 8, 3)
    nodev: np.ndarray                  # (ne, 8, 3)
    lattice_a: float = 1.0

    @property
    def natoms(self) -> int:
        return int(self.atom_x.shape[0])

    @property
    def nelements(self) -> int:
        return int(self.nodex.shape[0])

    def element_centres(self) -> np.ndarray:
        # the reference rejects a centre farther than 0.1 from the node mean
        # (element.cpp:608-622); write the mean in node order, as FixNVE does
        c = np.zeros((self.nelements, 3))
        for k in range(8):
            c += self.nodex[:, k, :]
        return c / 8.0

    def n_integration_points(self) -> int:
        return int(sum(len(self.etypes[t - 1].intp) for t in self.elem_type))

    def n_sites_metric(self) -> int:
        """Atoms plus integration points: the units of the site-steps/s metric."""
        return self.natoms + self.n_integration_points()


def fcc_sites(ncell: Sequence[int], a: float, origin=(0.0, 0.0, 0.0)) -> np.ndarray:
    """FCC lattice sites of an nx*ny*nz cubic block in lattice (cell-major) order."""
    nx, ny, nz = ncell
    ii, jj, kk = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    cells = np.stack([ii.ravel(), jj.ravel(), kk.ravel()], axis=1).astype(np.float64)
    pos = (cells[:, None, :] + FCC_BASIS[None, :, :]).reshape(-1, 3) * a
    return pos + np.asarray(origin, dtype=np.float64)


def element_nodes(origin: np.ndarray, nae: int, a: float) -> np.ndarray:
    """Node positions (8, 3) of a rhombohedral element whose node 0 is ``origin``."""
    return elements_nodes(np.asarray(origin, dtype=np.float64)[None, :], nae, a)[0]


def elements_nodes(origins: np.ndarray, nae: int, a: float) -> np.ndarray:
    """Node positions (n, 8, 3) of rhombohedral elements whose node 0 sits at
    ``origins`` (n, 3): origin + t0*span0 + t1*span1 + t2*span2, summed left to
    right, with t the node's parent corner mapped to {0, 1}."""
    span = (nae - 1) * a * PRIMITIVE           # edge vectors along a1, a2, a3
    t = (NODE_PARENT + 1) // 2                 # (8, 3)
    o = np.asarray(origins, dtype=np.float64)[:, None, :]
    return (o + t[None, :, 0:1] * span[0] + t[None, :, 1:2] * span[1]
            + t[None, :, 2:3] * span[2])


def gauss_intp(nae: int, with_nodes: bool) -> Tuple[np.ndarray, np.ndarray]:
    """2x2x2 integration points at the lattice sites nearest xi = +-1/sqrt(3).

    Weights share the element's nae^3 sites evenly over the 8 Gauss points.  With
    ``with_nodes`` the 8 corner nodes are added as weight-0 integration points,
    which PairEAM::ecompute needs for its nodal densities (find_node_list,
    element.cpp:1296-1319; pair_eam.cpp:927-986).
    """
    half = (nae - 1) / 2.0
    lo = int(round(half - half / math.sqrt(3.0)))
    hi = int(round(half + half / math.sqrt(3.0)))
    pts, w = [], []
    if with_nodes:
        for k in range(8):
            t = (NODE_PARENT[k] + 1) // 2
            pts.append([t[0] * (nae - 1), t[1] * (nae - 1), t[2] * (nae - 1)])
            w.append(0.0)
    wg = nae ** 3 / 8.0
    for i in (lo, hi):
        for j in (lo, hi):
            for k in (lo, hi):
                pts.append([i, j, k])
                w.append(wg)
    return np.array(pts, dtype=np.int64), np.array(w, dtype=np.float64)


def all_sites_intp(nae: int) -> Tuple[np.ndarray, np.ndarray]:
    """Every lattice site of the element as an integration point of weight 1."""
    idx = [[i, j, k] for i in range(nae) for j in range(nae) for k in range(nae)]
    return np.array(idx, dtype=np.int64), np.ones(len(idx))


def tile_elements(nae: int, a: float, base_x: float, layers: int, direction: int,
                  ly: float, lz: float) -> np.ndarray:
    """Origins (node 0) of ``layers`` planes of elements, tiled periodically in y,z.

    The element superlattice is nae*(a1, a2, a3); its node-0 x coordinates take the
    values base_x + s*nae*a/2.  Plane k (k = 0..layers-1) uses s = direction*k.
    Each plane holds 2*(ly/(nae a))*(lz/(nae a)) elements; ``ly`` and ``lz`` must be
    multiples of nae*a and ``base_x`` a multiple of a, which keeps every element
    site on the FCC lattice of the atoms.
    """
    per = nae * a
    half = 0.5 * per
    ny_, nz_ = int(round(ly / per)), int(round(lz / per))
    if layers <= 0 or ny_ <= 0 or nz_ <= 0:
        return np.zeros((0, 3))
    # plane k has s = direction*k; y = (n1 + s - n2)*half, z = (n1 + n2)*half,
    # u = n1 + s - n2 and w = n1 + n2 of equal parity with s
    s_ = direction * np.arange(layers, dtype=np.int64)
    uu, ww = np.meshgrid(np.arange(2 * ny_, dtype=np.int64), np.arange(2 * nz_, dtype=np.int64),
                         indexing="ij")
    ss = np.broadcast_to(s_[:, None, None], (layers,) + uu.shape)
    ub = np.broadcast_to(uu[None], ss.shape)
    wb = np.broadcast_to(ww[None], ss.shape)
    keep = (ub + wb - ss) % 2 == 0
    origins = np.stack([base_x + ss[keep] * half, ub[keep] * half, wb[keep] * half], axis=1)
    order = np.lexsort((origins[:, 2], origins[:, 1], origins[:, 0]))
    return origins[order]


def make_slab_model(a: float, mass: float, atom_cells: Tuple[int, int, int], nae: int,
                    elem_layers: int, intp: Tuple[np.ndarray, np.ndarray],
                    periodic_x: bool = False, margin: float = 0.0) -> Model:
    """Atomistic slab of ``atom_cells`` cubic cells flanked on -x and +x by elements.

    ``elem_layers`` is the number of element planes on each side; each plane holds
    2*(ly/(nae a))*(lz/(nae a)) elements.  The atom slab covers x in [0, ax*a); the
    +x element region starts on the next lattice plane (x = ax*a) and the -x region
    ends at x = -a, so no element site coincides with an atom or another element's
    site.  The y,z box is the atom slab's y,z extent, a multiple of nae*a.
    """
    ax, ay, az = atom_cells
    ly, lz = ay * a, az * a
    if nae > 0 and elem_layers > 0:
        per = nae * a
        if abs(ly / per - round(ly / per)) > 1e-9 or abs(lz / per - round(lz / per)) > 1e-9:
            raise ValueError("y,z extent must be a multiple of nae*a")
    atoms = fcc_sites((ax, ay, az), a)
    if nae > 0 and elem_layers > 0:
        left = tile_elements(nae, a, -nae * a, elem_layers, -1, ly, lz)
        right = tile_elements(nae, a, ax * a, elem_layers, +1, ly, lz)
        nodex = elements_nodes(np.concatenate([left, right]), nae, a).reshape(-1, 8, 3)
    else:
        nodex = np.zeros((0, 8, 3))
    if nodex.shape[0]:
        xmin = min(atoms[:, 0].min(), nodex[:, :, 0].min())
        xmax = max(atoms[:, 0].max(), nodex[:, :, 0].max())
    else:
        xmin, xmax = atoms[:, 0].min(), atoms[:, 0].max()
    if periodic_x:
        boxlo_x, boxhi_x = xmin - 0.25 * a, xmax + 0.25 * a + margin
    else:
        boxlo_x, boxhi_x = xmin - 0.5 * a - margin, xmax + 0.5 * a + margin
    ip, w = intp
    et = ElementType((nae, nae, nae), np.asarray(ip), np.asarray(w)) if nodex.shape[0] else None
    return Model(
        boxlo=np.array([boxlo_x, 0.0, 0.0]),
        boxhi=np.array([boxhi_x, ly, lz]),
        periodic=(periodic_x, True, True),
        mass=mass,
        atom_x=atoms,
        atom_v=np.zeros_like(atoms),
        etypes=[et] if et is not None else [],
        elem_type=np.ones(nodex.shape[0], dtype=np.int64),
        nodex=nodex,
        nodev=np.zeros_like(nodex),
        lattice_a=a,
    )


def thermalize(model: Model, temperature: float, kb: float, mvv2e: float, seed: int) -> None:
    """Seeded Gaussian velocities at ``temperature`` for atoms and nodes.

    The reference has no ``velocity create`` (velocity.cpp:56-58 offers set/ramp
    only), so velocities are generated here and written into the data file (the
    9-word Nodes form) or uploaded directly.  Net momentum is removed per set.
    """
    rng = np.random.default_rng(seed)
    if model.natoms:
        s = math.sqrt(kb * temperature / (model.mass * mvv2e))
        v = rng.standard_normal(model.atom_x.shape) * s
        v -= v.mean(axis=0)
        model.atom_v = v
    if model.nelements:
        # one (8, 3) draw per element in element order, scaled by the element
        # type's nodal thermal speed
        sd = np.array([math.sqrt(kb * temperature /
                                 (model.mass * et.nae[0] * et.nae[1] * et.nae[2] / 8.0 * mvv2e))
                       for et in model.etypes])
        v = rng.standard_normal(model.nodex.shape) * sd[np.asarray(model.elem_type) - 1][:, None, None]
        v -= v.reshape(-1, 3).mean(axis=0)
        model.nodev = v


def _fmt(x: float) -> str:
    return repr(float(x))


def write_data(model: Model, path: str, with_velocities: bool = False) -> None:
    """Write ``model`` as a reference data file (read_data.cpp:70-246)."""
    lines = ["CAC data file (synthetic, seeded)", ""]
    lines.append(f"{model.natoms} atoms")
    lines.append("1 atom types")
    if model.nelements:
        lines.append(f"{model.nelements} elements")
        lines.append(f"{len(model.etypes)} element types")
    lines.append(f"{_fmt(model.boxlo[0])} {_fmt(model.boxhi[0])} xlo xhi")
    lines.append(f"{_fmt(model.boxlo[1])} {_fmt(model.boxhi[1])} ylo yhi")
    lines.append(f"{_fmt(model.boxlo[2])} {_fmt(model.boxhi[2])} zlo zhi")
    lines += ["", "Masses", "", f"1 {_fmt(model.mass)}", ""]
    if model.nelements:
        lines += ["NAAE", ""]
        for t, et in enumerate(model.etypes, start=1):
            lines.append(f"{t} {et.nae[0]} {et.nae[1]} {et.nae[2]}")
        lines += ["", "Numint", ""]
        for t, et in enumerate(model.etypes, start=1):
            lines.append(f"{t} {len(et.intp)}")
        lines += ["", "Intp", ""]
        for t, et in enumerate(model.etypes, start=1):
            for m, (p, w) in enumerate(zip(et.intp, et.weight), start=1):
                lines.append(f"{t} {m} {int(p[0])} {int(p[1])} {int(p[2])} {_fmt(w)}")
        lines.append("")
    if model.natoms:
        lines += ["Atoms", ""]
        for i in range(model.natoms):
            x = model.atom_x[i]
            lines.append(f"{i + 1} 1 {_fmt(x[0])} {_fmt(x[1])} {_fmt(x[2])}")
        lines.append("")
    if model.nelements:
        centres = model.element_centres()
        lines += ["Elements", ""]
        for e in range(model.nelements):
            c = centres[e]
            lines.append(f"{e + 1} {int(model.elem_type[e])} {_fmt(c[0])} {_fmt(c[1])} {_fmt(c[2])}")
        lines += ["", "Nodes", ""]
        tag = 1
        for e in range(model.nelements):
            for k in range(8):
                x = model.nodex[e, k]
                if with_velocities:
                    v = model.nodev[e, k]
                    lines.append(f"{e + 1} {k + 1} {_fmt(x[0])} {_fmt(x[1])} {_fmt(x[2])} "
                                 f"{_fmt(v[0])} {_fmt(v[1])} {_fmt(v[2])} {tag}")
                else:
                    lines.append(f"{e + 1} {k + 1} {_fmt(x[0])} {_fmt(x[1])} {_fmt(x[2])} {tag}")
                tag += 1
        lines.append("")
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")


# ----------------------------------------------------------------------------
# analytic EAM Cu (Morse pair, exponential density, sqrt embedding)

@dataclasses.dataclass
class AnalyticEAM:
    """f(r)=exp(-beta(r/re-1)); phi = Morse(D, alpha, r0); F(rho) = -A*sqrt(rho).

    With ``taper`` > 0, f and phi are multiplied by psi(x) = x^4 / (1 + x^4),
    x = (r - cut) / taper (zero beyond the cutoff), so both vanish smoothly
    there and the total energy is conserved in NVE.
    """
    re: float = 2.556
    beta: float = 6.0
    D: float = 0.3429
    alpha: float = 1.3588
    r0: float = 2.866
    A: float = 1.2
    cut: float = 5.5
    mass: float = 63.546
    taper: float = 0.0

    def _psi(self, r):
        if self.taper <= 0.0:
            return 1.0
        x = (np.asarray(r, dtype=np.float64) - self.cut) / self.taper
        x4 = x ** 4
        return np.where(x < 0.0, x4 / (1.0 + x4), 0.0)

    def density(self, r):
        return np.exp(-self.beta * (np.asarray(r) / self.re - 1.0)) * self._psi(r)

    def pair(self, r):
        e = np.exp(-self.alpha * (np.asarray(r) - self.r0))
        return self.D * (e * e - 2.0 * e) * self._psi(r)

    def embed(self, rho):
        return -self.A * np.sqrt(np.maximum(np.asarray(rho), 0.0))


def write_eam_setfl(pot: AnalyticEAM, path: str, element: str = "Cu", nrho: int = 2000,
                    drho: Optional[float] = None, nr: int = 2000,
                    rho_max: Optional[float] = None, r_max: Optional[float] = None) -> None:
    """Tabulate ``pot`` as a one-element setfl file (the eam/alloy format):
    three comment lines, "1 el", "Nrho drho Nr dr cut", "Z mass a lattice",
    F(rho), rho(r), r*phi(r) -- the same grids and values as
    write_eam_funcfl with the same arguments."""
    dr = (pot.cut if r_max is None else r_max) / (nr - 1)
    if rho_max is None:
        rho_max = 40.0
    if drho is None:
        drho = rho_max / (nrho - 1)
    r = np.arange(nr) * dr
    rho = np.arange(nrho) * drho

    def block(vals):
        return [" ".join(f"{v:.16e}" for v in vals[i:i + 5]) for i in range(0, len(vals), 5)]
    lines = ["analytic EAM Cu: exp density, Morse pair, sqrt embedding (synthetic)",
             "setfl layout, one element", "tables as in the funcfl file of the same grids",
             f"1 {element}", f"{nrho} {drho:.16e} {nr} {dr:.16e} {pot.cut:.16e}",
             f"29 {pot.mass:.6f} 3.615 fcc"]
    lines += block(pot.embed(rho))
    lines += block(pot.density(r))
    lines += block(r * pot.pair(r))
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")


def funcfl_to_setfl(src: str, dst: str, element: str = "Cu", lattice: str = "3.615 fcc") -> None:
    """Re-emit a funcfl-variant file as a one-element setfl file with the
    very same number strings (F, rho, r*phi), so both parse to identical
    tables on any host."""
    with open(src) as f:
        lines = f.read().splitlines()
    z_mass = lines[1].split()
    out = [lines[0], "setfl layout, one element", "converted from the funcfl file",
           f"1 {element}", lines[2], f"{z_mass[0]} {z_mass[1]} {lattice}"] + lines[3:]
    with open(dst, "w") as f:
        f.write("\n".join(out) + "\n")


def write_eam_funcfl(pot: AnalyticEAM, path: str, nrho: int = 2000, drho: Optional[float] = None,
                     nr: int = 2000, rho_max: Optional[float] = None,
                     r_max: Optional[float] = None) -> None:
    """Tabulate ``pot`` in the file variant PairEAM::read_file reads.

    Grid r = (m-1)*dr, m = 1..nr with (nr-1)*dr = r_max (default: the cutoff;
    file2array then regrids to nr-1 points, pair_eam.cpp:338-339, so the last
    interval below the cutoff is clamped unless r_max extends past it).  The
    third table holds r*phi(r) directly, as the reference uses it without the
    Z-product conversion (pair_eam.cpp:487).
    """
    dr = (pot.cut if r_max is None else r_max) / (nr - 1)
    r = np.arange(nr) * dr
    if rho_max is None:
        rho_max = 40.0
    if drho is None:
        drho = rho_max / (nrho - 1)
    rho = np.arange(nrho) * drho
    F = pot.embed(rho)
    f = pot.density(r)
    z = r * pot.pair(r)

    def block(vals):
        out = []
        for i in range(0, len(vals), 5):
            out.append(" ".join(f"{v:.16e}" for v in vals[i:i + 5]))
        return out

    lines = ["analytic EAM Cu: exp density, Morse pair, sqrt embedding (synthetic)"]
    lines.append(f"29 {pot.mass:.6f}")
    lines.append(f"{nrho} {drho:.16e} {nr} {dr:.16e} {pot.cut:.16e}")
    lines += block(F)
    lines += block(f)
    lines += block(z)
    with open(path, "w") as fh:
        fh.write("\n".join(lines) + "\n")


def wrap_elements(model: Model) -> None:
    """Shift whole elements by periods so that every centre lies in the periodic
    box (nodes move with their centre, as Domain::elepbc moves them)."""
    if not model.nelements:
        return
    c = model.element_centres()
    for d in range(3):
        if not model.periodic[d]:
            continue
        lo, hi = float(model.boxlo[d]), float(model.boxhi[d])
        prd = hi - lo
        k = np.floor((c[:, d] - lo) / prd)
        model.nodex[:, :, d] -= (k * prd)[:, None]


def remap_into_box(model: Model) -> None:
    """Wrap atom positions and element centres into the periodic box.

    Same arithmetic as Domain::remap (domain.cpp:389-476), which read_data applies
    to every Atoms and Elements line; element nodes are read unwrapped
    (element.cpp:478-540), so only centres move here.
    """
    def wrap(x: np.ndarray) -> None:
        # per coordinate: add the period while below lo, subtract it while at
        # or above hi, then clamp to lo (the same operations, element-wise)
        for d in range(3):
            if not model.periodic[d]:
                continue
            lo, hi = float(model.boxlo[d]), float(model.boxhi[d])
            prd = hi - lo
            col = x[:, d]
            while True:
                m = col < lo
                if not m.any():
                    break
                col[m] += prd
            while True:
                m = col >= hi
                if not m.any():
                    break
                col[m] -= prd
            np.maximum(col, lo, out=col)
    wrap(model.atom_x)
