"""ctypes front end of the CPU restatement (liboracle.so) and runner of the
reference harness (oracle/_ref/cacref).

TEST INFRASTRUCTURE ONLY: imported by tests/, tests/golden/make_golden.py and
the CPU-baseline leg of bench.py, never by the product package.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import tempfile
from typing import Sequence, Dict, Optional

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
REF_BIN = os.path.join(HERE, "_ref", "cacref")
# the reference tree: CAC_REFERENCE_TREE, else the directory "reference"
# beside the repository
REF_TREE = os.environ.get("CAC_REFERENCE_TREE",
                          os.path.normpath(os.path.join(HERE, "..", "..", "reference")))

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)


def build(ref: bool = False) -> None:
    """Compile liboracle.so (and, with ``ref``, the reference harness)."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    if ref:
        subprocess.run(["make", "-s", "-j8", "-C", HERE, "ref", f"REFDIR={REF_TREE}"], check=True)


def ref_available() -> bool:
    return os.path.exists(REF_BIN)


def _lib() -> ctypes.CDLL:
    if not os.path.exists(LIB_PATH):
        build()
    lib = ctypes.CDLL(LIB_PATH)
    lib.orc_create.restype = ctypes.c_void_p
    lib.orc_destroy.argtypes = [ctypes.c_void_p]
    lib.orc_error.restype = ctypes.c_char_p
    lib.orc_error.argtypes = [ctypes.c_void_p]
    lib.orc_size.restype = ctypes.c_longlong
    lib.orc_size.argtypes = [ctypes.c_void_p, ctypes.c_int]
    lib.orc_get_cut.restype = ctypes.c_double
    lib.orc_get_cut.argtypes = [ctypes.c_void_p, ctypes.c_int]
    lib.orc_set_timestep.argtypes = [ctypes.c_void_p, ctypes.c_double]
    lib.orc_set_neighbor.argtypes = [ctypes.c_void_p, ctypes.c_double, ctypes.c_int,
                                     ctypes.c_int, ctypes.c_int, ctypes.c_double]
    for name in ("orc_set_units", "orc_set_elementsplit", "orc_setup", "orc_atom_list",
                 "orc_elem_lists", "orc_atom_forces", "orc_elem_forces", "orc_run"):
        getattr(lib, name).argtypes = [ctypes.c_void_p, ctypes.c_int] if name in (
            "orc_set_units", "orc_set_elementsplit", "orc_run") else [ctypes.c_void_p]
    lib.orc_set_eam_file.argtypes = [ctypes.c_void_p, ctypes.c_char_p]
    return lib


_LIB: Optional[ctypes.CDLL] = None


def lib() -> ctypes.CDLL:
    global _LIB
    if _LIB is None:
        _LIB = _lib()
    return _LIB


def _d(a: np.ndarray):
    return a.ctypes.data_as(_dp)


def _i(a: np.ndarray):
    return a.ctypes.data_as(_ip)


class OracleError(RuntimeError):
    pass


class Oracle:
    """One CPU CAC system driven through the restated reference routines."""

    def __init__(self, model, *, units: str = "lj", skin: float, pair: str,
                 lj=(1.0, 1.0, 2.5), eam_file: Optional[str] = None, every: int = 1,
                 delay: int = 0, check: bool = True, binsize: float = 0.0,
                 nsplit: int = 2, dt: Optional[float] = None):
        L = lib()
        self._L = L
        self.h = ctypes.c_void_p(L.orc_create())
        self._ok(L.orc_set_units(self.h, 1 if units == "metal" else 0))
        if dt is not None:
            self._ok(L.orc_set_timestep(self.h, dt))
        lo = np.ascontiguousarray(model.boxlo, dtype=np.float64)
        hi = np.ascontiguousarray(model.boxhi, dtype=np.float64)
        per = np.array([1 if p else 0 for p in model.periodic], dtype=np.int32)
        self._ok(L.orc_set_box(self.h, _d(lo), _d(hi), _i(per)))
        self._ok(L.orc_set_neighbor(self.h, skin, every, delay, 1 if check else 0, binsize))
        self._ok(L.orc_set_elementsplit(self.h, nsplit))
        mass = np.array([model.mass], dtype=np.float64)
        self._ok(L.orc_set_atom_types(self.h, 1, _d(mass)))
        x = np.ascontiguousarray(model.atom_x, dtype=np.float64)
        v = np.ascontiguousarray(model.atom_v, dtype=np.float64)
        t = np.ones(model.natoms, dtype=np.int32)
        self._ok(L.orc_set_atoms(self.h, model.natoms, _d(x), _d(v), _i(t)))
        if model.nelements:
            nae = np.array([et.nae for et in model.etypes], dtype=np.int32).reshape(-1)
            numint = np.array([len(et.intp) for et in model.etypes], dtype=np.int32)
            intp = np.ascontiguousarray(np.concatenate([et.intp for et in model.etypes]),
                                        dtype=np.int32)
            w = np.ascontiguousarray(np.concatenate([et.weight for et in model.etypes]),
                                     dtype=np.float64)
            self._ok(L.orc_set_element_types(self.h, len(model.etypes), _i(nae), _i(numint),
                                             _i(intp), _d(w)))
            et = np.ascontiguousarray(model.elem_type, dtype=np.int32)
            c = np.ascontiguousarray(model.element_centres(), dtype=np.float64)
            nx = np.ascontiguousarray(model.nodex, dtype=np.float64)
            nv = np.ascontiguousarray(model.nodev, dtype=np.float64)
            self._ok(L.orc_set_elements(self.h, model.nelements, _i(et), _d(c), _d(nx), _d(nv)))
        if pair == "lj/cut":
            e = np.array([lj[0]]); s = np.array([lj[1]]); cc = np.array([lj[2]])
            self._ok(L.orc_set_lj(self.h, 1, _d(e), _d(s), _d(cc)))
        elif pair == "eam":
            self._ok(L.orc_set_eam_file(self.h, eam_file.encode()))
        else:
            raise ValueError(pair)

    def _ok(self, rc: int) -> None:
        if rc != 0:
            raise OracleError(self._L.orc_error(self.h).decode())

    def __del__(self):
        try:
            self._L.orc_destroy(self.h)
        except Exception:
            pass

    def size(self, what: int) -> int:
        return int(self._L.orc_size(self.h, what))

    def setup(self):
        self._ok(self._L.orc_setup(self.h))

    def atom_list(self):
        self._ok(self._L.orc_atom_list(self.h))
        nl = self.size(0)
        num = np.zeros(nl, dtype=np.int32)
        nb = np.zeros(self.size(2), dtype=np.int32)
        self._L.orc_get_atom_list(self.h, _i(num), _i(nb))
        return num, nb

    def elem_lists(self):
        self._ok(self._L.orc_elem_lists(self.h))
        ne = self.size(3)
        enum = np.zeros(ne, dtype=np.int32)
        eneigh = np.zeros(self.size(5), dtype=np.int32)
        self._L.orc_get_elem_list(self.h, _i(enum), _i(eneigh))
        ipn = np.zeros(self.size(6), dtype=np.int32)
        ipj = np.zeros(self.size(7), dtype=np.int32)
        ipnj = np.zeros(self.size(7), dtype=np.int32)
        self._L.orc_get_ip_list(self.h, _i(ipn), _i(ipj), _i(ipnj))
        return enum, eneigh, ipn, ipj, ipnj

    def atom_forces(self) -> np.ndarray:
        self._ok(self._L.orc_atom_forces(self.h))
        return self.atoms()["f"]

    def elem_forces(self) -> np.ndarray:
        self._ok(self._L.orc_elem_forces(self.h))
        return self.elements()["nodef"]

    def centro(self) -> np.ndarray:
        """Centro-symmetry of the local atoms (orc_centro)."""
        out = np.zeros(self.size(0))
        self._ok(self._L.orc_centro(self.h, _d(out)))
        return out

    def set_masks(self, amask=None, emask=None):
        a = None if amask is None else np.ascontiguousarray(amask, dtype=np.int32)
        e = None if emask is None else np.ascontiguousarray(emask, dtype=np.int32)
        self._ok(self._L.orc_set_masks(self.h, _i(a) if a is not None else None,
                                       _i(e) if e is not None else None))

    def add_setforce(self, bit: int, values):
        """values: three floats or None (NULL keeps the component)."""
        st = np.array([0 if v is None else 1 for v in values], dtype=np.int32)
        vals = np.array([0.0 if v is None else float(v) for v in values])
        self._ok(self._L.orc_add_setforce(self.h, bit, _i(st), _d(vals)))

    def set_deform(self, erate):
        e = np.ascontiguousarray(erate, dtype=np.float64)
        self._ok(self._L.orc_set_deform(self.h, _d(e)))

    def box(self):
        lo, hi = np.zeros(3), np.zeros(3)
        self._L.orc_get_box(self.h, _d(lo), _d(hi))
        return lo, hi

    def add_viscous(self, bit: int, gamma: float):
        self._ok(self._L.orc_add_viscous(self.h, bit, ctypes.c_double(gamma)))

    def thermo(self) -> Dict[str, object]:
        """Energies, virial and kinetic tensors at the current state (orc_thermo)."""
        out = np.zeros(17)
        self._ok(self._L.orc_thermo(self.h, _d(out)))
        return {"pe_atoms": out[0], "pe_elements": out[1], "ke_atoms": out[2],
                "ke_nodes": out[3], "virial": out[4:10].copy(), "kinetic_tensor": out[10:16].copy(),
                "volume": out[16], "etotal": out[0] + out[1] + out[2] + out[3]}

    def run(self, n: int):
        self._ok(self._L.orc_run(self.h, n))

    def atoms(self, all_: bool = False) -> Dict[str, np.ndarray]:
        nl = self.size(0)
        n = nl + (self.size(1) if all_ else 0)
        x = np.zeros((n, 3)); v = np.zeros((nl, 3)); f = np.zeros((nl, 3))
        tag = np.zeros(n, dtype=np.int32)
        self._L.orc_get_atoms(self.h, 1 if all_ else 0, _d(x), _d(v), _d(f), _i(tag))
        return {"x": x, "v": v, "f": f, "tag": tag}

    def elements(self, all_: bool = False) -> Dict[str, np.ndarray]:
        nl = self.size(3)
        n = nl + (self.size(4) if all_ else 0)
        c = np.zeros((n, 3)); nx = np.zeros((n, 8, 3))
        nv = np.zeros((nl, 8, 3)); nf = np.zeros((nl, 8, 3))
        tag = np.zeros(n, dtype=np.int32)
        self._L.orc_get_elements(self.h, 1 if all_ else 0, _d(c), _d(nx), _d(nv), _d(nf), _i(tag))
        return {"x": c, "nodex": nx, "nodev": nv, "nodef": nf, "tag": tag}

    def cuts(self) -> np.ndarray:
        return np.array([self._L.orc_get_cut(self.h, i) for i in range(6)])


# ---------------------------------------------------------------------------
# reference harness

def input_script(data_file: str, *, units: str, boundary: str, pair: str, skin: float,
                 lj=(1.0, 1.0, 2.5), eam_file: Optional[str] = None, every: int = 1,
                 delay: int = 0, check: bool = True, binsize: float = 0.0, nsplit: int = 2,
                 dt: Optional[float] = None, extra: Sequence[str] = ()) -> str:
    """Reference input-script commands for one configuration (input.cpp:362-404)."""
    lines = [f"units {units}", f"boundary {boundary}"]
    if nsplit != 2:
        lines.append(f"elementsplit {nsplit}")
    lines.append(f"read_data {data_file}")
    if pair == "lj/cut":
        lines += [f"pair_style lj/cut {lj[2]!r}", f"pair_coeff 1 1 {lj[0]!r} {lj[1]!r}"]
    else:
        lines += ["pair_style eam", f"pair_coeff 1 1 {eam_file}"]
    lines.append(f"neighbor {skin!r} bin")
    mod = f"neigh_modify every {every} delay {delay} check {'yes' if check else 'no'}"
    if binsize > 0:
        mod += f" binsize {binsize!r}"
    lines.append(mod)
    if dt is not None:
        lines.append(f"timestep {dt!r}")
    lines.append("fix 1 all nve")
    lines += list(extra)
    return "\n".join(lines) + "\n"


def run_reference(script: str, directives: str, workdir: Optional[str] = None,
                  timeout: float = 600.0) -> Dict[str, np.ndarray]:
    """Run the reference harness; return every dumped array keyed by file stem."""
    if not ref_available():
        raise FileNotFoundError(REF_BIN)
    wd = workdir or tempfile.mkdtemp(prefix="cacref_")
    out = os.path.join(wd, "out")
    os.makedirs(out, exist_ok=True)
    with open(os.path.join(wd, "in.cac"), "w") as f:
        f.write(script)
    with open(os.path.join(wd, "directives.txt"), "w") as f:
        f.write(directives)
    p = subprocess.run([REF_BIN, "in.cac", "directives.txt", "out"], cwd=wd,
                       capture_output=True, text=True, timeout=timeout)
    if p.returncode != 0:
        raise RuntimeError(f"cacref failed ({p.returncode}): {p.stdout[-2000:]} {p.stderr[-2000:]}")
    res = {}
    for name in os.listdir(out):
        stem, ext = os.path.splitext(name)
        dt = np.int32 if ext == ".i32" else np.float64
        res[stem] = np.fromfile(os.path.join(out, name), dtype=dt)
    return res
