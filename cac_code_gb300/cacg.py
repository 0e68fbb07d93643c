"""ctypes binding of libcacg.so (include/cacg.h) and a thin Python mirror of the
reference's objects for the CAC force path.

``System`` is one CAC system resident on one GPU.  Its methods are the
reference entry points the C ABI replaces:

================================  ==========================================
System method                     reference routine
================================  ==========================================
command / file                    Input::execute_command / Input::file
init / setup                      CAC::init / Verlet::setup (without its abort)
neighbor_build/ebuild/nbuild      Neighbor::build / ebuild / nbuild
pair_compute / pair_ecompute      Pair::compute / Pair::ecompute
fix_nve_initial/final             FixNVE::(e)initial_integrate / (e)final_integrate
run                               Verlet::run
================================  ==========================================

There is no CPU fallback: a missing library or GPU raises.
"""
from __future__ import annotations

import ctypes
import os
from typing import Dict, Optional

import numpy as np

from . import build as _build

FP64_EXACT, FP64, MIXED = 0, 1, 2
_STATUS = {0: "ok", -1: "invalid", -2: "state", -3: "cuda", -4: "overflow", -5: "io",
           -6: "nomem", -7: "timeout", -8: "scratch"}

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)
_lp = ctypes.POINTER(ctypes.c_longlong)
_fp = ctypes.POINTER(ctypes.c_float)

EXPORTED = [
    "cacg_create", "cacg_destroy", "cacg_error", "cacg_version", "cacg_command", "cacg_file",
    "cacg_set_box", "cacg_set_masses", "cacg_set_atoms", "cacg_set_element_types",
    "cacg_set_elements", "cacg_set_precision", "cacg_init", "cacg_setup",
    "cacg_neighbor_build", "cacg_neighbor_ebuild", "cacg_neighbor_nbuild",
    "cacg_pair_compute", "cacg_pair_ecompute", "cacg_fix_nve_initial_integrate",
    "cacg_fix_nve_final_integrate", "cacg_run", "cacg_get_counts", "cacg_get_atoms",
    "cacg_get_elements", "cacg_get_atom_list", "cacg_get_elem_list", "cacg_get_ip_list",
    "cacg_get_cut", "cacg_set_timing", "cacg_get_timing", "cacg_measure_fp64_peak",
    "cacg_put_atoms", "cacg_put_nodes", "cacg_compute_thermo", "cacg_kinetic_noalloc",
    "cacg_mlp_create", "cacg_mlp_destroy", "cacg_mlp_error", "cacg_mlp_sizes",
    "cacg_mlp_get_params", "cacg_mlp_set_params", "cacg_mlp_set_normalization",
    "cacg_mlp_get_normalization", "cacg_mlp_loss_grad", "cacg_mlp_train", "cacg_mlp_predict",
    "cacg_gemm_bf16_tn", "cacg_surrogate_reference", "cacg_surrogate_samples",
    "cacg_surrogate_attach", "cacg_compute_centro", "cacg_dump_xyz", "cacg_dump_elements",
    "cacg_fix_post_force", "cacg_get_box", "cacg_set_graphs", "cacg_set_group",
    "cacg_run_host", "cacg_get_kernel_timing", "cacg_set_lj", "cacg_set_eam",
    "cacg_run_batch",
]


class CacgError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"[{_STATUS.get(status, status)}] {msg}")
        self.status = status


_LIB: Optional[ctypes.CDLL] = None


def load(build_if_missing: bool = False) -> ctypes.CDLL:
    """Load libcacg.so from the package directory (built in-tree)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    if not os.path.exists(_build.LIB):
        if not build_if_missing:
            raise FileNotFoundError(
                f"{_build.LIB} is missing: run cac_code_gb300.build.build_library() first")
        _build.build_library()
    lib = ctypes.CDLL(_build.LIB)
    lib.cacg_error.restype = ctypes.c_char_p
    lib.cacg_error.argtypes = [ctypes.c_void_p]
    lib.cacg_version.restype = ctypes.c_char_p
    lib.cacg_create.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.c_int]
    for name in ("cacg_destroy", "cacg_init", "cacg_setup", "cacg_neighbor_build",
                 "cacg_fix_post_force",
                 "cacg_neighbor_ebuild", "cacg_neighbor_nbuild", "cacg_pair_ecompute",
                 "cacg_fix_nve_initial_integrate", "cacg_fix_nve_final_integrate"):
        getattr(lib, name).argtypes = [ctypes.c_void_p]
    lib.cacg_command.argtypes = [ctypes.c_void_p, ctypes.c_char_p]
    lib.cacg_file.argtypes = [ctypes.c_void_p, ctypes.c_char_p]
    lib.cacg_run.argtypes = [ctypes.c_void_p, ctypes.c_int]
    lib.cacg_run_batch.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.c_int, ctypes.c_int]
    lib.cacg_run_host.argtypes = [ctypes.c_void_p, ctypes.c_int, _dp, _dp, _dp, _dp]
    lib.cacg_set_precision.argtypes = [ctypes.c_void_p, ctypes.c_int]
    lib.cacg_set_timing.argtypes = [ctypes.c_void_p, ctypes.c_int]
    lib.cacg_set_graphs.argtypes = [ctypes.c_void_p, ctypes.c_int]
    lib.cacg_set_group.argtypes = [ctypes.c_void_p, ctypes.c_char_p, _ip, _ip]
    lib.cacg_pair_compute.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int]
    lib.cacg_get_cut.argtypes = [ctypes.c_void_p, ctypes.c_int, _dp]
    lib.cacg_kinetic_noalloc.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                         ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                         ctypes.c_double, ctypes.c_void_p, ctypes.c_void_p]
    vp, i, d, f = ctypes.c_void_p, ctypes.c_int, ctypes.c_double, ctypes.c_float
    lib.cacg_mlp_create.argtypes = [ctypes.POINTER(vp), i, i, ctypes.c_ulonglong]
    lib.cacg_mlp_destroy.argtypes = [vp]
    lib.cacg_mlp_error.restype = ctypes.c_char_p
    lib.cacg_mlp_error.argtypes = [vp]
    lib.cacg_mlp_sizes.argtypes = [vp, _lp, i]
    lib.cacg_mlp_get_params.argtypes = [vp, i, _fp]
    lib.cacg_mlp_set_params.argtypes = [vp, i, _fp]
    lib.cacg_mlp_set_normalization.argtypes = [vp, _fp, _fp, _fp, _fp, d]
    lib.cacg_mlp_get_normalization.argtypes = [vp, _fp, _fp, _fp, _fp, _dp]
    lib.cacg_mlp_loss_grad.argtypes = [vp, i, _fp, _fp, i, _dp, _fp]
    lib.cacg_mlp_train.argtypes = [vp, _fp, _fp, ctypes.c_longlong, i, i, f, ctypes.c_ulonglong,
                                   _dp]
    lib.cacg_mlp_predict.argtypes = [vp, _fp, ctypes.c_longlong, _fp, _fp]
    lib.cacg_gemm_bf16_tn.argtypes = [vp, i, vp, i, vp, i, i, i, i, vp, vp]
    lib.cacg_surrogate_reference.argtypes = [vp, _dp]
    lib.cacg_surrogate_samples.argtypes = [vp, _fp, _fp, i]
    lib.cacg_surrogate_attach.argtypes = [vp, vp, d, d]
    lib.cacg_compute_centro.argtypes = [vp, _dp, i]
    lib.cacg_get_box.argtypes = [vp, _dp, _dp]
    lib.cacg_dump_xyz.argtypes = [vp, ctypes.c_char_p]
    lib.cacg_dump_elements.argtypes = [vp, ctypes.c_char_p, i]
    _LIB = lib
    return lib


def _d(a):
    return a.ctypes.data_as(_dp) if a is not None else None


def _i(a):
    return a.ctypes.data_as(_ip) if a is not None else None


def _f(a):
    return a.ctypes.data_as(_fp) if a is not None else None


class Mlp:
    """The nodal-force surrogate ensemble (cacg_mlp_*): host arrays in and out."""

    def __init__(self, device: int = 0, members: int = 4, seed: int = 1):
        self._L = load()
        self.h = ctypes.c_void_p()
        rc = self._L.cacg_mlp_create(ctypes.byref(self.h), device, members, seed)
        if rc != 0:
            raise CacgError(rc, "cacg_mlp_create failed (no CUDA device visible?)")
        sz = np.zeros(6, dtype=np.int64)
        self._ok(self._L.cacg_mlp_sizes(self.h, sz.ctypes.data_as(_lp), 6))
        self.members, self.nparam, self.nin, self.nout, self.hidden = (int(v) for v in sz[:5])

    def _ok(self, rc: int):
        if rc != 0:
            raise CacgError(rc, self._L.cacg_mlp_error(self.h).decode())

    def close(self):
        if self.h:
            self._L.cacg_mlp_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def params(self, member: int) -> np.ndarray:
        p = np.zeros(self.nparam, dtype=np.float32)
        self._ok(self._L.cacg_mlp_get_params(self.h, member, _f(p)))
        return p

    def set_params(self, member: int, p: np.ndarray):
        p = np.ascontiguousarray(p, dtype=np.float32)
        self._ok(self._L.cacg_mlp_set_params(self.h, member, _f(p)))

    def set_normalization(self, in_mean, in_std, out_mean, out_std, force_scale: float):
        a = [np.ascontiguousarray(v, dtype=np.float32) for v in (in_mean, in_std, out_mean, out_std)]
        self._ok(self._L.cacg_mlp_set_normalization(self.h, *(_f(v) for v in a), float(force_scale)))

    def fit_normalization(self, x: np.ndarray, t: np.ndarray):
        """Standardise inputs and outputs on a training set; force scale = rms
        per-element nodal-force norm."""
        sd = x.std(axis=0)
        osd = t.std(axis=0)
        fs = float(np.sqrt((t.astype(np.float64) ** 2).sum(axis=1).mean() / 8.0))
        self.set_normalization(x.mean(axis=0), np.where(sd > 0, sd, 1.0), t.mean(axis=0),
                               np.where(osd > 0, osd, 1.0), max(fs, 1e-30))

    def normalization(self):
        im, isd = np.zeros(self.nin, np.float32), np.zeros(self.nin, np.float32)
        om, osd = np.zeros(self.nout, np.float32), np.zeros(self.nout, np.float32)
        fs = np.zeros(1)
        self._ok(self._L.cacg_mlp_get_normalization(self.h, _f(im), _f(isd), _f(om), _f(osd),
                                                     _d(fs)))
        return im, isd, om, osd, float(fs[0])

    def loss_grad(self, member: int, x: np.ndarray, t: np.ndarray):
        x = np.ascontiguousarray(x, dtype=np.float32)
        t = np.ascontiguousarray(t, dtype=np.float32)
        loss = np.zeros(1)
        g = np.zeros(self.nparam, dtype=np.float32)
        self._ok(self._L.cacg_mlp_loss_grad(self.h, member, _f(x), _f(t), x.shape[0], _d(loss), _f(g)))
        return float(loss[0]), g

    def train(self, x: np.ndarray, t: np.ndarray, epochs: int, batch: int = 1024,
              lr: float = 1e-3, seed: int = 7) -> float:
        x = np.ascontiguousarray(x, dtype=np.float32)
        t = np.ascontiguousarray(t, dtype=np.float32)
        loss = np.zeros(1)
        self._ok(self._L.cacg_mlp_train(self.h, _f(x), _f(t), x.shape[0], epochs, batch, lr, seed,
                                        _d(loss)))
        return float(loss[0])

    def predict(self, x: np.ndarray):
        x = np.ascontiguousarray(x, dtype=np.float32)
        n = x.shape[0]
        mean = np.zeros((n, self.nout), dtype=np.float32)
        spread = np.zeros(n, dtype=np.float32)
        self._ok(self._L.cacg_mlp_predict(self.h, _f(x), n, _f(mean), _f(spread)))
        return mean, spread


class System:
    """One CAC system on one GPU, driven through the C ABI."""

    def __init__(self, device: int = 0):
        self._L = load()
        h = ctypes.c_void_p()
        rc = self._L.cacg_create(ctypes.byref(h), device)
        if rc != 0:
            raise CacgError(rc, "cacg_create failed (no CUDA device visible?)")
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self._L.cacg_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _ok(self, rc: int):
        if rc != 0:
            raise CacgError(rc, self._L.cacg_error(self.h).decode())

    # ---- input ----
    def command(self, line: str):
        self._ok(self._L.cacg_command(self.h, line.encode()))

    def commands(self, text: str):
        for line in text.splitlines():
            self.command(line)

    def file(self, path: str):
        self._ok(self._L.cacg_file(self.h, path.encode()))

    def set_precision(self, mode: int):
        self._ok(self._L.cacg_set_precision(self.h, mode))

    # ---- direct state ----
    def set_lj(self, lj1, lj2, cutsq):
        """PairLJCut tables after init_one, [ntypes + 1][ntypes + 1] each."""
        a = [np.ascontiguousarray(t, dtype=np.float64) for t in (lj1, lj2, cutsq)]
        nt = int(round(np.sqrt(a[0].size))) - 1
        self._ok(self._L.cacg_set_lj(self.h, nt, _d(a[0]), _d(a[1]), _d(a[2])))

    def set_eam(self, nr, dr, nrho, drho, frho7, rhor7, z2r7, cutforcesq, mass):
        """PairEAM splines of the one species ([n + 1][7] each) and grids."""
        f, r, z = (np.ascontiguousarray(t, dtype=np.float64) for t in (frho7, rhor7, z2r7))
        L = self._L
        L.cacg_set_eam.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_double, ctypes.c_int,
                                   ctypes.c_double, _dp, _dp, _dp, ctypes.c_double, ctypes.c_double]
        self._ok(L.cacg_set_eam(self.h, int(nr), float(dr), int(nrho), float(drho), _d(f), _d(r),
                                _d(z), float(cutforcesq), float(mass)))

    def set_box(self, lo, hi, periodic):
        lo = np.ascontiguousarray(lo, dtype=np.float64)
        hi = np.ascontiguousarray(hi, dtype=np.float64)
        per = np.ascontiguousarray([1 if p else 0 for p in periodic], dtype=np.int32)
        self._ok(self._L.cacg_set_box(self.h, _d(lo), _d(hi), _i(per)))

    def set_masses(self, mass):
        m = np.ascontiguousarray(mass, dtype=np.float64)
        self._ok(self._L.cacg_set_masses(self.h, len(m), _d(m)))

    def set_atoms(self, x, v=None, type_=None):
        x = np.ascontiguousarray(x, dtype=np.float64).reshape(-1, 3)
        v = None if v is None else np.ascontiguousarray(v, dtype=np.float64).reshape(-1, 3)
        t = None if type_ is None else np.ascontiguousarray(type_, dtype=np.int32)
        self._ok(self._L.cacg_set_atoms(self.h, x.shape[0], _d(x), _d(v), _i(t)))

    def set_element_types(self, etypes):
        nae = np.ascontiguousarray([et.nae for et in etypes], dtype=np.int32).reshape(-1)
        numint = np.ascontiguousarray([len(et.intp) for et in etypes], dtype=np.int32)
        intp = np.ascontiguousarray(np.concatenate([et.intp for et in etypes]), dtype=np.int32)
        w = np.ascontiguousarray(np.concatenate([et.weight for et in etypes]), dtype=np.float64)
        self._ok(self._L.cacg_set_element_types(self.h, len(etypes), _i(nae), _i(numint),
                                                _i(intp), _d(w)))

    def set_elements(self, etype, centre, nodex, nodev=None):
        et = np.ascontiguousarray(etype, dtype=np.int32)
        c = np.ascontiguousarray(centre, dtype=np.float64)
        nx = np.ascontiguousarray(nodex, dtype=np.float64)
        nv = None if nodev is None else np.ascontiguousarray(nodev, dtype=np.float64)
        self._ok(self._L.cacg_set_elements(self.h, len(et), _i(et), _d(c), _d(nx), _d(nv)))

    def load_model(self, model):
        """Upload a lattice.Model (the same data read_data would deliver)."""
        self.set_box(model.boxlo, model.boxhi, model.periodic)
        self.set_masses([model.mass])
        self.set_atoms(model.atom_x, model.atom_v, np.ones(model.natoms, dtype=np.int32))
        if model.nelements:
            self.set_element_types(model.etypes)
            self.set_elements(model.elem_type, model.element_centres(), model.nodex, model.nodev)

    # ---- path ----
    def init(self):
        self._ok(self._L.cacg_init(self.h))

    def setup(self):
        self._ok(self._L.cacg_setup(self.h))

    def neighbor_build(self):
        self._ok(self._L.cacg_neighbor_build(self.h))

    def neighbor_ebuild(self):
        self._ok(self._L.cacg_neighbor_ebuild(self.h))

    def neighbor_nbuild(self):
        self._ok(self._L.cacg_neighbor_nbuild(self.h))

    def pair_compute(self, eflag: int = 0, vflag: int = 0):
        self._ok(self._L.cacg_pair_compute(self.h, eflag, vflag))

    def pair_ecompute(self):
        self._ok(self._L.cacg_pair_ecompute(self.h))

    def fix_nve_initial_integrate(self):
        self._ok(self._L.cacg_fix_nve_initial_integrate(self.h))

    def fix_nve_final_integrate(self):
        self._ok(self._L.cacg_fix_nve_final_integrate(self.h))

    def run(self, n: int):
        self._ok(self._L.cacg_run(self.h, n))

    def run_host(self, n: int, x, v, nodex, nodev):
        """Advance host-resident state n steps: x, v (float64 [nlocal][3]) and
        nodex, nodev (float64 [enlocal][8][3]), C order, updated in place."""
        for a, tail in ((x, (3,)), (v, (3,)), (nodex, (8, 3)), (nodev, (8, 3))):
            if (a.dtype != np.float64 or a.shape[1:] != tail or not a.flags["C_CONTIGUOUS"]
                    or not a.flags["WRITEABLE"]):
                raise ValueError("run_host wants writeable float64 C-ordered arrays "
                                 "[nlocal][3] and [enlocal][8][3]")
        if x.shape != v.shape or nodex.shape != nodev.shape:
            raise ValueError("run_host: x, v (and nodex, nodev) differ in shape")
        self._ok(self._L.cacg_run_host(self.h, n, _d(x), _d(v), _d(nodex), _d(nodev)))

    # ---- state out ----
    def counts(self) -> Dict[str, int]:
        c = np.zeros(31, dtype=np.int64)
        self._ok(self._L.cacg_get_counts(self.h, c.ctypes.data_as(_lp), 31))
        keys = ["nlocal", "nghost", "atom_entries", "enlocal", "enghost", "elem_entries",
                "ip_rows", "ip_entries", "rebuilds", "nstencil", "step", "sites", "launches",
                "sites_needed", "force_rows", "short_entries", "surrogate_elements",
                "surrogate_evaluated", "surrogate_accepted", "graph_steps", "density_scan_entries",
                "ip_scan_entries", "ip_reorders", "rebuilds_atoms_only", "atom_reorders",
                "lines_referenced", "lines_referenced_force", "elem_fused",
                "loop_launches", "host_decisions", "band_reruns"]
        return dict(zip(keys, (int(v) for v in c)))

    def referenced_lines(self):
        """Lattice lines with a site in some integration-point list, and those
        with a site in a list of a row of nonzero weight."""
        c = self.counts()
        return c["lines_referenced"], c["lines_referenced_force"]

    def atoms(self, all_: bool = False) -> Dict[str, np.ndarray]:
        c = self.counts()
        nl = c["nlocal"]
        n = nl + (c["nghost"] if all_ else 0)
        x = np.zeros((n, 3)); v = np.zeros((nl, 3)); f = np.zeros((nl, 3))
        tag = np.zeros(n, dtype=np.int32)
        self._ok(self._L.cacg_get_atoms(self.h, 1 if all_ else 0, _d(x), _d(v), _d(f), _i(tag)))
        return {"x": x, "v": v, "f": f, "tag": tag}

    def elements(self, all_: bool = False) -> Dict[str, np.ndarray]:
        c = self.counts()
        nl = c["enlocal"]
        n = nl + (c["enghost"] if all_ else 0)
        cx = np.zeros((n, 3)); nx = np.zeros((n, 8, 3))
        nv = np.zeros((nl, 8, 3)); nf = np.zeros((nl, 8, 3))
        tag = np.zeros(n, dtype=np.int32)
        self._ok(self._L.cacg_get_elements(self.h, 1 if all_ else 0, _d(cx), _d(nx), _d(nv),
                                           _d(nf), _i(tag)))
        return {"x": cx, "nodex": nx, "nodev": nv, "nodef": nf, "tag": tag}

    def atom_list(self):
        c = self.counts()
        num = np.zeros(c["nlocal"], dtype=np.int32)
        nb = np.zeros(max(c["atom_entries"], 1), dtype=np.int32)
        self._ok(self._L.cacg_get_atom_list(self.h, _i(num), _i(nb)))
        return num, nb[:c["atom_entries"]]

    def elem_lists(self):
        c = self.counts()
        enum = np.zeros(c["enlocal"], dtype=np.int32)
        eneigh = np.zeros(max(c["elem_entries"], 1), dtype=np.int32)
        self._ok(self._L.cacg_get_elem_list(self.h, _i(enum), _i(eneigh)))
        ipn = np.zeros(c["ip_rows"], dtype=np.int32)
        ipj = np.zeros(max(c["ip_entries"], 1), dtype=np.int32)
        ipnj = np.zeros(max(c["ip_entries"], 1), dtype=np.int32)
        self._ok(self._L.cacg_get_ip_list(self.h, _i(ipn), _i(ipj), _i(ipnj)))
        return enum, eneigh[:c["elem_entries"]], ipn, ipj[:c["ip_entries"]], ipnj[:c["ip_entries"]]

    def cut(self, what: int) -> float:
        v = ctypes.c_double()
        self._ok(self._L.cacg_get_cut(self.h, what, ctypes.byref(v)))
        return v.value

    def cuts(self) -> np.ndarray:
        return np.array([self.cut(i) for i in range(6)])

    def thermo(self) -> Dict[str, object]:
        """Energies (pe/ke of atoms and elements), virial and kinetic tensors, volume."""
        out = np.zeros(17)
        self._ok(self._L.cacg_compute_thermo(self.h, _d(out), 17))
        return {"pe_atoms": out[0], "pe_elements": out[1], "ke_atoms": out[2],
                "ke_nodes": out[3], "virial": out[4:10].copy(), "kinetic_tensor": out[10:16].copy(),
                "volume": out[16], "etotal": out[0] + out[1] + out[2] + out[3]}

    def box(self):
        lo, hi = np.zeros(3), np.zeros(3)
        self._ok(self._L.cacg_get_box(self.h, _d(lo), _d(hi)))
        return lo, hi

    def fix_post_force(self):
        self._ok(self._L.cacg_fix_post_force(self.h))

    def centro(self) -> np.ndarray:
        """Centro-symmetry of the local atoms (Output::centro_atom)."""
        n = self.counts()["nlocal"]
        out = np.zeros(n)
        self._ok(self._L.cacg_compute_centro(self.h, _d(out), n))
        return out

    def dump_xyz(self, path: str):
        self._ok(self._L.cacg_dump_xyz(self.h, path.encode()))

    def dump_elements(self, path: str, append: bool = False):
        self._ok(self._L.cacg_dump_elements(self.h, path.encode(), 1 if append else 0))

    def surrogate_reference(self, nodex0=None):
        a = None if nodex0 is None else np.ascontiguousarray(nodex0, dtype=np.float64)
        self._ok(self._L.cacg_surrogate_reference(self.h, _d(a)))

    def surrogate_samples(self):
        n = self.counts()["enlocal"]
        x = np.zeros((n, 32), dtype=np.float32)
        t = np.zeros((n, 24), dtype=np.float32)
        self._ok(self._L.cacg_surrogate_samples(self.h, _f(x), _f(t), n))
        return x, t

    def surrogate_attach(self, mlp: Optional["Mlp"], tol: float = 1e-4, dist: float = 11.0):
        self._ok(self._L.cacg_surrogate_attach(self.h, mlp.h if mlp is not None else None,
                                               float(tol), float(dist)))

    def set_group(self, name: str, atom_in=None, elem_in=None):
        a = None if atom_in is None else np.ascontiguousarray(atom_in, dtype=np.int32)
        e = None if elem_in is None else np.ascontiguousarray(elem_in, dtype=np.int32)
        self._ok(self._L.cacg_set_group(self.h, name.encode(), _i(a), _i(e)))

    def set_graphs(self, enable: bool = True):
        self._ok(self._L.cacg_set_graphs(self.h, 1 if enable else 0))

    def set_timing(self, enable: bool = True):
        self._ok(self._L.cacg_set_timing(self.h, 1 if enable else 0))

    def timing(self) -> np.ndarray:
        """[total, integrate+comm/rebuild, atom pass 1, atom pass 2, element, final,
        EAM atom density kernel alone] in ms (all but the total: eager steps with
        timing on)"""
        ms = np.zeros(8)
        self._ok(self._L.cacg_get_timing(self.h, _d(ms), 8))
        return ms[:7]

    def kernel_timing(self) -> np.ndarray:
        """Device ms of the main kernels of the last run with timing on (eager
        steps): [atom pass 1, atom pass 2, element density, element force,
        surrogate, sites/lines, atom-list reorder, element row preparation,
        site F'], then the device ms of every rebuild since creation."""
        ms = np.zeros(10)
        self._ok(self._L.cacg_get_kernel_timing(self.h, _d(ms), 10))
        return ms

    def put_atoms(self, x, v):
        """Push host-owned owned-atom x, v (float64 [nlocal][3], C order)."""
        self._ok(self._L.cacg_put_atoms(self.h, _d(x), _d(v)))

    def put_nodes(self, nodex, nodev):
        self._ok(self._L.cacg_put_nodes(self.h, _d(nodex), _d(nodev)))

    def get_state_into(self, x, v, f):
        """Read owned-atom x, v, f into caller-provided float64 [nlocal][3] buffers
        (any of them None: not read)."""
        self._ok(self._L.cacg_get_atoms(self.h, 0, _d(x), _d(v), _d(f), None))

    def get_nodes_into(self, nodex, nodev):
        """Read owned-element node x, v into caller-provided float64
        [enlocal][8][3] buffers (either None: not read)."""
        self._ok(self._L.cacg_get_elements(self.h, 0, None, _d(nodex), _d(nodev), None, None))

    def fp64_peak(self) -> float:
        v = ctypes.c_double()
        self._ok(self._L.cacg_measure_fp64_peak(self.h, ctypes.byref(v)))
        return v.value


def run_batch(systems, n: int) -> None:
    """n steps on every System of `systems` (one device, "tune loop device")
    as the branches of one CUDA graph (cacg_run_batch); a failure raises the
    error of the handle that met it."""
    if not systems:
        return
    L = systems[0]._L
    arr = (ctypes.c_void_p * len(systems))(*[s.h.value for s in systems])
    rc = L.cacg_run_batch(arr, len(systems), n)
    if rc != 0:
        for s in systems:
            msg = L.cacg_error(s.h).decode()
            if msg:
                raise CacgError(rc, msg)
        raise CacgError(rc, "cacg_run_batch failed")
