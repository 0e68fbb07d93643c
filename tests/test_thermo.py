"""Energy, virial and kinetic energy: the oracle's restatement checked against
its own forces (finite differences, homogeneous strain, NVE conservation), and
the device path (cacg_compute_thermo) against the oracle."""
import copy

import numpy as np
import pytest

import cases as C


def _oracle(O, cfg, m, eam_file=C.EAM_FILE):
    o = O.Oracle(m, **C.settings_kwargs(cfg, eam_file))
    am, em, fixes = C.fix_setup(cfg, m)
    if fixes:
        o.set_masks(am, em)
        for kind, bit, arg in fixes:
            (o.add_setforce if kind == "setforce" else o.add_viscous)(bit, arg)
    o.setup()
    if m.natoms:
        o.atom_list()
    if m.nelements:
        o.elem_lists()
    return o


def _pe(O, cfg, m, eam_file=C.EAM_FILE):
    t = _oracle(O, cfg, m, eam_file).thermo()
    return t["pe_atoms"] + t["pe_elements"]


def _smooth_atoms(cfg, m, count=4):
    """Atoms none of whose pairs fall in the last r interval of the EAM tables.

    The reference regrids a funcfl file to nr = nr_file - 1 knots and clamps
    the spline index at nr - 1 (pair_eam.cpp:332-339, 651), so its tables end
    one interval short of the cutoff: a pair in that interval sees a constant
    energy but a nonzero force, and there the force is not the gradient.
    """
    if cfg["pair"] != "eam":
        return [0, 7, m.natoms // 2, m.natoms - 1][:count]
    with open(C.EAM_FILE) as fh:
        fh.readline(); fh.readline()
        _, _, nr, dr, cut = fh.readline().split()
    r_end = (int(nr) - 2) * float(dr)
    prd = m.boxhi - m.boxlo
    out = []
    for i in range(m.natoms):
        d = m.atom_x - m.atom_x[i]
        d -= prd * np.round(d / prd)
        r = np.linalg.norm(d, axis=1)
        if not np.any((r > r_end - 1e-3) & (r < float(cut) + 1e-3)):
            out.append(i)
        if len(out) == count:
            break
    return out


@pytest.mark.parametrize("name", ["lj_atoms", "eam_atoms"])
def test_oracle_energy_gradient_is_force(oracle_lib, name):
    cfg = C.CASES[name]
    m = C.build_model(cfg)
    f = _oracle(oracle_lib, cfg, m).atom_forces()
    h = 1e-5
    for i in _smooth_atoms(cfg, m):
        for d in range(3):
            mp, mm = copy.deepcopy(m), copy.deepcopy(m)
            mp.atom_x[i, d] += h
            mm.atom_x[i, d] -= h
            g = -(_pe(oracle_lib, cfg, mp) - _pe(oracle_lib, cfg, mm)) / (2 * h)
            assert abs(g - f[i, d]) <= 1e-5 * max(1.0, np.abs(f).max()), (i, d, g, f[i, d])


@pytest.mark.parametrize("name", ["lj_atoms", "eam_atoms"])
def test_oracle_virial_is_strain_derivative(oracle_lib, name, tmp_path):
    # W_aa = -dE/d(eps_aa) under x_a -> (1 + eps) x_a of positions and box.
    # The EAM tables here extend past the cutoff so that no pair sees the
    # clamped last interval (see _smooth_atoms).
    cfg = C.CASES[name]
    m = C.build_model(cfg)
    ef = _wide_eam(tmp_path)
    w = _oracle(oracle_lib, cfg, m, ef).thermo()["virial"]
    eps = 1e-6
    for d in range(3):
        es = []
        for sgn in (1, -1):
            ms = copy.deepcopy(m)
            s = 1 + sgn * eps
            ms.atom_x[:, d] = ms.boxlo[d] + (ms.atom_x[:, d] - ms.boxlo[d]) * s
            ms.boxhi = np.array(ms.boxhi, dtype=float)
            ms.boxhi[d] = ms.boxlo[d] + (ms.boxhi[d] - ms.boxlo[d]) * s
            es.append(_pe(oracle_lib, cfg, ms, ef))
        dE = (es[0] - es[1]) / (2 * eps)
        assert abs(-dE - w[d]) <= 1e-5 * np.abs(w[:3]).max(), (d, -dE, w[d])


def test_oracle_kinetic_energy(oracle_lib):
    cfg = C.CASES["eam_cac"]
    m = C.build_model(cfg)
    t = _oracle(oracle_lib, cfg, m).thermo()
    mv = C.MVV2E[cfg["units"]]
    ke_a = 0.5 * mv * m.mass * np.sum(m.atom_v ** 2)
    ke_n = 0.5 * mv * (np.prod(m.etypes[0].nae) * m.mass / 8) * np.sum(m.nodev ** 2)
    assert t["ke_atoms"] == pytest.approx(ke_a, rel=1e-13)
    assert t["ke_nodes"] == pytest.approx(ke_n, rel=1e-13)
    assert np.sum(t["kinetic_tensor"][:3]) == pytest.approx(2 * (ke_a + ke_n), rel=1e-13)


def _wide_eam(tmp_path, taper=0.0):
    from cac_code_gb300 import lattice as L
    ef = str(tmp_path / f"Cu_wide{taper}.eam")
    pot = L.AnalyticEAM(taper=taper)
    L.write_eam_funcfl(pot, ef, nrho=800, nr=800, r_max=pot.cut * 1.01)
    return ef


def test_oracle_nve_conserves_energy(oracle_lib, tmp_path):
    # a potential that vanishes smoothly at the cutoff (no energy jumps when
    # pairs cross it): velocity Verlet keeps the total within O(dt^2)
    ef = _wide_eam(tmp_path, taper=1.0)
    spread = []
    for dt, n in ((0.001, 20), (0.0005, 40)):
        cfg = dict(C.CASES["eam_atoms"], dt=dt)
        m = C.build_model(cfg)
        o = _oracle(oracle_lib, cfg, m, ef)
        o.atom_forces()
        es = []
        for _ in range(n):
            es.append(o.thermo()["etotal"])
            o.run(1)
            o.atom_list()
        ke = o.thermo()["ke_atoms"]
        spread.append(max(es) - min(es))
        assert spread[-1] <= 2e-4 * ke, (dt, spread[-1], ke)
    assert spread[0] / spread[1] > 3.0, spread  # second order in dt


# ---------------------------------------------------------------- device

def _close(g, r, what):
    for k in ("pe_atoms", "pe_elements", "ke_atoms", "ke_nodes", "volume"):
        assert abs(g[k] - r[k]) <= 1e-12 * max(1.0, abs(r[k])), (what, k, g[k], r[k])
    for k in ("virial", "kinetic_tensor"):
        sc = max(1.0, np.abs(r[k]).max())
        assert np.abs(g[k] - r[k]).max() <= 1e-12 * sc, (what, k, g[k], r[k])


@pytest.mark.gpu
@pytest.mark.parametrize("name", list(C.CASES))
def test_gpu_thermo_matches_oracle(oracle_lib, cacg_lib, name):
    from gpu_runner import configure
    cfg = C.CASES[name]
    cfg_, z = C.load_golden(name)
    m = C.model_from_arrays(z)
    o = _oracle(oracle_lib, cfg_, m)
    s = cacg_lib.System(0)
    try:
        configure(s, cfg_, m)
        s.set_precision(cacg_lib.FP64_EXACT)
        s.init()
        s.setup()
        if m.natoms:
            s.neighbor_build()
        if m.nelements:
            s.neighbor_ebuild()
            s.neighbor_nbuild()
        _close(s.thermo(), o.thermo(), "setup")
        steps = cfg["steps"]
        s.run(steps)
        o.run(steps)
        if m.natoms:
            o.atom_list()
        if m.nelements:
            o.elem_lists()
        _close(s.thermo(), o.thermo(), "after run")
    finally:
        s.close()
