"""Generate the golden fixtures from the UNMODIFIED reference.

Runs the reference CAC sources (compiled by ``make -C oracle ref`` into
oracle/_ref/cacref) through the oracle harness for every case in
tests/cases.py and stores inputs and outputs in tests/golden/<case>.npz:

* inputs: box, masses, atom positions/velocities, element tables, nodes;
* atom list, element list and integration-point list as the reference numbers
  them (local+ghost indices, with the ghost positions and tags to map them);
* atom forces, nodal forces and cutoffs after setup;
* positions, velocities and forces after ``steps`` Verlet steps.

Run from the repository root in a container that has the reference tree:
    python tests/golden/make_golden.py
"""
from __future__ import annotations

import json
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

from cac_code_gb300 import lattice as L  # noqa: E402
from oracle import oracle as O  # noqa: E402
import cases as C  # noqa: E402


def make_eam_file() -> None:
    # small enough to commit, same analytic potential and cutoff as the
    # benchmark tables (nr = nrho = 2000 there)
    L.write_eam_funcfl(L.AnalyticEAM(), C.EAM_FILE, nrho=800, nr=800)


def run_case(name: str, cfg: dict) -> None:
    m = C.build_model(cfg)
    wd = tempfile.mkdtemp(prefix=f"golden_{name}_")
    L.write_data(m, os.path.join(wd, "data.cac"), with_velocities=True)
    m.atom_v.astype(np.float64).tofile(os.path.join(wd, "v.bin"))
    kw = C.settings_kwargs(cfg)
    script = O.input_script("data.cac", boundary=cfg["boundary"], extra=C.fix_lines(cfg, m),
                            **kw)
    cap = 8 * (m.natoms + 64)
    directives = [f"capacity {cap}", "velocities v.bin", "setup"]
    # the reference's own pair tables after init (raw-table hand-over tests)
    directives.append("eam_tables" if cfg["pair"] == "eam" else "lj_tables")
    if m.natoms:
        directives += ["atom_list", "centro", "atom_forces"]
    if m.nelements:
        directives += ["elem_lists", "elem_forces"]
    directives += [f"step {cfg['steps']}", "state s1"]
    ref = O.run_reference(script, "\n".join(directives) + "\n", wd)
    out = C.model_to_arrays(m)
    out["settings"] = np.array(json.dumps(cfg))
    for k, v in ref.items():
        out["ref_" + k] = v
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
    print(f"{name}: atoms={m.natoms} elements={m.nelements} "
          f"-> {os.path.getsize(os.path.join(HERE, name + '.npz'))} bytes")


def main() -> None:
    if not O.ref_available():
        O.build(ref=True)
    make_eam_file()
    names = sys.argv[1:] or list(C.CASES)
    for name in names:
        run_case(name, C.CASES[name])


if __name__ == "__main__":
    main()
