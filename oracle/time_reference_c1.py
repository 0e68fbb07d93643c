"""Time the UNMODIFIED reference (oracle/_ref/cacref, built by ``make -C
oracle ref`` from the reference sources) on C1 in full: 16,384 LJ atoms + 64
elements, driven in Verlet::run order by the harness, single core.

The per-step cost is the difference between two runs that differ only in
their step count (start-up, set-up and list builds cancel).  C1 cannot run its
1,000 steps under the reference's algorithm (the elements' kinetic energy
grows until, at step 260, the bin grid no longer holds the atoms), so the
runs take 20 and 220 steps.

Run from the repository root in a container that has the reference tree:
    python oracle/time_reference_c1.py
"""
from __future__ import annotations

import json
import os
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path = [ROOT] + [p for p in sys.path if os.path.abspath(p or ".") != HERE]

from cac_code_gb300 import lattice as L  # noqa: E402
from cac_code_gb300 import workloads as W  # noqa: E402
from oracle import oracle as O  # noqa: E402


def _run(m, cfg, steps: int) -> float:
    wd = tempfile.mkdtemp(prefix="cacref_c1_")
    L.write_data(m, os.path.join(wd, "data.cac"), with_velocities=True)
    m.atom_v.astype(np.float64).tofile(os.path.join(wd, "v.bin"))
    kw = W.oracle_kwargs(cfg)
    script = O.input_script("data.cac", boundary=cfg["boundary"], units=kw["units"],
                            pair=kw["pair"], skin=kw["skin"], lj=kw.get("lj", (1.0, 1.0, 2.5)),
                            every=kw["every"], delay=kw["delay"], check=kw["check"],
                            dt=kw.get("dt"))
    directives = [f"capacity {8 * (m.natoms + 64)}", "velocities v.bin", "setup", "atom_list",
                  "elem_lists", f"step {steps}"]
    t0 = time.perf_counter()
    O.run_reference(script, "\n".join(directives) + "\n", wd, timeout=3600)
    return time.perf_counter() - t0


def main() -> None:
    m, cfg = W.c1_lj()
    sites = W.metric_sites(m, cfg)
    short, long_ = 20, 220
    t_s = min(_run(m, cfg, short) for _ in range(2))
    t_l = min(_run(m, cfg, long_) for _ in range(2))
    per_step = (t_l - t_s) / (long_ - short)
    print(json.dumps({"workload": "C1: LJ, 16,384 atoms + 64 elements (8 sites per edge)",
                      "code": "the reference's own C++ (oracle/_ref/cacref), -O3, one core",
                      "sites": sites, "s_per_step": per_step,
                      "site_steps_per_s": sites / per_step,
                      "runs_s": {str(short): t_s, str(long_): t_l}}))


if __name__ == "__main__":
    main()
