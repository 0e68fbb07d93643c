"""Drive libcacg through the C ABI the same way the oracle tests drive the
reference, returning the same output keys."""
import os
import tempfile

import numpy as np

import cases as C
from cac_code_gb300 import cacg
from cac_code_gb300 import lattice as L


def configure(s, cfg, m, via_files=False, eam_file=C.EAM_FILE, pair_lines=None):
    """Set up a System either through input commands + read_data (the drop-in
    path) or through direct array uploads."""
    kw = C.settings_kwargs(cfg, eam_file)
    if via_files:
        wd = tempfile.mkdtemp(prefix="cacg_")
        data = os.path.join(wd, "data.cac")
        L.write_data(m, data, with_velocities=True)
        from oracle import oracle as O
        script = O.input_script(data, boundary=cfg["boundary"], extra=C.fix_lines(cfg, m), **kw)
        path = os.path.join(wd, "in.cac")
        with open(path, "w") as f:
            f.write(script)
        s.file(path)
        # atom velocities have no data-file section; upload them directly
        s.set_atoms(m.atom_x, m.atom_v, np.ones(m.natoms, dtype=np.int32))
        return
    s.command(f"units {kw['units']}")
    s.command(f"boundary {cfg['boundary']}")
    s.load_model(m)
    if pair_lines:
        for line in pair_lines:
            s.command(line)
    elif kw["pair"] == "lj/cut":
        s.command(f"pair_style lj/cut {kw['lj'][2]!r}")
        s.command(f"pair_coeff 1 1 {kw['lj'][0]!r} {kw['lj'][1]!r}")
    else:
        s.command("pair_style eam")
        s.command(f"pair_coeff 1 1 {kw['eam_file']}")
    s.command(f"neighbor {kw['skin']!r} bin")
    mod = (f"neigh_modify every {kw['every']} delay {kw['delay']} "
           f"check {'yes' if kw['check'] else 'no'}")
    if kw["binsize"] > 0:
        mod += f" binsize {kw['binsize']!r}"
    s.command(mod)
    if kw["nsplit"] != 2:
        s.command(f"elementsplit {kw['nsplit']}")
    if kw["dt"] is not None:
        s.command(f"timestep {kw['dt']!r}")
    s.command("fix 1 all nve")
    for line in C.fix_lines(cfg, m):
        s.command(line)


def run_gpu(cfg, m, mode=cacg.FP64_EXACT, via_files=False, steps=None, pair_lines=None,
            before_init=None):
    s = cacg.System(0)
    try:
        configure(s, cfg, m, via_files=via_files, pair_lines=pair_lines)
        if before_init is not None:
            before_init(s)
        s.set_precision(mode)
        s.init()
        s.setup()
        out = {}
        if m.natoms:
            s.neighbor_build()
            out["atom_numneigh"], out["atom_neigh"] = s.atom_list()
            a = s.atoms(all_=True)
            out["atom_tag_all"], out["atom_x_all"] = a["tag"], a["x"].reshape(-1)
            out["centro"] = s.centro()
            s.pair_compute()
            out["atom_f"] = s.atoms()["f"].reshape(-1)
        if m.nelements:
            s.neighbor_ebuild()
            s.neighbor_nbuild()
            enum, eneigh, ipn, ipj, ipnj = s.elem_lists()
            out.update(elem_numneigh=enum, elem_neigh=eneigh, ip_numneigh=ipn,
                       ip_neigh_elem=ipj, ip_neigh_site=ipnj, elem_cuts=s.cuts())
            s.pair_ecompute()
            out["nodef"] = s.elements()["nodef"].reshape(-1)
        s.run(cfg["steps"] if steps is None else steps)
        a = s.atoms()
        e = s.elements()
        out.update(s1_x=a["x"].reshape(-1), s1_v=a["v"].reshape(-1), s1_f=a["f"].reshape(-1),
                   s1_nodex=e["nodex"].reshape(-1), s1_nodev=e["nodev"].reshape(-1),
                   s1_nodef=e["nodef"].reshape(-1), s1_elem_x=e["x"].reshape(-1),
                   rebuilds=np.array([s.counts()["rebuilds"]]))
        out["_counts"] = s.counts()
        return out
    finally:
        s.close()
