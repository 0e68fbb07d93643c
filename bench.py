#!/usr/bin/env python
"""Benchmark: site-steps/s of the CAC step on one GB300 per rank.

Default workload: the surrogate configuration, EAM Cu with a 1,982,464-atom
core between 499,712 rhombohedral elements of 11 sites per edge (10 primitive
spacings, 1,331 sites each; 8 Gauss points + 8 node rows per element), 300 K,
dt = 1 fs, neighbor 7.5 bin, every 10 steps with the distance check.  The
headline mode is mixed precision (FP32 pair terms) with the nodal-force
surrogate attached at an ensemble-spread tolerance of 1e-4; the plain FP64 and
bit-exact FP64 paths are timed on the same system, with every mode's force
difference from the bit-exact forces of one configuration.

A step is one full Verlet step of the reference's loop (verlet.cpp:163-218):
NVE half-kick and drift of atoms and nodes, rebuild decision (every 10 steps),
ghost refresh or rebuild, EAM density + embedding derivative + force passes
over the atom list, nodal densities and integration-point forces over the
element lists with the shape-function gather onto the nodes, and the final
half-kick.  site-steps/s = (atoms + Gauss integration points) * steps / s.

value: the K timed steps' device time, with the rebuilds and list reorders
that fell inside them replaced by the rates counted over a longer window
(>= 200 steps) at their event-timed costs, so that neighbor work enters at its
natural frequency.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--config c5|c2|c5-medium|...]
  python bench.py --impl reference ...   # the reference algorithm on the host cores

Multi-GPU (torchrun): replicas only -- every rank runs its own system, no
collective on the data path; value = all ranks' site-steps / max rank time.
"""
from __future__ import annotations

import argparse
import json
import multiprocessing as mp
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "site-steps/s on 1 GB300: mixed+surrogate vs plain FP64 at ≤1e-4 rel force err"
UNIT = "site-steps/s"

# (workload builder, label) per --config
CONFIGS = {
    "c5": ("c5_eam", "C5: EAM Cu CAC slab, 1,982,464 atoms + 499,712 elements of 11 sites per "
                     "edge (10 spacings, 1,331 sites), 8 Gauss points + 8 node rows each"),
    "c5-medium": ("c5_medium", "C5-structured medium slab: EAM Cu 247,808 atoms + 64,000 elements "
                               "of 11 sites per edge (profiling size)"),
    "c2": ("c2_eam", "C2: EAM Cu CAC slab, 1,016,400 atoms + 20,000 elements of 11 sites per "
                     "edge (10 spacings, 1,331 sites), 8 Gauss points + 8 node rows each"),
    "c2-medium": ("c2_medium", "C2-structured medium slab: EAM Cu 266,200 atoms + 7,200 elements "
                               "of 11 sites per edge (profiling size)"),
    "c2-small": ("c2_sample", "C2 sample: EAM Cu 9,680 atoms + 160 elements of 11 sites per edge"),
}
SAMPLES = {"c5": "c5_sample", "c5-medium": "c5_sample", "c2": "c2_sample",
           "c2-medium": "c2_sample", "c2-small": "c2_sample"}


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=50)
    p.add_argument("--warmup", type=int, default=5)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--config", default="c5", choices=sorted(CONFIGS))
    p.add_argument("--mode", default="mixed", choices=["fp64", "exact", "mixed"])
    p.add_argument("--loop", default="device", choices=["device", "host"],
                   help="steps as device-loop graph launches (rebuild decisions on the "
                        "device) or per-step graphs with host decisions (ncu lists the "
                        "kernels of the latter one by one)")
    p.add_argument("--no-surrogate", action="store_true",
                   help="mixed mode without the nodal-force surrogate")
    p.add_argument("--sur-tol", type=float, default=1e-4,
                   help="ensemble-spread tolerance (fraction of the rms nodal force)")
    p.add_argument("--sur-samples", type=int, default=2000000)
    p.add_argument("--sur-epochs", type=int, default=10)
    p.add_argument("--long-steps", type=int, default=200,
                   help="steps of the window that counts rebuilds and list reorders")
    p.add_argument("--c4-steps", type=int, default=2000,
                   help="steps of the batched-replica workload (256 replicas; 0: skip)")
    p.add_argument("--drift-steps", type=int, default=1000,
                   help="NVE steps of the energy-drift run after the timed region (0: skip)")
    p.add_argument("--cpu-steps", type=int, default=150,
                   help="steps of each host-core sample replica of the CPU baseline")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-modes", action="store_true", help="skip timing the other precision modes")
    p.add_argument("--study", choices=["strain", "drift", "surrogate", "c1"],
                   help="a longer measurement instead of the benchmark (one JSON line)")
    p.add_argument("--study-steps", type=int, default=0, help="steps of a study (0: its default)")
    return p.parse_args()


# ----------------------------------------------------------------------------- ranks

def dist_init():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("gloo", rank=rank, world_size=ws)
    return ws, rank, local


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def aggregate(ws, sites_per_rank, steps, ms_local):
    """Whole-job site-steps/s of independent replicas: every rank's sites over
    the slowest rank's device time (ranks exchange only this scalar)."""
    ms_max = allmax(ws, ms_local)
    return ws * sites_per_rank * steps / (ms_max * 1e-3), ms_max


def allmax(ws, v):
    if ws <= 1:
        return v
    import torch
    import torch.distributed as dist
    t = torch.tensor([v], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ----------------------------------------------------------------------------- clocks

class ClockSampler:
    """nvidia-smi clock/throttle samples every 200 ms during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": sorted(reasons),
                "samples": len(sm)}


def profiler_range(on):
    """With CACG_PROFILE_TIMED=1 in the environment, the timed region is the
    profiler's range (cuProfilerStart / cuProfilerStop of the driver), so that
    ncu --profile-from-start off lists the timed steps' launches alone."""
    if os.environ.get("CACG_PROFILE_TIMED") != "1":
        return
    import ctypes
    lib = ctypes.CDLL("libcuda.so.1")
    (lib.cuProfilerStart if on else lib.cuProfilerStop)()


def merge_clocks(*recs):
    """One clock record from the samplers of several windows of the same workload."""
    ok = [r for r in recs if r.get("sm_mhz") is not None]
    if not ok:
        return recs[0]
    n = sum(r.get("samples", 0) for r in ok)
    med = sorted((r["sm_mhz"] for r in ok for _ in range(max(r.get("samples", 1), 1))))
    return {"sm_mhz": med[len(med) // 2], "sm_max_mhz": max(r["sm_max_mhz"] for r in ok),
            "reasons": sorted(set().union(*(r["reasons"] for r in ok))), "samples": n}


# ----------------------------------------------------------------------------- CPU legs

def _cpu_worker(args):
    """One host core: the CPU restatement of the reference on a sample replica
    of the workload's structure, timed over ``steps`` steps."""
    sample, seed, steps, warm, eam = args
    sys.path.insert(0, ROOT)
    from cac_code_gb300 import workloads as W
    from oracle import oracle as O
    m, cfg = getattr(W, sample)(seed=seed)
    o = O.Oracle(m, **W.oracle_kwargs(cfg, eam))
    o.setup()
    if m.natoms:
        o.atom_list()
    if m.nelements:
        o.elem_lists()
    o.run(warm)
    t0 = time.perf_counter()
    o.run(steps)
    dt = time.perf_counter() - t0
    return W.metric_sites(m, cfg) * steps / dt, dt, W.metric_sites(m, cfg), m.natoms, m.nelements


def cpu_leg(sample, cores, steps, warm, eam):
    from oracle import oracle as O
    O.build()
    ctx = mp.get_context("spawn")
    with ctx.Pool(cores) as pool:
        res = pool.map(_cpu_worker, [(sample, 100 + k, steps, warm, eam) for k in range(cores)])
    return sum(r[0] for r in res), max(r[1] for r in res), res[0][2:]


# ----------------------------------------------------------------------------- byte models

# The algorithmic bytes of each main kernel per launch (compulsory traffic:
# every per-item input read once, every output written once, each list entry
# read once per pass; neighbor gathers count as cache hits).  c: counts after
# the timed steps; L: lattice lines the lists reference (all rows, force rows).

def kernel_bytes(name, c, mode, lines_all, lines_force, nae_lines):
    n = c["nlocal"]
    ne = c["enlocal"]
    ne_all = ne + c["enghost"]
    rows_n = 8 * ne                     # node rows (EAM nodal densities)
    rows_f = c["force_rows"]            # Gauss rows (nonzero weight)
    scan_e = c["ip_scan_entries"] / max(c["ip_rows"], 1)   # entries scanned per row
    n_s = c["short_entries"] / max(n, 1)
    if mode == "mixed" and c.get("elem_fused"):
        # the fused element passes (one warp per element): per element the split
        # nodes 192 (read in both passes), the nodal densities 64 (written by
        # the density pass, read by the force pass) and the nodal forces 192;
        # per row the row start pair 8, culling counts 16, lattice indices 16
        # and the list codes 4 n.  No line or site data reaches memory.
        n_scan = c["density_scan_entries"] / max(n, 1)
        return {
            "atom1": n * (16 + 4 + 4 * n_scan + 4 + 4 * n_s + 8 + 4),
            "atom2": n * (16 + 4 + 4 * n_s + 4 + 24),
            "elem_rho": ne * (192 + 64) + rows_n * (8 + 16 + 16 + 4 * scan_e),
            "elem_force": ne * (192 + 64 + 192) + rows_f * (8 + 16 + 16 + 4 * scan_e),
            # node split only (the lines are formed on list-reorder steps alone)
            "sites": ne_all * (192 + 192),
        }
    if mode == "mixed":
        n_scan = c["density_scan_entries"] / max(n, 1)
        return {
            # packed x_i 16, count 4, scanned entries 4n, short-list count 4 and
            # entries 4 n_s written, rho 8, F' 4
            "atom1": n * (16 + 4 + 4 * n_scan + 4 + 4 * n_s + 8 + 4),
            # packed x_i 16, short count 4 + entries 4 n_s, F'_i 4, f_i 24
            "atom2": n * (16 + 4 + 4 * n_s + 4 + 24),
            # per node row: element index data 8, row start pair 8, culling counts
            # 16, packed point 16, codes 4 n, nodal density 8; the line data
            # (48 B a line) of the lines the node rows reference, read once
            "elem_rho": rows_n * (8 + 8 + 16 + 16 + 4 * scan_e + 8) + lines_all * 48,
            # per Gauss row: row 4, element 4, row start pair 8, culling counts
            # 16, packed point 16, F' 4, codes 4 n, force 24; line data 48 and
            # density line 8 of the force rows' lines
            "elem_force": rows_f * (4 + 4 + 8 + 16 + 16 + 4 + 4 * scan_e + 24)
            + lines_force * (48 + 8),
            # node split (read 192, write 192 per element), lattice lines (node
            # halves 192 per element, masks 8 per line slot, 48 per formed line)
            "sites": ne_all * (192 + 192 + 192 + 8 * nae_lines) + lines_all * 48,
            # density lines: nodal densities 64 per element, masks, 8 per line;
            # row F': per Gauss row 16 in, 4 out
            "site_fp": ne_all * (64 + 8 * nae_lines) + lines_force * 8 + rows_f * 20,
        }
    # FP64 modes: per atom x_i 24, count 4, short list 4 n_s, rho/F' 16 or fp_i 8 + f_i 24
    return {
        "atom1": n * (24 + 4 + 4 * n_s + 16),
        "atom2": n * (24 + 4 + 4 * n_s + 8 + 24),
    }


# FP64 operations per launch of the plain FP64 path's kernels (a multiply and
# an add count two; the site kernels run without contraction, so each is one
# FP64 instruction).  Sites: 8 nodes x 3 coordinates, a multiply and an add
# each; site F': 8 density products and sums plus the spline derivative (8);
# atom density pass: difference, squared distance, root, index and cubic per
# short-list entry (20); atom force pass: 45 per entry (two splines, the
# derivative terms and the force components).

def fp64_flops(name, c):
    n = max(c["nlocal"], 1)
    n_s = c["short_entries"] / n
    return {"sites": 48.0 * c["sites_needed"], "site_fp": 24.0 * c["sites_needed"],
            "atom1": 20.0 * c["nlocal"] * n_s, "atom2": 45.0 * c["nlocal"] * n_s}.get(name)


# ----------------------------------------------------------------------------- arms

def run_ours(a, ws, rank, local):
    import numpy as np
    from cac_code_gb300 import build, cacg
    from cac_code_gb300 import workloads as W
    build.build_library()
    tmp = tempfile.mkdtemp(prefix="cacbench_")
    eam = W.write_eam(os.path.join(tmp, "Cu_analytic_2000.eam"))
    builder, label = CONFIGS[a.config]

    cpu = None
    if rank == 0 and ws == 1 and not a.no_cpu_baseline:
        # before the first GPU call: spawn the host-core sample
        cores = os.cpu_count() or 1
        val, wall, (s_sites, s_atoms, s_elems) = cpu_leg(SAMPLES[a.config], cores, a.cpu_steps, 5,
                                                         eam)
        cpu = {"value": val, "unit": UNIT, "cores": cores, "kind": "port",
               "sample": f"{cores} independent replicas of {s_atoms:,} atoms + {s_elems:,} "
                         f"elements ({s_sites:,} metric sites, the workload's structure) on the "
                         f"CPU restatement of the reference (oracle/cac_oracle.c, -O3), "
                         f"{a.cpu_steps} timed steps each after 5 warm-up, {wall:.1f} s"}

    m, cfg = getattr(W, builder)()
    sites = W.metric_sites(m, cfg)
    s = cacg.System(local)
    W.configure_system(s, m, cfg, eam)
    mode = {"fp64": cacg.FP64, "exact": cacg.FP64_EXACT, "mixed": cacg.MIXED}[a.mode]
    s.set_precision(mode)
    s.command(f"tune loop {a.loop}")  # device: steps as graph launches, decisions on the device
    s.init()
    s.setup()
    s.neighbor_build()
    if m.nelements:
        s.neighbor_ebuild()
        s.neighbor_nbuild()
    nae = m.etypes[0].nae[0] if m.nelements else 0

    # the surrogate: samples from the plain FP64 quadrature on strained,
    # thermally perturbed periodic element boxes of the workload's element
    # type, trained on the GPU, attached to the elements farther than 2 r_c
    # from the atoms
    sur, net = None, None
    use_sur = a.mode == "mixed" and not a.no_surrogate and m.nelements > 0
    if use_sur:
        from cac_code_gb300 import surrogate as S
        t0 = time.perf_counter()
        xs, ts, info = S.generate(eam, a.sur_samples, seed=11, nae=nae, planes=8, ny=8, nz=8,
                                  snapshots=16, device=local)
        xv, tv, _ = S.generate(eam, 32768, seed=12, nae=nae, planes=8, ny=8, nz=8, snapshots=4,
                               device=local)
        t_gen = time.perf_counter() - t0
        t0 = time.perf_counter()
        net, loss = S.train(xs, ts, members=4, epochs=a.sur_epochs, batch=2048, lr=2e-3,
                            device=local)
        t_train = time.perf_counter() - t0
        del xs, ts
        pm, psp = net.predict(xv)
        fs = net.normalization()[4]
        err_elem = np.abs(pm - tv).max(axis=1) / fs
        sur = {"tol": a.sur_tol, "distance_A": 11.0, "members": 4,
               "network": "32-256-256-256-24 SiLU, bf16 tensor cores, fp32 accumulation",
               "samples": info, "generate_s": round(t_gen, 2), "train_s": round(t_train, 2),
               "epochs": a.sur_epochs, "train_loss_normalised": loss,
               "heldout_force_error": S.force_errors(pm, tv),
               "heldout_spread_median_rel": float(np.median(psp) / fs),
               "heldout_fraction_spread_within_tol": float(np.mean(psp <= a.sur_tol * fs)),
               "heldout_fraction_error_within_tol": float(np.mean(err_elem <= a.sur_tol))}
        s.surrogate_reference(m.nodex)
        s.surrogate_attach(net, tol=a.sur_tol, dist=11.0)
    c0 = s.counts()
    s.run(max(a.warmup, 3))
    s.set_timing(False)  # steps run as device-loop graph launches
    K = a.steps

    # ---- neighbor work at its natural frequency: rebuilds and list reorders
    # counted over a longer window run before the timed region (it also
    # brings the surrogate's re-test back-off to its steady state); their
    # costs from events (rebuilds) and from one eager step right after a list
    # build, which reorders every list (reorders), less the same kernels' time
    # in a step that does not reorder
    n_long = max(a.long_steps, a.steps)
    cl0 = s.counts()
    rbl0 = s.kernel_timing()[9]
    clocks_long = ClockSampler(local)
    clocks_long.start()
    s.run(n_long)
    clk_long = clocks_long.stop()
    cl1 = s.counts()
    rb_ms_long = s.kernel_timing()[9] - rbl0
    lw = {k: cl1[k] - cl0[k] for k in ("rebuilds", "rebuilds_atoms_only", "atom_reorders",
                                       "ip_reorders")}

    # ---- the timed region: exactly K steps
    clocks = ClockSampler(local)
    barrier(ws)
    clocks.start()
    cs = s.counts()
    l0 = cs["launches"]
    rb_ms0 = s.kernel_timing()[9]
    t0 = time.perf_counter()
    profiler_range(True)
    s.run(a.steps)
    profiler_range(False)
    wall = time.perf_counter() - t0
    clk = clocks.stop()
    barrier(ws)
    dev_ms = float(s.timing()[0])
    c1 = s.counts()
    rb_ms_timed = s.kernel_timing()[9] - rb_ms0
    launches = c1["launches"] - l0
    graph_steps = c1["graph_steps"] - cs["graph_steps"]
    win = {k: c1[k] - cs[k] for k in ("rebuilds", "rebuilds_atoms_only", "atom_reorders",
                                      "ip_reorders")}

    # ---- the same number of steps run eagerly with events: phases and kernels
    s.set_graphs(False)
    s.set_timing(True)
    s.run(a.steps)
    tm = s.timing()
    kt = s.kernel_timing()
    eager_ms = float(tm[0])
    s.set_timing(False)
    s.set_graphs(True)
    if sur is not None:
        # element-steps of the timed window (warm-up included in c0 .. c1)
        ev = c1["surrogate_evaluated"] - cs["surrogate_evaluated"]
        ac = c1["surrogate_accepted"] - cs["surrogate_accepted"]
        far = c1["surrogate_elements"]
        sur["far_elements"] = far
        sur["elements"] = c1["enlocal"]
        sur["tested_fraction_timed"] = ev / (far * K) if far else 0.0
        sur["accepted_fraction_of_tests_timed"] = ac / ev if ev else 0.0
        sur["accepted_fraction_timed"] = ac / (far * K) if far else 0.0
        sur["retest"] = ("a rejected element is re-tested after 1, 3, 7, 15, 31, 63, then 127 "
                         "steps (the quadrature evaluates it meanwhile); an accepted one every "
                         "step")

    rb_cost = rb_ms_long / lw["rebuilds"] if lw["rebuilds"] else (
        rb_ms_timed / win["rebuilds"] if win["rebuilds"] else 0.0)

    st_a = s.atoms()
    st_e = s.elements()
    st = (st_a["x"].copy(), st_a["v"].copy(), st_e["nodex"].copy(), st_e["nodev"].copy())

    def restore():
        """The state right after the long window, lists rebuilt from it."""
        s.put_atoms(st[0], st[1])
        s.put_nodes(st[2], st[3])
        s.neighbor_build()
        if m.nelements:
            s.neighbor_ebuild()
            s.neighbor_nbuild()

    ro_cost_a = ro_cost_e = 0.0
    if a.mode == "mixed":
        restore()
        s.set_graphs(False)
        s.set_timing(True)
        s.run(1)   # reorders the atom and integration-point lists
        k_re = s.kernel_timing()
        s.run(1)   # reorders nothing
        k_no = s.kernel_timing()
        s.set_timing(False)
        s.set_graphs(True)
        ro_cost_a = max(k_re[6] - k_no[6], 0.0)
        ro_cost_e = max(k_re[7] - k_no[7], 0.0)
    K = a.steps
    extra = ((lw["rebuilds"] / n_long * K - win["rebuilds"]) * rb_cost
             + (lw["atom_reorders"] / n_long * K - win["atom_reorders"]) * ro_cost_a
             + (lw["ip_reorders"] / n_long * K - win["ip_reorders"]) * ro_cost_e)
    amort_ms = dev_ms + extra
    value, ms_max = aggregate(ws, sites, K, amort_ms)
    value_window, _ = aggregate(ws, sites, K, dev_ms)
    neighbor_work = {
        "long_window_steps": n_long, "long_window": lw, "timed_window": win,
        "rebuild_ms_each": rb_cost, "atom_list_reorder_ms_each": ro_cost_a,
        "ip_list_reorder_ms_each": ro_cost_e,
        "timed_ms": dev_ms, "amortised_ms": amort_ms,
        "value_timed_window_unamortised": value_window,
        "note": "value = sites * K / (timed device ms + (long-window rate * K - events in the "
                "timed window) * event cost) for rebuilds and both list reorders"}

    # ---- the dominant kernel: largest event-timed share of the eager run
    names = ["atom1", "atom2", "elem_rho", "elem_force", "sur", "sites", "apart", "eprep",
             "site_fp"]
    kms = {nm: float(kt[i]) / K for i, nm in enumerate(names)}
    lines_all, lines_force = s.referenced_lines() if m.nelements else (0, 0)
    nae_lines = nae * nae
    kb = kernel_bytes(None, c1, a.mode, lines_all, lines_force, nae_lines)
    peaks_path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    peak, peak_src = 6800.0, "fallback 6.8 TB/s"
    if os.path.exists(peaks_path):
        try:
            peak = float(json.load(open(peaks_path))["hbm_gbs"])
            peak_src = "measured (MEASURED_PEAKS.json hbm_gbs)"
        except Exception:
            pass
    kernels = {}
    step_ms = eager_ms / K
    for nm in names:
        if kms[nm] <= 0:
            continue
        e = {"ms": round(kms[nm], 4), "share_of_eager_step": round(kms[nm] / step_ms, 4)}
        if nm in kb:
            e["algorithmic_bytes"] = kb[nm]
            e["achieved_GBps"] = kb[nm] / (kms[nm] * 1e-3) / 1e9
            e["hbm_frac"] = e["achieved_GBps"] / peak
        kernels[nm] = e
    dom = max(kernels, key=lambda k: kernels[k]["ms"])
    kernel_names = {
        "atom1": "k_eam_rho_atoms (EAM density pass over the atom list)",
        "atom2": "k_eam_force_atoms (EAM force pass over the atom list)",
        "elem_rho": ("k_elem_rho_fused (nodal densities, one warp per element)"
                     if c1.get("elem_fused") else
                     "k_ipg<EAM, density> (nodal densities over the node rows)"),
        "elem_force": ("k_elem_force_fused (integration-point forces and nodal gather, one "
                       "warp per element)" if c1.get("elem_fused") else
                       "k_ipg<EAM, force> (integration-point forces over the Gauss rows)"),
        "sur": "surrogate (features, k_mlp_ensemble, acceptance)",
        "sites": "k_node_split + k_lines (lattice lines)",
        "site_fp": "k_line_rho + k_row_fp",
    }
    traffic = None
    tpath = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(tpath):
        try:
            tj = json.load(open(tpath))
            key = f"{a.config}:{a.mode}:{dom}_bytes_per_unit"
            if key in tj:
                unit = {"atom1": c1["nlocal"], "atom2": c1["nlocal"]}.get(dom, c1["enlocal"])
                traffic = tj[key] * unit
        except Exception:
            traffic = None
    dk = kernels[dom]
    fp64_peak = s.fp64_peak()

    # ---- the other precision modes on the same system: timing, and every
    # mode's force difference from the bit-exact FP64 forces of one configuration
    modes = {}
    force_error = None
    roof64 = None
    if not a.no_modes and ws == 1:
        def forces():
            s.pair_compute()
            s.pair_ecompute()
            return s.atoms()["f"].copy(), s.elements()["nodef"].copy()

        def rel_err(fa, fb):
            out = {}
            for key, (x, y) in {"atoms": (fa[0], fb[0]), "nodes": (fa[1], fb[1])}.items():
                x = x.reshape(-1, 3)
                y = y.reshape(-1, 3)
                if y.size:
                    d = np.linalg.norm(x - y, axis=1)
                    n_ = np.linalg.norm(y, axis=1)
                    out[key] = {"rms_rel": float(np.sqrt((d ** 2).mean() / (n_ ** 2).mean())),
                                "max_rel": float(d.max() / n_.max())}
            return out
        # (name, precision, surrogate tolerance or None, timed steps)
        variants = [("exact", cacg.FP64_EXACT, None, min(K, 5)),
                    ("fp64", cacg.FP64, None, min(K, 10)),
                    ("mixed", cacg.MIXED, None, K)]
        head = a.mode
        if use_sur:
            head = "mixed+surrogate"
            variants += [(head, cacg.MIXED, a.sur_tol, K),
                         ("mixed+surrogate(tol=1e-2)", cacg.MIXED, 1e-2, K)]

        def setv(mcode, tol):
            s.set_precision(mcode)
            if use_sur:
                s.surrogate_attach(net if tol is not None else None, tol=tol or 0.0, dist=11.0)
        fs_ = {}
        restore()
        for name, mcode, tol, _ in variants:
            setv(mcode, tol)
            fs_[name] = forces()
        errs = {name: rel_err(fs_[name], fs_["exact"]) for name, _, _, _ in variants}
        del fs_
        force_error = {"vs": "bit-exact FP64 forces at the same configuration", **errs[head]}
        for name, mcode, tol, nst in variants:
            if name == head:
                continue
            setv(mcode, tol)
            restore()
            cs0 = s.counts()
            s.run(2)
            s.run(nst)  # graphs on, as in the headline
            t_all = s.timing()[0]
            cs1 = s.counts()
            s.set_graphs(False)
            s.set_timing(True)
            s.run(nst)
            tmm = s.timing()
            ktm = s.kernel_timing()
            s.set_timing(False)
            s.set_graphs(True)
            modes[name] = {"value": sites * nst / (t_all * 1e-3), "steps": nst,
                           "ms_per_step": t_all / nst,
                           "phase_ms_per_step_eager": [round(v / nst, 4) for v in tmm[1:6]],
                           "kernel_ms_per_step_eager": {nm: round(float(ktm[i]) / nst, 4)
                                                        for i, nm in enumerate(names)
                                                        if ktm[i] > 0},
                           "force_err_vs_exact": errs[name]}
            if tol is not None:
                ev = cs1["surrogate_evaluated"] - cs0["surrogate_evaluated"]
                far = cs1["surrogate_elements"]
                modes[name]["accepted_fraction"] = (
                    (cs1["surrogate_accepted"] - cs0["surrogate_accepted"]) / (far * (nst + 2))
                    if far else 0.0)
            if name == "fp64":
                # the plain FP64 path against the FP64 roof: its dominant kernel's
                # FP64 operations per launch over its event time
                k64 = modes[name]["kernel_ms_per_step_eager"]
                dk64 = max(k64, key=k64.get)
                fl = fp64_flops(dk64, s.counts())
                roof64 = {"bound": "fp64", "kernel": dk64, "ms": k64[dk64], "flops_per_launch": fl,
                          "achieved": fl / (k64[dk64] * 1e-3) if fl else None,
                          "peak": fp64_peak, "unit": "FLOP/s",
                          "frac": (fl / (k64[dk64] * 1e-3) / fp64_peak) if fl else None,
                          "peak_source": "measured FP64 FMA loop on this GPU (cacg_measure_fp64_peak)"}
        setv(mode, a.sur_tol if use_sur else None)

    # ---- e2e through the C ABI with host-resident state: x,v (atoms + nodes)
    # in from pinned host memory, one step, the new x,v (atoms + nodes) back
    # out, every step (cacg_run_host)
    e2e = None
    if not a.no_e2e:
        try:
            import torch
            pin = torch.cuda.is_available()
        except Exception:
            pin = False
        n = c1["nlocal"]
        ne = c1["enlocal"]

        def host(shape):
            if pin:
                import torch
                return torch.empty(shape, dtype=torch.float64).pin_memory().numpy()
            return np.empty(shape, dtype=np.float64)
        restore()
        hx, hv, hf = host((n, 3)), host((n, 3)), host((n, 3))
        hnx, hnv = host((ne, 8, 3)), host((ne, 8, 3))
        s.get_state_into(hx, hv, hf)
        el = s.elements()
        hnx[...] = el["nodex"]
        hnv[...] = el["nodev"]
        del el
        s.set_timing(False)
        e_steps = max(10, min(K, 50))
        # untimed warm-up through the same call (the first steps after the
        # restore re-partition the lists)
        for _ in range(max(a.warmup, 3)):
            s.run_host(1, hx, hv, hnx, hnv)
        barrier(ws)
        ce0 = s.counts()
        t0 = time.perf_counter()
        for _ in range(e_steps):
            s.run_host(1, hx, hv, hnx, hnv)
        e_wall = time.perf_counter() - t0
        ce1 = s.counts()
        e_wall = allmax(ws, e_wall)
        e2e = {"value": ws * sites * e_steps / e_wall, "unit": UNIT,
               "h2d_bytes_per_step": int(hx.nbytes + hv.nbytes + hnx.nbytes + hnv.nbytes),
               "d2h_bytes_per_step": int(hx.nbytes + hv.nbytes + hnx.nbytes + hnv.nbytes),
               "steps": e_steps, "warmup": max(a.warmup, 3),
               "graph_replays": ce1["graph_steps"] - ce0["graph_steps"],
               "atom_reorders": ce1["atom_reorders"] - ce0["atom_reorders"],
               "surrogate_tests": ce1["surrogate_evaluated"] - ce0["surrogate_evaluated"],
               "note": "state round trip per step: x, v of atoms and nodes in and out of "
                       "pinned host buffers through cacg_run_host, one call per step (copies "
                       "overlap the step where the data allow)"}

    # ---- energy drift of the headline mode, atoms and elements apart (they do
    # not interact): FP64 energies before and after an NVE run.  The potential
    # is not smoothed at the cutoff (phi(rc) = -0.0189 eV): a pair crossing it
    # makes the total jump by that much
    drift = None
    if a.drift_steps > 0:
        s.set_timing(False)
        restore()
        t_a = s.thermo()
        s.run(a.drift_steps)
        t_b = s.thermo()
        ea0, ea1 = t_a["pe_atoms"] + t_a["ke_atoms"], t_b["pe_atoms"] + t_b["ke_atoms"]
        ee0, ee1 = t_a["pe_elements"] + t_a["ke_nodes"], t_b["pe_elements"] + t_b["ke_nodes"]
        ngp = cfg["gauss_per_element"] * max(c1["enlocal"], 1)
        drift = {"steps": a.drift_steps, "mode": a.mode + ("+surrogate" if use_sur else ""),
                 "atoms": {"e_start_ev": ea0, "e_end_ev": ea1,
                           "ev_per_atom": (ea1 - ea0) / max(c1["nlocal"], 1)},
                 "elements": {"e_start_ev": ee0, "e_end_ev": ee1,
                              "ev_per_gauss_point": (ee1 - ee0) / ngp,
                              "ke_nodes_start_ev": t_a["ke_nodes"],
                              "ke_nodes_end_ev": t_b["ke_nodes"]},
                 "ev_per_site": (t_b["etotal"] - t_a["etotal"]) / sites,
                 "note": ("atoms and elements do not interact. The elements' energy grows "
                          "under the reference's element force, which is not the gradient of "
                          "their energy (the CPU restatement of the reference grows the same "
                          "way), so the element and per-site figures measure that dynamics, "
                          "not integration error. The effect of the precision on NVE energy "
                          "is measured by bench.py --study drift (atoms, 10,000 steps, mixed "
                          "against bit-exact FP64 on the same trajectory).")}

    # ---- the batched-replica workload: 256 independent replicas packed by
    # pair style and size class, autotuned, graph-replayed
    c4 = None
    if a.c4_steps > 0 and ws == 1:
        s.close()
        s = None
        from cac_code_gb300 import batch as B
        t0 = time.perf_counter()
        c4 = B.run_batch(eam, n=256, steps=a.c4_steps, seed=4, tune=True, device=local)
        c4["wall_s_with_setup_and_tuning"] = round(time.perf_counter() - t0, 1)
        c4["note"] = ("per class one handle (replicas side by side); every class's step loop "
                      "is a branch of one CUDA graph (rebuild decisions on the device), one "
                      "launch runs all classes until each is done or needs a rebuild, which the "
                      "host performs before the next launch; site_steps_per_s = all classes' "
                      "site-steps over the wall time of the timed run")

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": K,
            "warmup": max(a.warmup, 3), "ms_per_step": dev_ms / K,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64" if a.mode != "mixed" else "f32+f64", "data": "synthetic",
            "config": {
                "workload": label, "config": a.config,
                "mode": a.mode + ("+surrogate" if use_sur else ""),
                "sites_per_edge": nae, "atoms": c0["nlocal"], "ghost_atoms": c0["nghost"],
                "elements": c0["enlocal"], "ghost_elements": c0["enghost"],
                "gauss_points": cfg["gauss_per_element"] * c0["enlocal"],
                "integration_rows": c0["ip_rows"], "sites": sites,
                "interpolated_sites": c0["sites"], "sites_referenced": c0["sites_needed"],
                "atom_list_mean": round(c0["atom_entries"] / max(c0["nlocal"], 1), 2),
                "density_pass_scan_mean": round(c1["density_scan_entries"] / max(c1["nlocal"], 1), 2),
                "short_list_mean": round(c1["short_entries"] / max(c1["nlocal"], 1), 2),
                "ip_list_mean": round(c0["ip_entries"] / max(c0["ip_rows"], 1), 2),
                "ip_scan_mean": round(c1["ip_scan_entries"] / max(c1["ip_rows"], 1), 2),
                "lattice_lines_referenced": lines_all,
                "rebuild": "every 10 steps if any displacement > skin/2 (check yes); a rebuild "
                           "that only atoms trigger keeps the element lists",
                "neighbor_work": neighbor_work,
                "l2": "inputs larger than L2 (positions + lists >> 129 MB resident)",
                "parallelism": f"replicas{ws}",
                "phase_ms_per_step_eager": {k: round(float(v) / K, 4) for k, v in
                                            zip(["integrate+comm", "atom_pass1", "atom_pass2",
                                                 "element", "final"], tm[1:6])},
                "eager_ms_per_step": round(eager_ms / K, 4),
                "graph_steps_timed": graph_steps,
                "wall_s": round(wall, 3)},
            "roofline": {"bound": "hbm", "achieved": dk.get("achieved_GBps"), "peak": peak,
                         "unit": "GB/s", "frac": dk.get("hbm_frac"), "traffic": traffic,
                         "kernel": kernel_names.get(dom, dom),
                         "algorithmic_bytes_per_launch": dk.get("algorithmic_bytes"),
                         "kernel_ms": dk["ms"],
                         "kernel_ms_source": "CUDA events around each launch on its stream, "
                                             "averaged over an equal eager run right after the "
                                             "timed one",
                         "peak_source": peak_src,
                         "kernels": kernels},
            "roofline_fp64": roof64,
            "fp64_peak_flops_measured": fp64_peak,
            "cpu_baseline": cpu,
            "e2e": e2e,
            "clocks": dict(merge_clocks(clk, clk_long), timed_region=clk,
                           window=("samples every 200 ms over the timed region and over the "
                                   f"{n_long} steps of the same workload right before it")),
            "gpu_launches": launches,
            "other_modes": modes,
            "energy_drift": drift,
            "force_error": force_error,
            "surrogate": sur,
            "batched_replicas": c4,
        }
        if "fp64" in modes:
            line["speedup_vs_plain_fp64"] = value / modes["fp64"]["value"]
        print(json.dumps(line), flush=True)
    if s is not None:
        s.close()
    if net is not None:
        net.close()


def run_reference(a, ws, rank):
    if rank != 0:
        return
    from cac_code_gb300 import workloads as W
    tmp = tempfile.mkdtemp(prefix="cacref_bench_")
    eam = W.write_eam(os.path.join(tmp, "Cu_analytic_2000.eam"))
    cores = os.cpu_count() or 1
    steps = max(1, min(a.steps, 200))
    warm = max(3, min(a.warmup, 5))
    val, wall, (s_sites, s_atoms, s_elems) = cpu_leg(SAMPLES[a.config], cores, steps, warm, eam)
    line = {
        "impl": "reference", "metric": METRIC, "value": val, "unit": UNIT, "n_gpus": ws,
        "steps": steps, "warmup": warm, "ms_per_step": None, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": CONFIGS[a.config][1] + ", sampled on the host cores as "
                                                      "independent replicas of its structure",
                   "config": a.config, "parallelism": f"{cores} host processes"},
        "cpu_baseline": {"value": val, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": f"{cores} independent replicas of {s_atoms:,} atoms + "
                                   f"{s_elems:,} elements ({s_sites:,} metric sites), {steps} "
                                   f"timed steps each, {wall:.1f} s; the reference's own binary "
                                   f"is built for x86 here only, so its CPU restatement "
                                   f"(bit-identical outputs) is timed"},
        "e2e": {"value": val, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)




# ----------------------------------------------------------------------------- studies
#
# Longer measurements run on request (--study), one JSON line each; none is
# part of the default run.

def _system(cacg, W, m, cfg, eam, mode, extra=(), damp_elements=0.0):
    import numpy as np
    s = cacg.System(0)
    W.configure_system(s, m, cfg, eam)
    for c in extra:
        s.command(c)
    if damp_elements > 0.0 and m.nelements:
        s.set_group("elems", None, np.ones(m.nelements, dtype=np.int32))
        s.command(f"fix 3 elems viscous {damp_elements!r}")
    s.set_precision(mode)
    s.init()
    s.setup()
    if m.natoms:
        s.neighbor_build()
    if m.nelements:
        s.neighbor_ebuild()
        s.neighbor_nbuild()
    return s


def _rel(f, ref):
    import numpy as np
    f = np.asarray(f, dtype=np.float64).reshape(-1, 3)
    ref = np.asarray(ref, dtype=np.float64).reshape(-1, 3)
    if not ref.size:
        return None
    d = np.linalg.norm(f - ref, axis=1)
    n = np.linalg.norm(ref, axis=1)
    return {"rms_rel": float(np.sqrt((d ** 2).mean() / (n ** 2).mean())),
            "max_rel": float(d.max() / n.max())}


def study_strain(a):
    """C3: 4,017,200 atoms + 200,000 elements under the uniaxial ramp
    (1e8 / s along x = 1e-4 / ps, "fix 2 all deform 1 x erate 1e-4"), run
    in mixed precision and, side by side, in FP64 (FMA).  Every 100 steps:
    the mixed forces against an FP64 evaluation of the same state (atoms and
    nodes), and the two trajectories' energies and virials.  The nodes are
    damped ("fix 3 elems viscous 100", both runs, a relaxation time of about
    11 fs for nodes of 1331 / 8 atomic masses): under the reference's element
    force the isolated elements of this configuration gain kinetic energy
    without bound (node kinetic energy 8 eV -> 2e6 eV by step 1,400 on a
    1,452-atom + 24-element slab in the oracle, and likewise here), deform and
    leave the box; a damping of 10 only delays that to about step 4,000.  The
    atoms are not damped."""
    import numpy as np
    from cac_code_gb300 import build, cacg
    from cac_code_gb300 import workloads as W
    build.build_library()
    eam = W.write_eam(os.path.join(tempfile.mkdtemp(), "Cu_analytic_2000.eam"))
    m, cfg = W.c3_eam()
    sites = W.metric_sites(m, cfg)
    deform = ["fix 2 all deform 1 x erate 1e-4"]
    t0 = time.perf_counter()
    A = _system(cacg, W, m, cfg, eam, cacg.MIXED, deform, damp_elements=100.0)
    B = _system(cacg, W, m, cfg, eam, cacg.FP64, deform, damp_elements=100.0)
    steps = a.study_steps or 5000
    rec, err = [], None
    lo0, hi0 = A.box()
    L0 = hi0[0] - lo0[0]
    k = 0
    try:
        while True:
            A.pair_compute()
            A.pair_ecompute()
            fm = (A.atoms()["f"].copy(), A.elements()["nodef"].copy())
            A.set_precision(cacg.FP64)
            A.pair_compute()
            A.pair_ecompute()
            f64 = (A.atoms()["f"].copy(), A.elements()["nodef"].copy())
            A.set_precision(cacg.MIXED)
            ta, tb = A.thermo(), B.thermo()
            lo, hi = A.box()
            vs = max(np.abs(tb["virial"]).max(), 1e-30)
            rec.append({"step": k, "strain_x": float((hi[0] - lo[0]) / L0 - 1.0),
                        "force_err_atoms": _rel(fm[0], f64[0]),
                        "force_err_nodes": _rel(fm[1], f64[1]),
                        "e_mixed_ev_per_site": ta["etotal"] / sites,
                        "e_fp64_ev_per_site": tb["etotal"] / sites,
                        "de_ev_per_site": (ta["etotal"] - tb["etotal"]) / sites,
                        "de_atoms_ev_per_atom": ((ta["pe_atoms"] + ta["ke_atoms"]) -
                                                 (tb["pe_atoms"] + tb["ke_atoms"])) / m.natoms,
                        "virial_rel_diff": float(np.abs(ta["virial"] - tb["virial"]).max() / vs)})
            if k >= steps:
                break
            A.run(100)
            B.run(100)
            k += 100
    except Exception as ex:  # the synthetic elements can leave the box's range
        err = f"stopped at step {k}: {ex}"
    out = {"study": "strain", "workload": "C3: EAM Cu 4,017,200 atoms + 200,000 elements of "
                                         "11 sites per edge, x ramp 1e8/s, mixed beside FP64, "
                                         "nodes damped (fix viscous 100)",
           "steps": k, "records": rec, "error": err,
           "max_force_err_nodes": max((r["force_err_nodes"]["max_rel"] for r in rec), default=None),
           "max_force_err_atoms": max((r["force_err_atoms"]["max_rel"] for r in rec), default=None),
           "wall_s": round(time.perf_counter() - t0, 1),
           "counts_mixed": A.counts(), "counts_fp64": B.counts()}
    A.close()
    B.close()
    print(json.dumps(out), flush=True)


def study_c1(a):
    """C1 in full (LJ, 16,384 atoms + 64 elements) on the GPU in every
    precision mode: 200 steps (the reference's algorithm stops at step 260,
    when the growing elements' bin grid no longer holds the atoms), after 10
    warm-up steps, site-steps/s from CUDA events; the bit-exact mode computes
    what the reference computes, bit for bit."""
    from cac_code_gb300 import build, cacg
    from cac_code_gb300 import workloads as W
    build.build_library()
    m, cfg = W.c1_lj()
    sites = W.metric_sites(m, cfg)
    steps = a.study_steps or 200
    out = {"study": "c1", "workload": "C1: LJ, 16,384 atoms + 64 elements of 8 sites per edge, "
                                      "T* = 0.1, dt = 0.005, neighbor 2.8 bin, every 10 check yes",
           "sites": sites, "steps": steps, "modes": {}}
    for name, mode in (("exact", cacg.FP64_EXACT), ("fp64", cacg.FP64), ("mixed", cacg.MIXED)):
        s = cacg.System(0)
        try:
            W.configure_system(s, m, cfg)
            s.set_precision(mode)
            s.command("tune loop device")
            s.init()
            s.setup()
            s.neighbor_build()
            s.neighbor_ebuild()
            s.neighbor_nbuild()
            s.run(10)
            s.run(steps - 10)
            ms = float(s.timing()[0])
            c = s.counts()
            out["modes"][name] = {"site_steps_per_s": sites * (steps - 10) / (ms * 1e-3),
                                  "ms_per_step": ms / (steps - 10), "rebuilds": c["rebuilds"]}
        finally:
            s.close()
    print(json.dumps(out), flush=True)


def study_drift(a):
    """Energy of the atom subsystem over NVE steps (atoms and elements do not
    interact, so the atoms alone carry the precision question): the C2 atom
    slab (1,016,400 atoms, free x faces, periodic y, z, 300 K), bit-exact FP64
    against mixed precision with F'(rho) of the atoms from the FP64 or the FP32
    spline, with the configuration's potential (not smoothed: phi(r_c) =
    -0.0189 eV) and with the same potential tapered to zero at the cutoff."""
    import numpy as np
    from cac_code_gb300 import build, cacg
    from cac_code_gb300 import lattice as L
    from cac_code_gb300 import workloads as W
    build.build_library()
    tmp = tempfile.mkdtemp()
    pots = {"plain": W.write_eam(os.path.join(tmp, "Cu_plain.eam")),
            "tapered": os.path.join(tmp, "Cu_tapered.eam")}
    pot = L.AnalyticEAM(taper=1.0)
    L.write_eam_funcfl(pot, pots["tapered"], nrho=2000, nr=2000, r_max=pot.cut * 1.01)
    m, cfg = W.c2_eam(cells=(21, 110, 110), layers=0)
    n = m.natoms
    steps = a.study_steps or 10000
    every = 100
    variants = [("exact", cacg.FP64_EXACT, []), ("mixed", cacg.MIXED, []),
                ("mixed_fp32_fprime", cacg.MIXED, ["tune fprime fp32"])]
    out = {"study": "drift", "atoms": n, "steps": steps, "dt_fs": 1.0, "results": {}}
    t0 = time.perf_counter()
    for pname, pfile in pots.items():
        series = {}
        for name, mode, extra in variants:
            s = _system(cacg, W, m, cfg, pfile, mode, extra)
            e = []
            for k in range(0, steps + 1, every):
                t = s.thermo()
                e.append(t["pe_atoms"] + t["ke_atoms"])
                if k < steps:
                    s.run(every)
            series[name] = np.array(e)
            s.close()
        res = {}
        for name, e in series.items():
            res[name] = {"drift_ev_per_atom": float((e[-1] - e[0]) / n),
                         "max_excursion_ev_per_atom": float(np.abs(e - e[0]).max() / n),
                         "max_diff_from_exact_ev_per_atom": float(np.abs(e - series["exact"]).max() / n),
                         "e_every_100_ev_per_atom": [round(float(v / n), 9) for v in e[::10]]}
        out["results"][pname] = res
    out["wall_s"] = round(time.perf_counter() - t0, 1)
    print(json.dumps(out), flush=True)


def study_surrogate(a):
    """The surrogate's error floor against training-set size, epochs and
    ensemble size, on held-out elements of 11 sites per edge: rms and max
    nodal-force error relative to the force scale, the per-element largest
    error, the ensemble spread, and the fractions within 1e-4."""
    import numpy as np
    from cac_code_gb300 import build
    from cac_code_gb300 import surrogate as S
    from cac_code_gb300 import workloads as W
    build.build_library()
    eam = W.write_eam(os.path.join(tempfile.mkdtemp(), "Cu_analytic_2000.eam"))
    t0 = time.perf_counter()
    xs, ts, info = S.generate(eam, 2000000, seed=11, snapshots=16)
    xv, tv, _ = S.generate(eam, 65536, seed=12, snapshots=4)
    a_ = np.hstack([xs[:400000], np.ones((400000, 1), np.float32)]).astype(np.float64)
    coef, *_ = np.linalg.lstsq(a_, ts[:400000].astype(np.float64), rcond=None)
    lin = np.hstack([xv, np.ones((xv.shape[0], 1))]) @ coef
    rows = [{"model": "linear least squares (400k samples)", **S.force_errors(lin, tv)}]
    for nsamp, members, epochs in ((250000, 4, 10), (1000000, 4, 10), (2000000, 4, 10),
                                   (2000000, 2, 30), (2000000, 4, 30)):
        t1 = time.perf_counter()
        net, loss = S.train(xs[:nsamp], ts[:nsamp], members=members, epochs=epochs, batch=2048,
                            lr=2e-3)
        tt = time.perf_counter() - t1
        pm, psp = net.predict(xv)
        fs = net.normalization()[4]
        per = np.abs(pm - tv).max(axis=1) / fs
        rows.append({"samples": nsamp, "members": members, "epochs": epochs,
                     "train_s": round(tt, 1), "loss": loss, **S.force_errors(pm, tv),
                     "median_element_max_err_rel": float(np.median(per)),
                     "spread_median_rel": float(np.median(psp) / fs),
                     "fraction_err_within_1e-4": float(np.mean(per <= 1e-4)),
                     "fraction_spread_within_1e-4": float(np.mean(psp <= 1e-4 * fs))})
        net.close()
    print(json.dumps({"study": "surrogate", "samples": info, "heldout": int(xv.shape[0]),
                      "rows": rows, "wall_s": round(time.perf_counter() - t0, 1)}), flush=True)


def main():
    a = parse()
    if a.study:
        {"strain": study_strain, "drift": study_drift, "surrogate": study_surrogate,
         "c1": study_c1}[a.study](a)
        return
    ws, rank, local = dist_init()
    if a.impl == "reference":
        run_reference(a, ws, rank)
    else:
        run_ours(a, ws, rank, local)


if __name__ == "__main__":
    main()
