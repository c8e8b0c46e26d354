"""Benchmark: cell-steps/s of the OpenCFD-AMR RHS + RK update path on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--config jet-eb-amr|dmr-amr|react|sod|dmr|cube] [--form fp64|fp32]

Default workload (jet-eb-amr, the largest single-GPU configuration): a Mach 2
planar jet past a z-aligned cylinder (embedded boundary, r = 0.1) in 2x1x1, base
256x128x128 with two refined levels (ratio 2, |d rho| >= 0.05 tagging, regrid
every 2 coarse steps, blocking factor 8, max grid 64: about 2000 boxes of
8^3..64^3), subcycled SSP-RK3 at CFL 0.5, cut boxes in the reference's cut-cell
scheme with its small-cell rescale.  The hierarchy is developed 20 coarse steps
from t = 0 (untimed, FP64), then every form is timed for K coarse steps from
that same state.  A step is one coarse step: regridding when due (host
clustering included), then one CUDA-graph launch that advances every level
with its substeps (ghost fills, coarse-fine interpolation, fused RHS/RK
stages, cut-cell batches, reflux, average-down, CFL).
value  = leaf cell-steps (cells not covered by a finer level, times the
         substeps of their level) / device time of the K timed steps, state
         resident in HBM, L2 flushed between steps (untimed), for the plain FP64
         form (the drop-in); the mixed FP32-flux form is timed the same way and
         reported in config.mixed_form with its own e2e and its L1 error
         against FP64 after 20 coarse steps on identical grids
e2e    = the same through the C ABI from pinned host buffers: every step uploads
         every level's valid cells, advances, downloads every level's valid
         cells (ocfd_amr_copy_valid_in / _out)
--impl reference times the reference algorithm on the host cores (the oracle
         port of its per-box arithmetic, threads over boxes) on the developed
         hierarchy's grids (tests/golden/jet_eb_amr_grids.json, written by
         --write-grids), each timed step a 1/8 sample of every level's boxes.
dmr-amr: double Mach reflection, 1024x256x2 base + 2 levels (blocking 32, max
         grid 128), developed to t = 0.05, both forms timed.
react:   the 128^3 H2/air box with 8 hot spots (9 species, implicit chemistry,
         mixture-averaged transport); plain FP64, binned FP64 and the mixed form
         (headline), then the MLP surrogate trained inside the run.
The single-level configs (sod, dmr, cube) time one level of boxes.
Multi-GPU: independent replicas (the workload does not shard over GPUs here);
value is summed over ranks with the max time.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
for p in (os.path.join(ROOT, "opencfd-amr_gb300"), os.path.join(ROOT, "oracle")):
    sys.path.insert(0, p)

METRIC = "cell-steps/s on 1 GB300, plain FP64 vs mixed/batched form at matched L1 error"
CFL = 0.5


T_DEV = 0.05
L1_STEPS = 20
# the reference's inviscid right-hand side of one cell (c2prim, split and
# five-component WENO-Z per direction, divop), counted on its own headers with
# a counting Real (make -C oracle flops), plus the fused Shu-Osher update
FLOPS_PER_CELL_STAGE = 3233 + 25

# DRAM traffic of each workload's roofline kernel, per cell of one launch:
# (dram__bytes_read.sum + dram__bytes_write.sum) of a launch captured by ncu on the
# same workload and form, divided by the cells that launch processed.  The
# captures and their commands are summarised in profiles/.
NCU_DRAM_BYTES_PER_CELL = {
    # k_rhs_regular<float, 8, 8, 8>, DMR finest level: 310.9 MB over 2,048,000 cells
    ("dmr-amr", "fp32"): 310.9e6 / 2048000,
    # k_rhs_regular<float, 8, 8, 8>, 3D blast 256x256x64: 566.6 MB over 4,194,304 cells
    ("cube", "fp32"): 566.6e6 / 4194304,
    # k_chem_advance_list, 128^3 reacting box: 309 + 126 MB over 2,097,152 cells
    ("react", "chem"): (309e6 + 126e6) / 2097152,
    # k_rhs_regular<double, 8, 8, 8> (the jet's FP64 headline kernel), captured on the 3D blast
    # 256x256x64 (64^3 boxes, as the jet's regular boxes): 414.7 + 140.8 MB over 4,194,304 cells
    ("jet-eb-amr", "fp64"): (414.7e6 + 140.8e6) / 4194304,
    ("cube", "fp64"): (414.7e6 + 140.8e6) / 4194304,
}


def ncu_traffic(workload, form, cells):
    b = NCU_DRAM_BYTES_PER_CELL.get((workload, form))
    return None if b is None else b * cells


def roofline_stage_ms(level, flags, reps=10):
    """Device ms of one RK-stage launch of `level` (CUDA events on its stream),
    inside the NVTX range bench_roofline_stage that an ncu capture of the roofline
    kernel filters on."""
    import torch
    torch.cuda.nvtx.range_push("bench_roofline_stage")
    try:
        return level.profile_stage(flags, reps=reps)
    finally:
        torch.cuda.nvtx.range_pop()


def amr_workload():
    from ocfd import cases
    c = cases.dmr_amr(1024, 256, 2, max_level=2, blocking_factor=32, max_grid=128, n_error_buf=1,
                      refine_dengrad=0.05, regrid_int=2)
    c["name"] = ("Double Mach reflection 1024x256x2 base + 2 levels (ratio 2, |drho|>=0.05 tagging, "
                 "regrid every 2 coarse steps, blocking 32, max grid 128), subcycled SSP-RK3, CFL 0.5, "
                 "timed from t=%.2f" % T_DEV)
    return c


def workload(name):
    from ocfd import cases
    if name == "sod":
        c = cases.sod(512, 64, 4)
        c["name"] = "Sod shock tube 512x64x4 (2D slab), single level, SSP-RK3, CFL 0.5, inviscid"
        c["max_grid"] = (128, 64, 4)
    elif name == "dmr":
        c = cases.dmr(1024, 256, 2)
        c["name"] = "Double Mach reflection base level 1024x256x2, boxes 128x128x2, SSP-RK3, CFL 0.5"
        c["max_grid"] = (128, 128, 2)
    elif name == "cube":
        c = cases.blast3d(256, 256, 64)
        c["name"] = "3D periodic blast 256x256x64, boxes 64x64x64, SSP-RK3, CFL 0.5"
        c["max_grid"] = (64, 64, 64)
    else:
        raise SystemExit("unknown config " + name)
    return c


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return d.get("hbm_gbs", 6800.0), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clock / throttle samples during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        import statistics
        sm, smax, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                smax = max(smax, float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[4:8]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("gloo")
    return world, rank, local


def allreduce_max(x, world):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


# ---------------------------------------------------------------- CPU (oracle)
def cpu_time_steps(c, steps, threads=None):
    """Time `steps` RK3 steps of the oracle port (OpenMP) on the full workload
    domain as one box; returns seconds and cells."""
    import numpy as np
    from oracle import Oracle, BCStruct
    if threads:
        os.environ["OMP_NUM_THREADS"] = str(threads)
    o = Oracle(openmp=True)
    bc = BCStruct()
    bc.lo_bc[:] = list(c["lo_bc"]); bc.hi_bc[:] = list(c["hi_bc"])
    bc.dirichlet_case = c["bc_case"]
    bc.prob_lo[:] = list(c["prob_lo"]); bc.dx[:] = list(c["dx"])
    bc.dom_lo[:] = [0, 0, 0]; bc.dom_hi[:] = [n - 1 for n in c["n"]]
    if c["bc_case"] == 1:
        bc.dmr_left[:] = list(c["case_params"][:5]); bc.dmr_right[:] = list(c["case_params"][5:10])
    if c["bc_case"] == 3:
        bc.jet[:] = list(c["case_params"][:8])
    S = np.ascontiguousarray(c["G"].copy())
    t0 = time.perf_counter()
    o.advance_rk3(bc, S, CFL, steps, form=1)
    dt = time.perf_counter() - t0
    cells = c["n"][0] * c["n"][1] * c["n"][2]
    return dt, cells


def cpu_sample_workload(config):
    """The CPU sample: the workload itself for single-level configs, the base
    grid of the DMR hierarchy (one level, the same boxes' arithmetic) for dmr-amr."""
    if config == "dmr-amr":
        c = workload("dmr")
        c["name"] = amr_workload()["name"]
        c["sample_note"] = "base grid 1024x256x2 only (no refined levels)"
        return c
    if config == "jet-eb-amr":
        from ocfd import cases
        c = cases.jet_eb(*JET_N)
        c["name"] = jet_workload()["name"]
        c["sample_note"] = ("base grid %dx%dx%d only, regular scheme everywhere (no refined levels, the cylinder's "
                            "cut cells not included)" % JET_N)
        return c
    c = workload(config)
    c["sample_note"] = "full workload"
    return c


def run_reference(args, world, rank):
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    if args.config == "react":
        dt, ncs = react_cpu_sample(64, 1, threads)
        v = ncs / dt
        print(json.dumps({
            "impl": "reference", "metric": METRIC, "value": v, "unit": "cell-steps/s", "n_gpus": args.gpus,
            "steps": 1, "warmup": 0, "ms_per_step": dt * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "3D H2/air reacting box (sample 64^3 of the 128^3 workload)", "form": "fp64"},
            "cpu_baseline": {"value": v, "unit": "cell-steps/s", "cores": threads, "kind": "port",
                             "sample": "1 Strang step of a periodic 64^3 sample, oracle restatement (OpenMP)"},
            "e2e": {"value": v, "unit": "cell-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}),
            flush=True)
        return
    c = cpu_sample_workload(args.config)
    # bounded: warm-up steps then K timed steps, each a full-domain RK3 step
    cpu_time_steps(c, max(1, min(args.warmup, 2)), threads)
    dt, cells = cpu_time_steps(c, args.steps, threads)
    v = cells * args.steps / dt
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "cell-steps/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": dt / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": c["name"], "form": "fp64", "cells": cells},
            "cpu_baseline": {"value": v, "unit": "cell-steps/s", "cores": threads, "kind": "port",
                             "sample": "%d RK3 steps of the oracle restatement (OpenMP), %s" % (
                                 args.steps, c["sample_note"])},
            "e2e": {"value": v, "unit": "cell-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------- GPU (ours)
def make_hierarchy(ctx, c, regrid_int):
    from ocfd.amr import Hierarchy
    from ocfd.level import chop_domain
    return Hierarchy(ctx, chop_domain(c["n"], c["max_grid_size"]), c["n"], c["lo_bc"], c["hi_bc"], c["dx"],
                     c["prob_lo"], c["bc_case"], c["case_params"], c["max_level"], c["blocking_factor"],
                     c["max_grid_size"], c["n_error_buf"], regrid_int, c["refine_dengrad"])


def amr_matched_l1(ctx, c, snap, steps=L1_STEPS, mk=None):
    """L1 (sum|a-b| / sum|b| over valid cells, as fcompare) of density and
    pressure between the FP32 and FP64 forms after `steps` coarse steps from the
    same state: the FP64 run regrids every 2 steps and the FP32 run replays its
    grids, so every level compares on identical grids."""
    import numpy as np
    import ocfd
    mk = mk or (lambda ri: make_hierarchy(ctx, c, ri))
    Hd = mk(0)
    Hd.restore(snap)
    grids_at = {}
    for i in range(steps):
        if i > 0 and i % c["regrid_int"] == 0:
            Hd.regrid(0)
            grids_at[i] = Hd.all_grids()[1:]
        Hd.advance(1, CFL, 0)
    t_end = Hd.time()[0]
    ref = [Hd.level_global(l) for l in range(Hd.nlevels())]
    Hd.close()
    Hf = mk(0)
    Hf.restore(snap)
    Hf.set_stop_time(t_end)
    for i in range(steps):
        if i in grids_at:
            Hf.set_grids(grids_at[i])
        Hf.advance(1, CFL, ocfd.FLUX_FP32)
    t_f = Hf.time()[0]
    got = [Hf.level_global(l) for l in range(Hf.nlevels())]
    Hf.close()
    pr = lambda U: 0.4 * (U[4] - 0.5 * (U[1] ** 2 + U[2] ** 2 + U[3] ** 2) / U[0])
    l1 = lambda x, y: float(np.abs(x - y).sum() / np.abs(y).sum())
    out = {"t0": snap["time"], "t": t_end, "t_fp32": t_f, "coarse_steps": steps, "forms": "fp32-flux vs fp64",
           "grids": "fp64 regrids replayed"}
    per = []
    for l, ((a, m), (b, _)) in enumerate(zip(got, ref)):
        A, B = a[:, m], b[:, m]
        per.append({"level": l, "rho": l1(A[0], B[0]), "p": l1(pr(A), pr(B))})
    out["rho"] = per[0]["rho"]            # level 0 after average-down: the composite solution
    out["p"] = per[0]["p"]
    out["per_level"] = per
    out["linf_rho_rel"] = max(float(np.abs(a[0][m] - b[0][m]).max() / np.abs(b[0][m]).max())
                              for (a, m), (b, _) in zip(got, ref))
    return out


def amr_matched_l1_from_start(ctx, c, t_end):
    """The matched error over a whole run: the FP64 form from the initial data
    (t = 0) to t_end, regridding every regrid_int coarse steps, then the FP32
    form from the same initial data replaying those grids with the same stop
    time; L1 of density and pressure per level as amr_matched_l1."""
    import numpy as np
    import ocfd
    runs = []
    grids_at = {}
    for fl in (0, ocfd.FLUX_FP32):
        H = make_hierarchy(ctx, c, 0)
        H.build(c["fab"])
        H.set_stop_time(t_end)
        i = 0
        t0 = time.time()
        while H.time()[0] < t_end * (1.0 - 1e-12):
            if i > 0 and i % c["regrid_int"] == 0:
                if fl == 0:
                    H.regrid(0)
                    grids_at[i] = H.all_grids()[1:]
                elif i in grids_at:
                    H.set_grids(grids_at[i])
            H.advance(1, CFL, fl)
            i += 1
        runs.append(([H.level_global(l) for l in range(H.nlevels())], H.time()[0], i, time.time() - t0))
        H.close()
    (got, t_f, n_f, s_f), (ref, t_d, n_d, s_d) = runs[1], runs[0]
    pr = lambda U: 0.4 * (U[4] - 0.5 * (U[1] ** 2 + U[2] ** 2 + U[3] ** 2) / U[0])
    l1 = lambda x, y: float(np.abs(x - y).sum() / np.abs(y).sum())
    per = []
    for l, ((a, m), (b, _)) in enumerate(zip(got, ref)):
        A, B = a[:, m], b[:, m]
        per.append({"level": l, "rho": l1(A[0], B[0]), "p": l1(pr(A), pr(B))})
    return {"t0": 0.0, "t": t_d, "t_fp32": t_f, "coarse_steps": n_d, "coarse_steps_fp32": n_f,
            "seconds_fp64": s_d, "seconds_fp32": s_f, "forms": "fp32-flux vs fp64",
            "grids": "fp64 regrids replayed", "rho": per[0]["rho"], "p": per[0]["p"], "per_level": per}


JET_N = tuple(int(x) for x in os.environ.get("OCFD_BENCH_JET_BASE", "256,128,128").split(","))
JET_DEV_STEPS = 20
JET_MAX_GRID = 64
JET_BLOCKING = 8
JET_DENGRAD = 0.05
JET_GRIDS = os.path.join(ROOT, "tests", "golden", "jet_eb_amr_grids.json")


def jet_workload():
    from ocfd import cases
    c = cases.jet_eb_amr(*JET_N, max_level=2, blocking_factor=JET_BLOCKING, max_grid=JET_MAX_GRID, n_error_buf=1,
                         refine_dengrad=JET_DENGRAD, regrid_int=2)
    c["name"] = ("Mach 2 planar jet past a z-cylinder EB (r=0.1) in 2x1x1, base %dx%dx%d + 2 levels (ratio 2, "
                 "|drho|>=%g tagging, regrid every 2 coarse steps, blocking %d, max grid %d), KH perturbation "
                 "1e-2 (seed %d), inflow jet / outflow / periodic z, subcycled SSP-RK3, CFL 0.5, cut cells with "
                 "the small-cell rescale, timed after %d coarse steps" % (
                     JET_N + (JET_DENGRAD, JET_BLOCKING, JET_MAX_GRID, c["seed"], JET_DEV_STEPS)))
    return c


def jet_grids_fixture():
    """The developed hierarchy's grids (after JET_DEV_STEPS coarse steps of the
    FP64 form from t = 0), as `bench.py --write-grids` wrote them."""
    with open(JET_GRIDS) as f:
        d = json.load(f)
    return [[(tuple(lo), tuple(hi)) for lo, hi in lev] for lev in d["grids"]], d


def cpu_info():
    model = None
    try:
        with open("/proc/cpuinfo") as f:
            for ln in f:
                k = ln.split(":")[0].strip().lower()
                if k in ("model name", "cpu part", "hardware") and model is None:
                    model = ln.split(":", 1)[1].strip()
    except OSError:
        pass
    return {"nproc": os.cpu_count(), "OMP_NUM_THREADS": os.environ.get("OMP_NUM_THREADS"),
            "cpu": model, "machine": os.uname().machine}


def jet_cpu_sample(grids, fab, parts, nparts, warm=1, threads=None):
    """CPU leg on the jet hierarchy: the oracle's per-box SSP-RK3 work (regular
    WENO-Z boxes, cut-cell boxes, nothing for covered boxes), threads over
    boxes, on interleaved 1/nparts samples of every level's boxes; returns
    (seconds, leaf cell-steps, all cell-steps) summed over `parts`."""
    from hier_sample import HierarchySample, classify
    c = jet_workload()
    classes, geoms = classify(c["eb"], grids, c["dx"], c["prob_lo"])
    hs = HierarchySample(grids, fab, classes, geoms, c["dx"], redistribute=c["eb"]["redistribute"],
                         threads=threads)
    for w in range(warm):
        hs.time(hs.select((parts[0] + nparts // 2 + w) % nparts, nparts * 4))
    sec = leaf = allc = 0
    for p in parts:
        a, b, cc = hs.time(hs.select(p % nparts, nparts))
        sec += a
        leaf += b
        allc += cc
    counts = [[cl.count(k) for k in (0, 1, 2)] for cl in classes]
    return sec, leaf, allc, counts


def run_reference_jet(args, world, rank):
    """--impl reference on the jet hierarchy: the oracle port of the reference's
    per-box arithmetic on the developed hierarchy's grids (committed fixture),
    each timed step a 1/8 interleaved sample of every level's boxes."""
    if rank != 0:
        return
    from ocfd import cases
    grids, meta = jet_grids_fixture()
    c = jet_workload()
    threads = os.cpu_count() or 1

    def fab(l, b):
        lo, hi = grids[l][b]
        return c["fab"](l, lo, hi, tuple(x / (1 << l) for x in c["dx"]))
    nparts = 8
    warm = max(1, min(args.warmup, 2))
    sec, leaf, allc, counts = jet_cpu_sample(grids, fab, range(args.steps), nparts, warm=warm, threads=threads)
    v = leaf / sec
    sample = ("%d steps, each the per-box SSP-RK3 work of 1/%d of every level's boxes (interleaved) of the developed "
              "hierarchy (%s boxes per level, regular/cut/covered %s), WENO-Z / cut-cell right-hand sides and "
              "Shu-Osher updates of the oracle restatement (-O3, serial per box), %d threads over boxes; ghost "
              "exchange, coarse-fine interpolation and reflux not timed" % (
                  args.steps, nparts, [len(g) for g in grids], counts, threads))
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "cell-steps/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": sec / args.steps * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": c["name"], "form": "fp64", "grids": "developed hierarchy (%s)" % (
                os.path.relpath(JET_GRIDS, ROOT)), "boxes": sum(len(g) for g in grids),
                "leaf_cell_steps_sampled": leaf, "all_cell_steps_sampled": allc, "host": cpu_info()},
            "cpu_baseline": {"value": v, "unit": "cell-steps/s", "cores": threads, "kind": "port",
                             "sample": sample},
            "e2e": {"value": v, "unit": "cell-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_ours_jet(args, world, rank, local):
    """The multi-level embedded-boundary workload (Mach 2 jet past a cylinder,
    configs' largest single-GPU case).  Developed JET_DEV_STEPS coarse steps in
    FP64 from t = 0 (untimed), then timed from that state: the plain FP64 form
    (headline: `value`, `e2e`), the mixed FP32-flux form, both in the batched
    graph (regular boxes in one tile-kernel launch per level and stage, cut and
    covered boxes in the cut-cell batch, autotuned), and the reference's
    execution model (FP64 per-box launches from the host)."""
    import numpy as np
    import torch
    import ocfd
    from ocfd.level import eb_desc

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    c = jet_workload()
    ctx = ocfd.Context(device=local)
    eb = eb_desc(center=c["eb"]["center"], radius=c["eb"]["radius"], redistribute=c["eb"]["redistribute"])

    def mk(regrid_int):
        h = make_hierarchy(ctx, c, regrid_int)
        h.set_eb(eb)
        return h
    H = mk(c["regrid_int"])
    H.build(c["fab"])
    H.advance(JET_DEV_STEPS, CFL, 0)            # untimed: bow shock, shear layers (FP64)
    snap = H.snapshot()
    grids = snap["grids"]
    if args.write_grids and rank == 0:
        with open(args.write_grids, "w") as f:
            json.dump({"workload": c["name"], "time": snap["time"],
                       "grids": [[[list(lo), list(hi)] for lo, hi in g] for g in grids]}, f)
            f.write("\n")
    stream = torch.cuda.current_stream(dev)
    l2flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    tuned = {}

    def timed(fl, steps, tune=True):
        H.restore(snap)
        if tune and not (fl & ocfd.PER_BOX):
            H.autotune(fl, reps=3)
            tuned["fp32" if fl & ocfd.FLUX_FP32 else "fp64"] = [H.tuned(l) for l in range(H.nlevels())]
        H.advance(args.warmup, CFL, fl)
        torch.cuda.synchronize()
        barrier(world)
        torch.cuda.synchronize()
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
        leaf = allc = 0
        k0 = H.kernels_launched()
        torch.cuda.nvtx.range_push("bench_timed_jet_%d" % fl)
        for e0, e1 in ev:
            l2flush.fill_(1.0)
            e0.record(stream)
            H.advance(1, CFL, fl)
            e1.record(stream)
            a, b = H.cell_steps()
            leaf += a
            allc += b
        torch.cuda.synchronize()
        torch.cuda.nvtx.range_pop()
        barrier(world)
        ms = allreduce_max(sum(e0.elapsed_time(e1) for e0, e1 in ev), world)
        return ms, leaf, allc, H.kernels_launched() - k0

    pins = {}

    def pin(l, n):
        if l not in pins or pins[l].numel() < n:
            pins[l] = torch.empty(int(n * 1.5) + 1, dtype=torch.float64).pin_memory()
        return pins[l]

    def e2e(fl):
        """every level uploaded from pinned host memory (valid cells, through the
        C ABI), one coarse step, every level downloaded; per step"""
        H.restore(snap)
        H.advance(1, CFL, fl)
        torch.cuda.synchronize()
        for l in range(H.nlevels()):
            H.copy_valid_out(l, pin(l, H.valid_elems(l)), stream)
        torch.cuda.synchronize()
        steps = max(2, min(args.steps, 5))
        h2d = d2h = 0
        e0 = torch.cuda.Event(enable_timing=True); e1 = torch.cuda.Event(enable_timing=True)
        leaf = 0
        e0.record(stream)
        for _ in range(steps):
            for l in range(H.nlevels()):
                H.copy_valid_in(l, pins[l], stream)
                h2d += 8 * H.valid_elems(l)
            H.advance(1, CFL, fl, stream)
            leaf += H.cell_steps()[0]
            for l in range(H.nlevels()):
                n = H.valid_elems(l)
                H.copy_valid_out(l, pin(l, n), stream)
                d2h += 8 * n
        e1.record(stream)
        torch.cuda.synchronize()
        v = leaf * world / (allreduce_max(e0.elapsed_time(e1), world) * 1e-3)
        return {"value": v, "unit": "cell-steps/s", "h2d_bytes_per_step": int(h2d / steps),
                "d2h_bytes_per_step": int(d2h / steps)}

    ms_m, leaf_m, _, k_m = timed(ocfd.FLUX_FP32, args.steps)
    if args.headline_only:
        ms_p, leaf_p, k_p = 1.0, 0, 0
    else:
        ms_p, leaf_p, _, k_p = timed(ocfd.PER_BOX, max(1, min(args.steps, 3)))
    with ClockSampler(local) as clk:
        ms, leaf, allc, kernels = timed(0, args.steps)
    value = leaf * world / (ms * 1e-3)
    v32 = leaf_m * world / (ms_m * 1e-3)
    vpb = leaf_p * world / (ms_p * 1e-3)
    levels = [{"level": l, "boxes": len(H.grids(l)), "cells": H.level(l).cells(),
               "boxes_regular_cut_covered": [H.box_classes(l).count(k) for k in (0, 1, 2)]}
              for l in range(H.nlevels())]
    nbox = sum(x["boxes"] for x in levels)
    sizes = sorted(max(hi[d] - lo[d] + 1 for d in range(3)) for g in grids for lo, hi in g)
    # the dominant kernel (the regular boxes' tile kernel, three quarters of the
    # FP64 step), timed alone on the finest level inside the NVTX range the ncu
    # capture filters on
    fin = H.level(H.nlevels() - 1)
    torch.cuda.nvtx.range_push("bench_roofline_stage")
    reg_ms, reg_cells = fin.profile_regular(0, reps=10)
    reg_ms32, _ = fin.profile_regular(ocfd.FLUX_FP32, reps=10)
    # the whole stage of the finest level: its regular boxes' tile kernel, then
    # the cut and covered boxes' tile kernel
    stage_ms = {"fp64": fin.profile_stage(0, reps=10), "fp32": fin.profile_stage(ocfd.FLUX_FP32, reps=10)}
    torch.cuda.nvtx.range_pop()
    fin_stage = {"cells": fin.cells(), "regular_cells": reg_cells, "cut_and_covered_cells": fin.cells() - reg_cells,
                 "fp64": {"stage_ms": stage_ms["fp64"], "regular_ms": reg_ms,
                          "cut_ms": stage_ms["fp64"] - reg_ms},
                 "fp32": {"stage_ms": stage_ms["fp32"], "regular_ms": reg_ms32,
                          "cut_ms": stage_ms["fp32"] - reg_ms32}}
    hbm_peak, peak_src = peaks()
    fp64 = ctypes.c_double(); fp32 = ctypes.c_double(); fp32x2 = ctypes.c_double()
    ocfd.check(ocfd.load().ocfd_measure_fma_peaks(ctypes.byref(fp64), ctypes.byref(fp32)))
    ocfd.check(ocfd.load().ocfd_measure_ffma2_peak(ctypes.byref(fp32x2)))
    achieved = 120.0 * reg_cells / (reg_ms * 1e-3) / 1e9
    achieved32 = 120.0 * reg_cells / (reg_ms32 * 1e-3) / 1e9
    flops64 = FLOPS_PER_CELL_STAGE * reg_cells / (reg_ms * 1e-3) / 1e9
    flops32 = FLOPS_PER_CELL_STAGE * reg_cells / (reg_ms32 * 1e-3) / 1e9

    e2e64 = e2e(0)
    e2e32 = e2e(ocfd.FLUX_FP32)
    l1err = amr_matched_l1(ctx, c, snap, mk=mk) if rank == 0 and not args.headline_only else None
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        data = snap["data"]

        def fab(l, b):
            off = 0
            for i, (lo, hi) in enumerate(grids[l]):
                n = (5, hi[2] - lo[2] + 9, hi[1] - lo[1] + 9, hi[0] - lo[0] + 9)
                sz = n[0] * n[1] * n[2] * n[3]
                if i == b:
                    return data[l][off:off + sz].reshape(n).copy()
                off += sz
        sec, cleaf, _, counts = jet_cpu_sample(grids, fab, range(8), 8, warm=1)
        cpu = {"value": cleaf / sec, "unit": "cell-steps/s", "cores": os.cpu_count(), "kind": "port",
               "sample": "every box of the timed hierarchy (the GPU state at the start of the timed steps) once, "
                         "in 8 interleaved parts of every level's boxes as the reference arm's steps, per-box "
                         "SSP-RK3 work of the oracle restatement (-O3, serial per box), %d threads over boxes; "
                         "classes regular/cut/covered %s" % (os.cpu_count(), counts),
               "host": cpu_info()}
    grids_match = None
    if os.path.exists(JET_GRIDS):
        try:
            fg, _ = jet_grids_fixture()
            grids_match = [len(a) == len(b) and sorted(a) == sorted(b) for a, b in zip(fg, grids)]
        except (OSError, ValueError, KeyError):
            grids_match = None
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "cell-steps/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": c["name"], "form": "plain FP64 (the drop-in), batched graph, autotuned",
                       "levels": levels, "boxes": nbox, "box_edge_min_max": [sizes[0], sizes[-1]],
                       "refine_dengrad": JET_DENGRAD, "max_grid": JET_MAX_GRID, "blocking_factor": JET_BLOCKING,
                       "leaf_cell_steps_per_coarse_step": leaf / args.steps,
                       "forms_cell_steps_per_s": {"fp64_batched": value, "fp32_flux_batched": v32,
                                                  "fp64_per_box_launches": vpb},
                       "mixed_form": {"value": v32, "e2e": e2e32, "ms_per_step": ms_m / args.steps,
                                      "speedup_over_fp64": v32 / value, "l1_vs_fp64": l1err,
                                      "roofline_regular_kernel": {
                                          "achieved_gbs": achieved32, "frac": achieved32 / hbm_peak,
                                          "ms_per_launch": reg_ms32, "achieved_gflops": flops32,
                                          "fp32_fma_peak_gflops": fp32.value,
                                          "frac_of_fp32_fma_peak": flops32 / fp32.value}},
                       "speedup_batched_over_per_box_fp64": (value / vpb) if vpb else None,
                       "finest_level_stage": fin_stage,
                       "kernels_per_coarse_step": {"fp64_batched": kernels / args.steps,
                                                   "fp64_per_box": k_p / max(1, min(args.steps, 3))},
                       "autotuned_tile_sched_per_level": tuned,
                       "grids_match_reference_arm_fixture": grids_match,
                       "l2": "flushed between timed steps (512 MB write, untimed)",
                       "parallelism": "replicas" if world > 1 else "single GPU"},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                         "frac": achieved / hbm_peak, "peak_source": peak_src,
                         "traffic": ncu_traffic("jet-eb-amr", "fp64", reg_cells),
                         "kernel": "k_rhs_regular<double> fused RK stage over the finest level's regular boxes "
                                   "(%d cells); the FP64 pipe, not HBM, binds it (see fp64)" % reg_cells,
                         "ms_per_launch": reg_ms, "alg_bytes_per_cell": 120,
                         "fp64": {"achieved_gflops": flops64, "peak_gflops": fp64.value,
                                  "frac": flops64 / fp64.value,
                                  "flops_per_cell_stage": FLOPS_PER_CELL_STAGE},
                         "fp32_fma_peak_gflops": fp32.value, "fp32x2_fma_peak_gflops": fp32x2.value},
            "cpu_baseline": cpu,
            "e2e": e2e64,
            "clocks": clk.summary(),
            "gpu_launches": kernels,
        }
        print(json.dumps(line), flush=True)
    H.close()
    ctx.close()


def run_ours_amr(args, world, rank, local):
    import numpy as np
    import torch
    import ocfd

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    flags = ocfd.FLUX_FP32 if args.form == "fp32" else 0
    c = amr_workload()
    ctx = ocfd.Context(device=local)
    H = make_hierarchy(ctx, c, c["regrid_int"])
    H.build(c["fab"])
    while H.time()[0] < T_DEV:                       # untimed: develop the flow
        H.advance(10, CFL, ocfd.FLUX_FP32)
    snap = H.snapshot()
    stream = torch.cuda.current_stream(dev)
    l2flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)

    def timed(fl):
        """K coarse steps of form `fl` from the snapshot, each timed with CUDA
        events (regridding inside the events), L2 flushed between steps
        outside them; returns (ms, leaf cell-steps, all cell-steps, kernels)."""
        H.restore(snap)
        H.advance(args.warmup, CFL, fl)
        torch.cuda.synchronize()
        barrier(world)
        torch.cuda.synchronize()
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
              for _ in range(args.steps)]
        leaf = allc = 0
        k0 = H.kernels_launched()
        torch.cuda.nvtx.range_push("bench_timed_" + ("fp32" if fl else "fp64"))
        for e0, e1 in ev:
            l2flush.fill_(1.0)
            e0.record(stream)
            H.advance(1, CFL, fl)
            e1.record(stream)
            a, b = H.cell_steps()
            leaf += a
            allc += b
        torch.cuda.synchronize()
        torch.cuda.nvtx.range_pop()
        barrier(world)
        ms = allreduce_max(sum(e0.elapsed_time(e1) for e0, e1 in ev), world)
        return ms, leaf, allc, H.kernels_launched() - k0

    other = 0 if flags else ocfd.FLUX_FP32
    ms_o, leaf_o, all_o, _ = timed(other)
    with ClockSampler(local) as clk:
        ms, leaf, allc, kernels = timed(flags)
    value = leaf * world / (ms * 1e-3)
    value_other = leaf_o * world / (ms_o * 1e-3)
    levels = [{"level": l, "boxes": len(H.grids(l)), "cells": H.level(l).cells()} for l in range(H.nlevels())]

    # dominant kernel, timed live: the fused RK-stage kernel on the finest level
    fin = H.level(H.nlevels() - 1)
    stage_ms = roofline_stage_ms(fin, flags)
    fcells = fin.cells()
    alg_bytes = 120.0 * fcells
    hbm_peak, peak_src = peaks()
    achieved = alg_bytes / (stage_ms * 1e-3) / 1e9
    fp64 = ctypes.c_double(); fp32 = ctypes.c_double()
    ocfd.check(ocfd.load().ocfd_measure_fma_peaks(ctypes.byref(fp64), ctypes.byref(fp32)))

    # end to end through the C ABI with host buffers: upload every level,
    # advance one coarse step, download every level
    H.restore(snap)
    H.advance(1, CFL, flags)
    torch.cuda.synchronize()
    pins = {}

    def pin(l, n):
        if l not in pins or pins[l].numel() < n:
            pins[l] = torch.empty(int(n * 1.5) + 1, dtype=torch.float64).pin_memory()
        return pins[l]
    for l in range(H.nlevels()):
        H.copy_valid_out(l, pin(l, H.valid_elems(l)), stream)
    torch.cuda.synchronize()
    e2e_steps = max(2, min(args.steps, 10))
    h2d = d2h = 0
    e0 = torch.cuda.Event(enable_timing=True); e1 = torch.cuda.Event(enable_timing=True)
    e2e_leaf = 0
    e0.record(stream)
    for _ in range(e2e_steps):
        for l in range(H.nlevels()):
            n = H.valid_elems(l)
            H.copy_valid_in(l, pins[l], stream)
            h2d += 8 * n
        H.advance(1, CFL, flags, stream)
        e2e_leaf += H.cell_steps()[0]
        for l in range(H.nlevels()):
            n = H.valid_elems(l)
            H.copy_valid_out(l, pin(l, n), stream)
            d2h += 8 * n
    e1.record(stream)
    torch.cuda.synchronize()
    e2e_ms = allreduce_max(e0.elapsed_time(e1), world)
    e2e_value = e2e_leaf * world / (e2e_ms * 1e-3)

    if rank != 0:
        l1err = None
    elif args.l1_time:
        l1err = amr_matched_l1_from_start(ctx, c, args.l1_time)
    else:
        l1err = amr_matched_l1(ctx, c, snap)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        cs = cpu_sample_workload("dmr-amr")
        cpu_steps = 2
        dt, ccells = cpu_time_steps(cs, cpu_steps, os.cpu_count())
        cpu = {"value": ccells * cpu_steps / dt, "unit": "cell-steps/s", "cores": os.cpu_count(), "kind": "port",
               "sample": "%d RK3 steps of the oracle restatement (OpenMP), %s" % (cpu_steps, cs["sample_note"])}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "cell-steps/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64" if args.form == "fp64" else "f32-flux/f64-state", "data": "synthetic",
            "config": {"workload": c["name"], "form": args.form, "levels": levels,
                       "leaf_cell_steps_per_coarse_step": leaf / args.steps,
                       "all_cell_steps_per_coarse_step": allc / args.steps,
                       "l1_vs_other_form": l1err,
                       "forms_cell_steps_per_s": {args.form: value, ("fp64" if flags else "fp32"): value_other},
                       "speedup_fp32_over_fp64": (value / value_other) if flags else (value_other / value),
                       "l2": "flushed between timed steps (512 MB write, untimed)",
                       "parallelism": "replicas" if world > 1 else "single GPU"},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                         "frac": achieved / hbm_peak, "peak_source": peak_src,
                         "traffic": ncu_traffic("dmr-amr", args.form, fcells),
                         "kernel": "k_rhs_regular fused RK stage, finest level (%d cells)" % fcells,
                         "ms_per_launch": stage_ms, "alg_bytes_per_cell": 120,
                         "fp64_fma_peak_gflops": fp64.value, "fp32_fma_peak_gflops": fp32.value},
            "cpu_baseline": cpu,
            "e2e": {"value": e2e_value, "unit": "cell-steps/s",
                    "h2d_bytes_per_step": int(h2d / e2e_steps), "d2h_bytes_per_step": int(d2h / e2e_steps)},
            "clocks": clk.summary(),
            "gpu_launches": kernels,
        }
        print(json.dumps(line), flush=True)
    H.close()
    ctx.close()


REACT_N = 128
REACT_DT = 1e-8


def react_cpu_sample(n=64, steps=1, threads=None):
    """CPU leg of the reacting workload: the oracle port (OpenMP) of one Strang
    step (4 + 4 chemistry substeps, RK2 with the multispecies RHS, species
    renormalisation) on a periodic n^3 sample with the workload's cell size.
    Returns (seconds, cells x steps)."""
    import numpy as np
    from oracle import BCStruct, Oracle
    from ocfd.cases import PHI1_AIR_X, hot_spot_temperature
    if threads:
        os.environ["OMP_NUM_THREADS"] = str(threads)
    o = Oracle(openmp=True)
    NG = 4
    T, dxs, _ = hot_spot_temperature(n, 0.01 * n / REACT_N)
    dx = (dxs, dxs, dxs)
    y = o.ckxty(np.array(PHI1_AIR_X))
    S = np.zeros((5,) + T.shape)
    sp = np.zeros((9,) + T.shape)
    flatT = T.ravel()
    for c in range(flatT.size):
        rho = o.ckrhoy(101325.0, flatT[c], y)
        r = rho * y
        idx = np.unravel_index(c, T.shape)
        S[(0,) + idx] = rho
        S[(4,) + idx] = o.ckubms(flatT[c], r)
        sp[(slice(None),) + idx] = r
    bc = BCStruct()
    bc.dx[:] = list(dx)
    bc.dom_hi[:] = [n - 1] * 3
    inner = (slice(None), slice(NG, -NG), slice(NG, -NG), slice(NG, -NG))
    dt = REACT_DT

    def chem_half(S, sp):
        for _ in range(4):
            a = np.ascontiguousarray(S[inner].reshape(5, -1))
            b = np.ascontiguousarray(sp[inner].reshape(9, -1))
            o.chem_advance(a, b, 0.5 * dt / 4)
            S[inner] = a.reshape(S[inner].shape)
            sp[inner] = b.reshape(sp[inner].shape)
    t0 = time.perf_counter()
    for _ in range(steps):
        chem_half(S, sp)
        U0, V0 = S.copy(), sp.copy()
        Us, Vs = S, sp
        for a, b in ((0.0, 1.0), (0.5, 0.5)):
            o.fill_ghosts(bc, Us)
            o.fill_ghosts(bc, Vs)
            dS, dSs, *_ = o.rhs_chem(Us, Vs, tuple(1.0 / x for x in dx), do_visc=True)
            Un, Vn = Us.copy(), Vs.copy()
            Un[inner] = a * U0[inner] + b * (Us[inner] + dt * dS)
            Vn[inner] = a * V0[inner] + b * (Vs[inner] + dt * dSs)
            Us, Vs = Un, Vn
        S, sp = Us, Vs
        chem_half(S, sp)
        a = np.ascontiguousarray(S[inner].reshape(5, -1))
        b = np.ascontiguousarray(sp[inner].reshape(9, -1))
        o.spec_renorm(a, b)
        sp[inner] = b.reshape(sp[inner].shape)
    return time.perf_counter() - t0, n ** 3 * steps


SUR_GUARD_SWEEP = (0.0, 1.0, 0.1, 0.01, 0.001)
# the per-output criterion relative to each Y_k itself (a floor far below the
# 1e-11 radical mass fractions of the induction phase)
SUR_Y_FLOOR = 1e-20


def react_surrogate_form(args, world, ctx, make, stream, l2flush, ref, cells, same_steps, value_plain):
    """The learned chemistry form of the reacting workload: the MLP surrogate
    (12 -> 128 x4 GELU -> 10, BF16 on tcgen05) trained here on ~1e7 samples of
    the FP64 implicit substep taken from 0D constant-pressure ignition
    trajectories (T0 1000-2500 K, phi 0.5-2, p 0.8-10 atm), then embedded in the
    reacting level with the guard's FP64 fallback.  The per-output criterion of
    the guard (no Y_n may change by more than dy_rel_max x max(Y_n, SUR_Y_FLOOR)
    in a substep) is swept over SUR_GUARD_SWEEP (0 = off); for each setting the
    fallback rate, the cell-steps/s and the L1 error in rho, p, T, Y_OH, Y_H2O
    against the plain FP64 run after the same steps.  matched_1e-4 is the
    loosest setting whose rho, p and Y_OH errors are all <= 1e-4 (None when
    none is)."""
    import numpy as np
    import torch
    from ocfd import surrogate
    from ocfd._abi import check, load

    t0 = time.time()
    X, T = surrogate.generate(ctx, n_traj=32768, n_snap=300, seed=20261203, mode="pressure")
    gen_s = time.time() - t0
    sur, rep = surrogate.train(ctx, X, T, epochs=args.sur_epochs, batch=8192, lr=2e-3, seed=2)
    del X, T
    torch.cuda.empty_cache()
    substeps = 8 * same_steps
    props = lambda U: surrogate.cells_props(ctx, torch.as_tensor(U.reshape(14, -1), device="cuda").contiguous())
    pa = props(ref)
    l1 = lambda x, y: float((x - y).abs().sum() / y.abs().sum())

    sweep = []
    for d in SUR_GUARD_SWEEP:
        guard = sur.guard.with_dy_rel(d, SUR_Y_FLOOR)
        R = make(True, f32=True)
        check(load().ocfd_react_set_surrogate(R.h, sur.net.h, ctypes.byref(guard)), "set_surrogate")
        R.advance(args.warmup)
        torch.cuda.synchronize()
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
              for _ in range(args.steps)]
        for e0, e1 in ev:
            l2flush.fill_(1.0)
            e0.record(stream)
            R.advance(1)
            e1.record(stream)
        torch.cuda.synchronize()
        ms = allreduce_max(sum(e0.elapsed_time(e1) for e0, e1 in ev), world)
        fb = ctypes.c_int64()
        check(load().ocfd_react_fallbacks(R.h, ctypes.byref(fb), None), "fallbacks")
        got = R.level.get_global()
        R.close()
        pb = props(got)
        v = cells * args.steps * world / (ms * 1e-3)
        sweep.append({"dy_rel_max": d, "y_floor": SUR_Y_FLOOR, "cell_steps_per_s": v,
                      "speedup_over_fp64_plain": v / value_plain,
                      "fallback_rate": fb.value / float(cells * substeps), "fallback_cells": int(fb.value),
                      "l1_vs_fp64_after_steps": {
                          "steps": same_steps, "T": l1(pb[0], pa[0]), "Y_OH": l1(pb[2 + 5], pa[2 + 5]),
                          "Y_H2O": l1(pb[2 + 2], pa[2 + 2]), "p": l1(pb[1], pa[1]),
                          "rho": float(np.abs(got[0] - ref[0]).sum() / np.abs(ref[0]).sum())}})
    matched = None
    for e in sweep:
        err = e["l1_vs_fp64_after_steps"]
        if max(err["rho"], err["p"], err["Y_OH"]) <= 1e-4:
            matched = e
            break
    base = sweep[0]
    return {
        "form": "mixed FP32 faces + MLP surrogate chemistry (FP64 fallback on guard failure)",
        "cell_steps_per_s": base["cell_steps_per_s"],
        "fallback_rate": base["fallback_rate"],
        "fallback_cells": base["fallback_cells"], "cell_substeps": int(cells * substeps),
        "l1_vs_fp64_after_steps": base["l1_vs_fp64_after_steps"],
        "guard_sweep": sweep,
        "matched_1e-4": matched,
        "training": {"data": "0D constant-pressure ignition trajectories", "samples": rep["samples"],
                     "generate_seconds": gen_s, "train_seconds": rep["train_seconds"],
                     "epochs": rep["epochs"], "val_loss": rep["val_loss"], "val_rel_l1_dT": rep["val_rel_l1_dT"],
                     "val_rel_l1_dY_OH": rep["val_rel_l1_dY_OH"]},
    }


def run_ours_react(args, world, rank, local):
    """The reacting workload: 128^3 periodic H2/air with 8 hot spots, Strang chemistry around
    the RK2 multispecies flow step, dt = 1e-8 s."""
    import numpy as np
    import torch
    import ocfd
    from ocfd.cases import react_cube
    from ocfd.level import chop_domain
    from ocfd.react import Reactor

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    ctx = ocfd.Context(device=local)
    case = react_cube(ctx, n=REACT_N)
    n = case["n"]
    boxes = chop_domain(n, 64)
    cells = n[0] * n[1] * n[2]
    stream = torch.cuda.current_stream(dev)
    l2flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)

    def make(binned, rk=2, f32=False):
        R = Reactor(ctx, boxes, tuple(x - 1 for x in n), case["dx"], dt=REACT_DT, rk_order=rk, chem_substeps=4,
                    visc=True, binned=binned, flux_fp32=f32)
        R.level.set_global(case["G"])
        return R

    def timed(binned, f32=False):
        R = make(binned, f32=f32)
        R.advance(args.warmup)
        torch.cuda.synchronize()
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
        torch.cuda.nvtx.range_push("bench_timed_react_%s%s" % ("binned" if binned else "plain", "_f32" if f32 else ""))
        for e0, e1 in ev:
            l2flush.fill_(1.0)
            e0.record(stream)
            R.advance(1)
            e1.record(stream)
        torch.cuda.synchronize()
        torch.cuda.nvtx.range_pop()
        ms = allreduce_max(sum(e0.elapsed_time(e1) for e0, e1 in ev), world)
        return ms, R

    ms_plain, Rp = timed(False)
    ms_bin, Rb = timed(True)
    with ClockSampler(local) as clk:
        ms_mix, Rm = timed(True, f32=True)
    value = cells * args.steps * world / (ms_mix * 1e-3)
    value_bin = cells * args.steps * world / (ms_bin * 1e-3)
    value_plain = cells * args.steps * world / (ms_plain * 1e-3)
    same_steps = args.warmup + args.steps
    a = Rp.level.get_global()
    b = Rb.level.get_global()
    mix = Rm.level.get_global()
    Rm.close()
    identical = bool(np.array_equal(a, b))
    from ocfd import surrogate as _sur
    props = lambda U: _sur.cells_props(ctx, torch.as_tensor(U.reshape(14, -1), device="cuda").contiguous())
    pa, pm = props(a), props(mix)
    l1t = lambda x, y: float((x - y).abs().sum() / y.abs().sum())
    mixed_err = {"steps": same_steps, "rho": float(np.abs(mix[0] - a[0]).sum() / np.abs(a[0]).sum()),
                 "p": l1t(pm[1], pa[1]), "T": l1t(pm[0], pa[0]), "Y_OH": l1t(pm[7], pa[7]),
                 "Y_H2O": l1t(pm[4], pa[4])}
    chem_ms = Rb.profile_chem(reps=3)
    launches = Rb.launches_per_step()
    Rp.close()
    # RK3 beside the reference's RK2 after the same number of steps
    R3 = make(False, rk=3)
    R3.advance(same_steps)
    c3 = R3.level.get_global()
    R3.close()
    y = lambda U, s: U[5 + s] / U[0]
    l1 = lambda x, y_: float(np.abs(x - y_).sum() / np.abs(y_).sum())
    rk3_vs_rk2 = {"rho": l1(c3[0], a[0]), "Y_OH": l1(y(c3, 5), y(a, 5)), "Y_H2O": l1(y(c3, 2), y(a, 2)),
                  "steps": same_steps}

    sur_rep = react_surrogate_form(args, world, ctx, make, stream, l2flush, a, cells, same_steps, value_plain) \
        if not args.no_surrogate else None

    # end to end: upload the state, one step, download, per step
    flat = Rb.level.copy_valid_out()
    pin = torch.from_numpy(flat).pin_memory()
    out = torch.empty_like(pin).pin_memory()
    e2e_steps = max(2, min(args.steps, 5))
    e0 = torch.cuda.Event(enable_timing=True); e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(e2e_steps):
        Rb.level.lib.ocfd_level_copy_valid_in(Rb.level.h, ctypes.c_void_p(pin.data_ptr()),
                                              ctypes.c_void_p(stream.cuda_stream))
        Rb.advance(1, stream)
        Rb.level.lib.ocfd_level_copy_valid_out(Rb.level.h, ctypes.c_void_p(out.data_ptr()),
                                               ctypes.c_void_p(stream.cuda_stream))
    e1.record(stream)
    torch.cuda.synchronize()
    e2e_value = cells * e2e_steps * world / (allreduce_max(e0.elapsed_time(e1), world) * 1e-3)
    Rb.close()

    hbm_peak, peak_src = peaks()
    fp64 = ctypes.c_double(); fp32 = ctypes.c_double()
    ocfd.check(ocfd.load().ocfd_measure_fma_peaks(ctypes.byref(fp64), ctypes.byref(fp32)))
    achieved = 192.0 * cells / (chem_ms * 1e-3) / 1e9

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        dt_cpu, ncs = react_cpu_sample(64, 1, os.cpu_count())
        cpu = {"value": ncs / dt_cpu, "unit": "cell-steps/s", "cores": os.cpu_count(), "kind": "port",
               "sample": "1 Strang step (4+4 chemistry substeps, RK2 multispecies flow, renormalisation) of a "
                         "periodic 64^3 sample with the workload's cell size, oracle restatement (OpenMP)"}
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "cell-steps/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_mix / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32-flux/f64-state", "data": "synthetic",
            "config": {"workload": "3D H2/air reacting box 128^3 periodic, 9 species / 19 reactions, phi=1, 1 atm, "
                                   "1200 K + 8 hot spots (seed %d, edge 1 cm), mixture-averaged transport, "
                                   "Strang chemistry (4+4 substeps), RK2, dt=1e-8 s" % case["seed"],
                       "form": "mixed: FP32 split + WENO-Z faces, binned batched FP64 chemistry",
                       "forms_cell_steps_per_s": {"mixed_binned": value, "fp64_binned": value_bin,
                                                  "fp64_plain": value_plain},
                       "speedup_mixed_over_fp64_plain": value / value_plain,
                       "speedup_binned_over_plain_fp64": value_bin / value_plain,
                       "binned_identical_to_plain": identical,
                       "l1_mixed_vs_fp64": mixed_err,
                       "rk3_vs_rk2_l1": rk3_vs_rk2, "surrogate": sur_rep, "boxes": len(boxes), "cells": cells,
                       "l2": "flushed between timed steps (512 MB write, untimed)"},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                         "frac": achieved / hbm_peak, "peak_source": peak_src,
                         "traffic": ncu_traffic("react", "chem", cells),
                         "kernel": "k_chem_advance_list (one chemistry substep)", "ms_per_launch": chem_ms,
                         "alg_bytes_per_cell": 192, "fp64_fma_peak_gflops": fp64.value},
            "cpu_baseline": cpu,
            "e2e": {"value": e2e_value, "unit": "cell-steps/s", "h2d_bytes_per_step": int(flat.nbytes),
                    "d2h_bytes_per_step": int(flat.nbytes)},
            "clocks": clk.summary(),
            "gpu_launches": launches * args.steps,
        }
        print(json.dumps(line), flush=True)
    ctx.close()


def run_ours(args, world, rank, local):
    import numpy as np
    import torch
    import ocfd
    from ocfd.level import Level, chop_domain

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    flags = ocfd.FLUX_FP32 if args.form == "fp32" else 0
    c = workload(args.config)
    ctx = ocfd.Context(device=local)
    boxes = chop_domain(c["n"], c["max_grid"])
    lev = Level(ctx, boxes, tuple(n - 1 for n in c["n"]), c["lo_bc"], c["hi_bc"], c["dx"],
                c["prob_lo"], c["bc_case"], c["case_params"])
    cells = lev.cells()
    flat = np.ascontiguousarray(lev.pack(c["G"]))
    stream = torch.cuda.current_stream(dev)
    lev.copy_in(flat)
    l2flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)

    def timed(fl):
        """K steps of form `fl`, each step timed with CUDA events, L2 flushed between
        steps outside the events; returns the summed device time in ms."""
        lev.copy_in(flat)
        lev.advance(args.warmup, CFL, fl)
        torch.cuda.synchronize()
        barrier(world)
        torch.cuda.synchronize()
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
              for _ in range(args.steps)]
        for e0, e1 in ev:
            l2flush.fill_(1.0)            # untimed: evicts the state from L2
            e0.record(stream)
            lev.advance(1, CFL, fl)
            e1.record(stream)
        torch.cuda.synchronize()
        barrier(world)
        return allreduce_max(sum(e0.elapsed_time(e1) for e0, e1 in ev), world)

    other = 0 if flags else ocfd.FLUX_FP32
    ms_other = timed(other)
    with ClockSampler(local) as clk:
        ms_max = timed(flags)
    value = cells * args.steps * world / (ms_max * 1e-3)
    value_other = cells * args.steps * world / (ms_other * 1e-3)

    # dominant kernel, timed live: the fused RK-stage kernel (stage 2)
    stage_ms = roofline_stage_ms(lev, flags)
    alg_bytes = 120.0 * cells          # read U_s and U_0, write U_out (5 doubles each)
    hbm_peak, peak_src = peaks()
    achieved = alg_bytes / (stage_ms * 1e-3) / 1e9
    fp64 = ctypes.c_double(); fp32 = ctypes.c_double()
    ocfd.check(ocfd.load().ocfd_measure_fma_peaks(ctypes.byref(fp64), ctypes.byref(fp32)))

    # end to end through the C ABI with host buffers (the valid cells)
    lev.copy_in(flat)
    vflat = lev.copy_valid_out()
    pin = torch.from_numpy(vflat).pin_memory()
    out = torch.empty_like(pin).pin_memory()
    e2e_steps = max(2, min(args.steps, 10))
    lev.copy_valid_in(pin, stream)
    lev.advance(1, CFL, flags)
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True); e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(e2e_steps):
        lev.lib.ocfd_level_copy_valid_in(lev.h, ctypes.c_void_p(pin.data_ptr()), ctypes.c_void_p(stream.cuda_stream))
        lev.advance(1, CFL, flags, stream)
        lev.lib.ocfd_level_copy_valid_out(lev.h, ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(stream.cuda_stream))
    e1.record(stream)
    torch.cuda.synchronize()
    e2e_ms = allreduce_max(e0.elapsed_time(e1) / e2e_steps, world)
    e2e_value = cells * world / (e2e_ms * 1e-3)

    # matched error: the other form from the same initial state to the same time
    l1err = None
    if rank == 0:
        l1err = matched_l1(ctx, c, boxes, flags)

    # the regular tile kernel of one stage for every tile shape (the pencil
    # shapes 0-5, and in the FP32-flux form the TMA-staged shapes 6-8), one-CTA-
    # per-tile schedule (last: it leaves the level on the last shape)
    # (each inside the NVTX range bench_tile_<index> for ncu)
    from ocfd._abi import OcfdError
    tile_ms = {}
    for t in range(9):
        try:
            lev.set_schedule(t, 0)
            torch.cuda.nvtx.range_push("bench_tile_%d" % t)
            try:
                tile_ms[str(t)] = lev.profile_regular(flags, reps=10)[0]
            finally:
                torch.cuda.nvtx.range_pop()
        except OcfdError:
            tile_ms[str(t)] = None

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        cpu_steps = 2
        dt, ccells = cpu_time_steps(c, cpu_steps, os.cpu_count())
        cpu = {"value": ccells * cpu_steps / dt, "unit": "cell-steps/s", "cores": os.cpu_count(),
               "kind": "port", "sample": "%d full-domain RK3 steps of the oracle restatement (OpenMP)" % cpu_steps}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "cell-steps/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_max / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64" if args.form == "fp64" else "f32-flux/f64-state", "data": "synthetic",
            "config": {"workload": c["name"], "form": args.form, "cells": cells, "boxes": len(boxes),
                       "l1_vs_other_form": l1err,
                       "forms_cell_steps_per_s": {args.form: value, ("fp64" if flags else "fp32"): value_other},
                       "speedup_fp32_over_fp64": (value / value_other) if flags else (value_other / value),
                       "regular_kernel_ms_per_tile_shape": tile_ms,
                       "l2": "flushed between timed steps (512 MB write, untimed)",
                       "parallelism": "replicas" if world > 1 else "single GPU"},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                         "frac": achieved / hbm_peak, "peak_source": peak_src,
                         "traffic": ncu_traffic(args.config, args.form, cells),
                         "kernel": "k_rhs_regular fused RK stage", "ms_per_launch": stage_ms,
                         "alg_bytes_per_cell": 120,
                         "fp64_fma_peak_gflops": fp64.value, "fp32_fma_peak_gflops": fp32.value},
            "cpu_baseline": cpu,
            "e2e": {"value": e2e_value, "unit": "cell-steps/s",
                    "h2d_bytes_per_step": int(vflat.nbytes), "d2h_bytes_per_step": int(vflat.nbytes)},
            "clocks": clk.summary(),
            "gpu_launches": lev.launches_per_step(flags) * args.steps,
        }
        print(json.dumps(line), flush=True)
    lev.close()
    ctx.close()


def matched_l1(ctx, c, boxes, flags, steps=40):
    """L1 (sum|a-b| / sum|b|, as fcompare) of density and pressure between this
    form and the other one after `steps` CFL steps of the FP64 form, both
    stopped at the same time."""
    import numpy as np
    import ocfd
    from ocfd.level import Level
    out = {}
    t_end = None
    for f in (0, ocfd.FLUX_FP32):
        lev = Level(ctx, boxes, tuple(n - 1 for n in c["n"]), c["lo_bc"], c["hi_bc"], c["dx"],
                    c["prob_lo"], c["bc_case"], c["case_params"])
        lev.set_global(c["G"])
        if t_end is None:
            lev.advance(steps, CFL, f)
            t_end = lev.time()[0]
        else:
            lev.set_stop_time(t_end)
            lev.advance(4 * steps, CFL, f)
        out[f] = lev.get_global()
        lev.close()
    a, b = out[ocfd.FLUX_FP32], out[0]
    pr = lambda U: 0.4 * (U[4] - 0.5 * (U[1] ** 2 + U[2] ** 2 + U[3] ** 2) / U[0])
    l1 = lambda x, y: float(np.abs(x - y).sum() / np.abs(y).sum())
    return {"rho": l1(a[0], b[0]), "p": l1(pr(a), pr(b)), "t": t_end, "steps_fp64": steps,
            "forms": "fp32-flux vs fp64"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", default="jet-eb-amr",
                    choices=["jet-eb-amr", "dmr-amr", "react", "sod", "dmr", "cube"])
    ap.add_argument("--form", default="fp64", choices=["fp64", "fp32"],
                    help="dmr-amr and the single-level configs: headline form (the other form is timed too and "
                         "reported in config); jet-eb-amr always heads with FP64")
    ap.add_argument("--write-grids", default=None,
                    help="jet-eb-amr: write the developed hierarchy's grids (the reference arm's fixture) here")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-surrogate", action="store_true", help="react: skip the surrogate form")
    ap.add_argument("--headline-only", action="store_true",
                    help="jet-eb-amr: time the headline form only (no other forms, no L1 run); for profiling")
    ap.add_argument("--sur-epochs", type=int, default=6, help="react: surrogate training epochs")
    ap.add_argument("--l1-time", type=float, default=None,
                    help="dmr-amr: matched L1 of a whole run from t = 0 to this time (the double Mach reflection's end time is 0.2) in "
                         "place of the 20 coarse steps from the developed state")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    world, rank, local = dist_setup()
    if args.impl == "reference":
        if args.config == "jet-eb-amr":
            run_reference_jet(args, world, rank)
        else:
            run_reference(args, world, rank)
    elif args.config == "dmr-amr":
        run_ours_amr(args, world, rank, local)
    elif args.config == "react":
        run_ours_react(args, world, rank, local)
    elif args.config == "jet-eb-amr":
        run_ours_jet(args, world, rank, local)
    else:
        run_ours(args, world, rank, local)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
