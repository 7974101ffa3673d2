"""Benchmark: two-photon luminosity / cross-section tables and event sampling.

Workload (default "c2"): the full-grid Pb-Pb configuration -- Woods-Saxon
form-factor flux (FLUX_POINT 0), gamma-gamma -> tau tau (PROC_ID 15), XNXN
breakup (BREAKUP_MODE 2), m in [3.56, 50] GeV x 1001 bins, y in [-6, 6] x 121
bins, z x 100 bins, pT > 1 GeV and |eta| < 2.4, 1e7 accepted events.  The
inputs are this parameter set (no dataset is involved).

One step = the complete table build of UpcGenerator::init on the GPU: nuclear
tables (form factor, G_AA, breakup), the 121,121-cell luminosity, the nuclear
cross section and the sampling CDFs.  It is timed with CUDA events on the
library's stream, after a 256 MB L2 flush.  `value` is cells / s of the fast
form (tensor-core contraction); `parity` compares its table, every cell,
with the committed oracle fixture (the converged flux integral and the
reference's own quadrature), and the plain FP64 path is timed in the same run.
The 1e7-event sampling is a second timed phase (events_per_s).  Extra keys:
the CPU restatement's phases (cpu_baseline), the 64-configuration batched
scan (c5_scan) and the event-file rates (event_files).

--impl reference times the CPU restatement of the reference (oracle/, C++ with
OpenMP on every host core) on a bounded sample of the same workload.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOADS = {
    "c2": {"NUCLEUS_Z": 82, "NUCLEUS_A": 208, "WS_R": 6.68, "WS_A": 0.447, "SQRTS": 5020,
           "PROC_ID": 15, "LEP_A": 0, "FLUX_POINT": 0, "BREAKUP_MODE": 2,
           "MMIN": 3.56, "MMAX": 50, "BINS_M": 1001, "YMIN": -6, "YMAX": 6, "BINS_Y": 121,
           "ZMIN": -1, "ZMAX": 1, "BINS_Z": 100, "DO_PT_CUT": 1, "PT_MIN": 1,
           "DO_ETA_CUT": 1, "ETA_MIN": -2.4, "ETA_MAX": 2.4, "SEED": 1},
    "c1": {"NUCLEUS_Z": 82, "NUCLEUS_A": 208, "WS_R": 6.68, "WS_A": 0.447, "SQRTS": 5020,
           "PROC_ID": 13, "LEP_A": 0, "FLUX_POINT": 1, "BREAKUP_MODE": 1,
           "MMIN": 3.56, "MMAX": 50, "BINS_M": 201, "YMIN": -6, "YMAX": 6, "BINS_Y": 61,
           "ZMIN": -1, "ZMAX": 1, "BINS_Z": 100, "SEED": 1},
}
EVENTS = {"c2": 10_000_000, "c1": 100_000, "c5": 1_000_000_000}


def c5_configs():
    """The batched scan: Pb, Au, Xe, O x sqrt(s) 200/5020/5360/5440 GeV x
    breakup modes 1-4, ALP (M = 1 GeV, width 0.01), m-bins cycling through
    201/501/1001, 121 y-bins."""
    nuclei = [(82, 208, 6.68, 0.447), (79, 197, 6.38, 0.535), (54, 129, 5.36, 0.59),
              (8, 16, 2.608, 0.513)]
    out, k = [], 0
    for z, a, r, d in nuclei:
        for sq in (200, 5020, 5360, 5440):
            for mode in (1, 2, 3, 4):
                out.append({"NUCLEUS_Z": z, "NUCLEUS_A": a, "WS_R": r, "WS_A": d, "SQRTS": sq,
                            "PROC_ID": 51, "ALP_MASS": 1, "ALP_WIDTH": 0.01, "BREAKUP_MODE": mode,
                            "BINS_M": (201, 501, 1001)[k % 3], "BINS_Y": 121, "SEED": 1 + k})
                k += 1
    return out
METRIC = "gamma-gamma lumi (m,y) cells/s"
FAST_GRID_P = 1024  # radial grid of the fast form (csrc/upcg_fast.cu)


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            return json.load(f), "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}, "fallback"


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index, self.rows, self.proc, self.thread = index, [], None, None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "50"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (OSError, FileNotFoundError):
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 7:
                self.rows.append(parts)

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)

        def num(v):
            try:
                return float(v)
            except ValueError:
                return None
        sm = [num(r[0]) for r in self.rows if num(r[0]) is not None]
        mx = [num(r[1]) for r in self.rows if num(r[1]) is not None]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4) if r[3 + i] == "Active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(self.rows)}


def workload_name(workload, params, nm, ny, nev):
    """The config.workload string both arms print for a single-table workload."""
    return (f"{workload}: Pb-Pb {nm}x{ny} (m,y) cells, FLUX_POINT {params['FLUX_POINT']}, "
            f"BREAKUP_MODE {params['BREAKUP_MODE']}, PROC_ID {params['PROC_ID']}, {nev} events")


def row_blocks(nm, nblocks, block):
    """`nblocks` blocks of `block` consecutive m-rows spread evenly over the
    mass range (low, middle and top masses; the quadrature cost grows with
    the mass)."""
    if nblocks * block >= nm:
        return [(0, nm)]
    starts = np.linspace(0, nm - block, nblocks).round().astype(int)
    return [(int(a), int(a) + block) for a in starts]


def cpu_lumi_sample(o, blocks):
    """Luminosity rows of the blocks on every host thread; (seconds, cells)."""
    ny = o.grid()["ny"]
    t0 = time.perf_counter()
    for a, b in blocks:
        o.lumi_table(a, b)
    return time.perf_counter() - t0, sum(b - a for a, b in blocks) * ny


def cpu_phases(params, threads, blocks, n_events, lumi=None):
    """The CPU restatement's phases, each timed on its own: init (form factor,
    G_AA and breakup splines: src/UpcCrossSection.cpp:364-461), the luminosity
    on a row sample (:221-271, 463-592, OpenMP over m-rows), the fold and the
    samplers (:337-362, 594-698; UpcSampler.h:37-142), and event generation
    single-threaded as in the reference (src/UpcGenerator.cpp:715-926).
    `lumi` (the full table) feeds the fold; without it the sampled rows are
    tiled over the grid (the fold's cost does not depend on the values)."""
    from oracle.oracle import Oracle
    o = Oracle(params, threads=threads)
    t0 = time.perf_counter()
    o.init_tables()
    t_init = time.perf_counter() - t0
    g = o.grid()
    t_lumi, cells = cpu_lumi_sample(o, blocks)
    if lumi is None:
        rows = np.concatenate([o.lumi_table(a, b) for a, b in blocks[:1]])
        lumi = np.resize(rows, (g["nm"], g["ny"]))
    o1 = Oracle(params, threads=1)
    o1.init_tables()
    t0 = time.perf_counter()
    cs, tot, ratio = o1.nuc_cs_ym(lumi)
    zm = o1.cs_zm_table()
    t1 = time.perf_counter()
    o1.generate(cs, zm, 1, 1)  # builds the samplers (and draws one event)
    t_samp = time.perf_counter() - t1
    t_fold = time.perf_counter() - t0
    t0 = time.perf_counter()
    _, rej, _ = o1.generate(cs, zm, n_events, 1)
    t_ev = time.perf_counter() - t0 - t_samp
    return {
        "init_s": t_init,
        "lumi_cells_per_s": cells / t_lumi, "lumi_sample_cells": cells, "lumi_sample_s": t_lumi,
        "lumi_full_table_s_est": t_lumi * g["nm"] * g["ny"] / cells,
        "fold_and_samplers_s": t_fold,
        "events_per_s_1_thread": n_events / max(t_ev, 1e-9),
        "events_sample": n_events, "events_rejected": rej,
        "threads_lumi": threads, "threads_fold_events": 1,
        "sample": f"luminosity rows {blocks} (all {g['ny']} y-bins), FP64 on {threads} threads; "
                  f"fold + samplers on the full {g['nm']}x{g['ny']} grid; {n_events} events "
                  f"single-threaded",
    }


def run_reference(args):
    """CPU restatement of the reference on all host threads, bounded sample:
    each step computes 4 blocks of m-rows (as many rows per block as host
    threads) spread over the mass range."""
    from oracle.oracle import Oracle
    params = WORKLOADS[args.workload]
    threads = os.cpu_count() or 1
    o = Oracle(params, threads=threads)
    t0 = time.perf_counter()
    o.init_tables()
    t_init = time.perf_counter() - t0
    g = o.grid()
    # blocks as wide as the thread count (the OpenMP slicing is over m-rows)
    width = max(4, threads)
    if args.ref_rows:
        blocks = row_blocks(g["nm"], max(1, args.ref_rows // width), min(width, args.ref_rows))
    else:
        blocks = row_blocks(g["nm"], 4, width) if args.workload == "c2" else [(0, g["nm"])]
    for _ in range(min(args.warmup, 1)):
        o.lumi_table(0, 1)
    times = []
    for _ in range(args.steps):
        dt, cells = cpu_lumi_sample(o, blocks)
        times.append(dt)
    v = cells / float(np.mean(times))
    sample = (f"m-row blocks {blocks} of {g['nm']} x {g['ny']} y-bins = {cells} cells per step "
              f"(spread over the mass range)")
    n_ev = args.ref_events if args.ref_events else (20000 if args.workload == "c2" else 100000)
    phases = cpu_phases(params, threads, blocks[:2], n_ev)
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "cells/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * float(np.mean(times)), "higher_is_better": True,
            "scaling": "strong", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": workload_name(args.workload, params, g["nm"], g["ny"],
                                                 args.events if args.events is not None
                                                 else EVENTS[args.workload]),
                       "sample": sample},
            "init_tables_s": t_init,
            "cpu_phases": phases,
            "cpu_baseline": {"value": v, "unit": "cells/s", "cores": threads, "kind": "port",
                             "sample": sample},
            "e2e": {"value": v, "unit": "cells/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def cpu_baseline_sample(workload, lumi=None):
    """The GPU arm's CPU leg: the restatement's phases on this host (about
    15 s), cells/s of the luminosity sample as the headline figure."""
    params = WORKLOADS[workload]
    threads = os.cpu_count() or 1
    from oracle.oracle import Oracle
    nm = Oracle(params, threads=1).grid()["nm"]
    blocks = row_blocks(nm, 8, max(4, threads)) if workload == "c2" else [(0, nm)]
    ph = cpu_phases(params, threads, blocks, 20000 if workload == "c2" else 100000, lumi)
    return {"value": ph["lumi_cells_per_s"], "unit": "cells/s", "cores": threads, "kind": "port",
            "sample": ph["sample"], "phases": ph}


# DRAM bytes per launch (read + write) per computed row, from one ncu capture
# of each kernel on the c2 table (63,063 rows, one launch each): the
# contraction reads the dense operands and G once; k_fast_weights writes them
CONTRACT_DRAM_BYTES_PER_ROW = (487.054848e6 + 4.045312e6) / 63063
WEIGHTS_DRAM_BYTES_PER_ROW = (10.726400e6 + 456.792576e6) / 63063


def c2_parity(fast, tot_fast, plain=None):
    """The full 1001 x 121 table against the committed oracle fixture
    (tests/golden/c2_lumi.npz): the fast form against the converged flux
    quadrature and against the reference's own quadrature (QAGS at 1e-4), the
    plain path against the reference's quadrature; every cell."""
    path = os.path.join(ROOT, "tests", "golden", "c2_lumi.npz")
    if not os.path.exists(path):
        return None
    d = np.load(path)
    conv, ref = d["conv"], d["ref"]
    mx = conv.max()

    def stats(a, b):
        rel = np.abs(a / b - 1)
        out = {}
        for name, thr in (("above_1e-4_of_max", 1e-4), ("above_1e-5_of_max", 1e-5), ("all", 0.0)):
            m = conv >= thr * mx
            out[name] = {"cells": int(m.sum()), "max_rel": float(rel[m].max()),
                         "median_rel": float(np.median(rel[m])),
                         "cells_rel_above_1e-4": int((rel[m] > 1e-4).sum())}
        return out

    res = {"fixture": "tests/golden/c2_lumi.npz (oracle: ref = QAGS 1e-4 as the reference, "
                      "conv = converged flux integral)",
           "fast_vs_converged": stats(fast, conv),
           "fast_vs_reference_quadrature": stats(fast, ref),
           "reference_quadrature_vs_converged": stats(ref, conv),
           "fast_sigma_tot_vs_converged": abs(tot_fast / float(d["sigma_tot_conv"]) - 1),
           "fast_sigma_tot_vs_reference_quadrature": abs(tot_fast / float(d["sigma_tot_ref"]) - 1)}
    if plain is not None:
        res["plain_vs_reference_quadrature_max_rel"] = float(np.max(np.abs(plain / ref - 1)))
    return res


def event_file_rates(gen, n_cols=10_000_000, n_hepmc=2_000_000):
    """generateEvents with file output (src/UpcGenerator.cpp:589-628, 834-926):
    the particle-tree columns (n_cols events) and HepMC3 text (n_hepmc events)
    written to a temporary directory, wall clock through the API; each file
    is removed afterwards."""
    import shutil
    import tempfile
    out = {}
    d = tempfile.mkdtemp(prefix="upcg_bench_")
    try:
        for fmt, n, name in (("columns", n_cols, "events.cols"), ("hepmc", n_hepmc, "events.hepmc")):
            path = os.path.join(d, name)
            gen.writeEvents(path, 1000, fmt)  # the writer's buffers and threads
            t0 = time.perf_counter()
            gen.writeEvents(path, n, fmt)
            dt = time.perf_counter() - t0
            size = os.path.getsize(path)
            os.remove(path)
            out[fmt] = {"events": n, "events_per_s": n / dt, "file_gb_per_s": size / dt / 1e9,
                        "file_bytes": size}
    finally:
        shutil.rmtree(d, ignore_errors=True)
    out["host_threads"] = os.cpu_count()
    out["note"] = ("device generation of batch k+1 overlaps the host's formatting and writing of "
                   "batch k; HepMC3 text is formatted on every host core")
    return out


def scan_c5(ug, torch, steps, warmup, nev):
    """C5: the 64 ALP configurations built by one captured scan (upcg_scan_*),
    replayed; then nev events over them into one device buffer.  A step is one
    replay (every configuration's tables, one persistent contraction, the
    samplers)."""
    import ctypes as C
    cfgs = c5_configs()
    gens = [ug.UpcGenerator(c) for c in cfgs]
    scan = ug.Scan(gens)
    t0 = time.perf_counter()
    setup_first = scan.run()
    setup_wall = time.perf_counter() - t0
    for _ in range(warmup):
        scan.run()
    torch.cuda.synchronize()
    ms = [scan.run() for _ in range(steps)]
    cells = sum(g.grid()["nm"] * g.grid()["ny"] for g in gens)
    ms_step = float(np.mean(ms))
    per = nev // len(gens)
    buf = torch.empty(max(per, 1) * 48, dtype=torch.uint8, device="cuda")
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for g in gens:
        r = C.c_int64()
        ug._check(g._L.upcg_generate_events_device(g._h, per, C.c_void_p(buf.data_ptr()), None,
                                                   C.byref(r)))
    torch.cuda.synchronize()
    t_ev = time.perf_counter() - t0
    info = scan.info()
    return {"configurations": len(gens), "cells": cells, "ms_per_replay": ms_step,
            "cells_per_s": cells / (ms_step * 1e-3), "replays": steps,
            "rows": info["rows"], "items": info["items"], "shape": info["shape"],
            "setup_and_first_run_s": setup_wall, "first_run_ms": setup_first,
            "events": per * len(gens), "events_per_s": per * len(gens) / t_ev,
            "events_wall_s": t_ev,
            "note": "64 ALP configurations (Pb, Au, Xe, O x sqrt(s) 200/5020/5360/5440 GeV x "
                    "breakup modes 1-4; m-bins 201/501/1001, 121 y-bins), one captured graph "
                    "per replay; events without cuts, device buffer"}


def run_scan(args, ug, torch):
    """--workload c5: the scan as the line's own workload."""
    nev = args.events if args.events is not None else EVENTS["c5"]
    r = scan_c5(ug, torch, args.steps, args.warmup, nev)
    print(json.dumps({
        "metric": METRIC, "value": r["cells_per_s"], "unit": "cells/s", "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": r["ms_per_replay"],
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64+bf16x3",
        "data": "synthetic (the workload is a parameter set)",
        "config": {"workload": f"c5: {r['configurations']} ALP configurations, {r['cells']} (m,y) "
                               f"cells, one captured scan per step; {r['events']} events",
                   "rows": r["rows"], "items": r["items"], "shape": r["shape"],
                   "setup_and_first_run_s": r["setup_and_first_run_s"]},
        "events_per_s": r["events_per_s"], "events_wall_s": r["events_wall_s"],
    }))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="c2", choices=sorted(WORKLOADS) + ["c5"])
    ap.add_argument("--events", type=int, default=None)
    ap.add_argument("--ref-rows", type=int, default=None)
    ap.add_argument("--ref-events", type=int, default=None,
                    help="events of the reference arm's single-threaded event phase")
    ap.add_argument("--plain-steps", type=int, default=None)
    ap.add_argument("--e2e-steps", type=int, default=20)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-scan", action="store_true", help="skip the 64-configuration scan")
    ap.add_argument("--no-files", action="store_true", help="skip the event-file output timing")
    ap.add_argument("--lumi-method", default="fast",
                    help="the fast form's operand path for the timed build: fast, gather or fused")
    args = ap.parse_args()

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if args.impl == "reference":
        if rank == 0:
            run_reference(args)
        return

    import torch

    import upcgen_gb300 as ug
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if args.workload == "c5":
        if rank == 0:
            run_scan(args, ug, torch)
        return
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    params = dict(WORKLOADS[args.workload])
    # N > 1: one table split over the ranks by m-rows (the reference's OpenMP
    # m-slices, src/UpcCrossSection.cpp:537-538), all-gathered over NCCL on the
    # device; every rank builds the replicated samplers and draws its share of
    # the events from its own Philox counter range (upcgen_gb300/shard.py)
    nev_total = args.events if args.events is not None else EVENTS[args.workload]
    nev = nev_total // world + (1 if rank < nev_total % world else 0)
    stream = torch.cuda.Stream()
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    evbuf = torch.empty(max(nev, 1) * 48, dtype=torch.uint8, device="cuda")

    def make(method):
        g = ug.UpcGenerator(params)
        g.setStream(stream.cuda_stream)
        g.setLumiMethod(method)
        return g

    def flush_l2():
        with torch.cuda.stream(stream):
            flush.add_(1.0)

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    def step(gen, with_events):
        s0, s1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        flush_l2()
        if world > 1:
            # the sharded build synchronises with the host (the all-gather runs
            # on torch's stream): timed by the host clock between barriers
            from upcgen_gb300 import shard
            barrier()
            t0 = time.perf_counter()
            shard.sharded_init(gen, rank, world)
            torch.cuda.synchronize()
            tab_ms = 1e3 * (time.perf_counter() - t0)
        else:
            s0.record(stream)
            gen.init()
            s1.record(stream)
        ev_ms, rej = None, None
        if with_events and nev:
            flush_l2()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            r = ug.C.c_int64()
            ug._check(gen._L.upcg_generate_events_device(gen._h, nev, ug.C.c_void_p(evbuf.data_ptr()),
                                                         None, ug.C.byref(r)))
            e1.record(stream)
            stream.synchronize()
            ev_ms, rej = e0.elapsed_time(e1), r.value
        stream.synchronize()
        if world == 1:
            tab_ms = s0.elapsed_time(s1)
        return tab_ms, ev_ms, rej, gen.timings()

    fast = make(args.lumi_method)
    g0 = fast.grid()
    cells = g0["nm"] * g0["ny"]
    # the cold first init of a process (one configuration per process, as the
    # reference's main runs): allocations, static uploads, the contraction
    # autotuner, every table; host wall clock, init returns synchronised
    t0 = time.perf_counter()
    fast.init()
    cold_init_ms = 1e3 * (time.perf_counter() - t0)
    for _ in range(args.warmup):
        step(fast, True)
    barrier()
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)  # the sampler's first rows
    n_launch0 = ug.kernel_launches()
    runs = [step(fast, True) for _ in range(args.steps)]
    barrier()
    n_launch = ug.kernel_launches() - n_launch0
    clk = clocks.stop()
    ms_tab = float(np.mean([r[0] for r in runs]))
    ms_ev = float(np.mean([r[1] for r in runs])) if nev else None
    ms_contract = float(np.mean([r[3]["contract_ms"] for r in runs]))
    ms_project = float(np.mean([r[3]["project_ms"] for r in runs]))
    if dist is not None:
        t = torch.tensor([ms_tab, ms_ev or 0.0, ms_contract], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms_tab, ms_ev, ms_contract = float(t[0]), float(t[1]) or None, float(t[2])
    # one table per step whatever the rank count: its cells over the slowest
    # rank's time (strong scaling: the same table at every N)
    value = cells / (ms_tab * 1e-3)

    # the plain FP64 path on the same workload (the reference's quadrature)
    pk = args.plain_steps if args.plain_steps is not None else (2 if args.workload == "c2" else args.steps)
    fvp = None
    pruns = []
    lf = fast.lumiTable()
    _, tot_f = fast.nucCSYM()
    if pk > 0:
        plain = make("plain")
        step(plain, False)
        pruns = [step(plain, False) for _ in range(pk)]
        ms_plain = float(np.mean([r[0] for r in pruns]))
        lp = plain.lumiTable()
        _, tot_p = plain.nucCSYM()
        big = np.abs(lp) >= 1e-5 * np.abs(lp).max()
        rel = np.abs(lf - lp)[big] / np.abs(lp[big])
        fvp = {"max_rel_err_cells_above_1e-5_of_max": float(rel.max()),
               "median_rel_err": float(np.median(rel)),
               "sigma_tot_rel_err": abs(tot_f / tot_p - 1),
               "note": "vs the plain path, i.e. the reference's own QAGS at 1e-4; see parity",
               "plain_ms_per_step": ms_plain,
               "plain_cells_per_s": cells / (ms_plain * 1e-3),
               "speedup": ms_plain / ms_tab}
        del plain
    parity = c2_parity(lf, tot_f, lp if pk > 0 else None) if args.workload == "c2" else None

    # end to end through the public API, host buffers: init, then the
    # luminosity table, sigma(y, m) and its total copied to the host, into
    # page-locked arrays the caller allocated once
    gr = fast.grid()
    lumi_h = ug.pinned_array((gr["nm"], gr["ny"]), np.float64)
    cs_h = ug.pinned_array((gr["ny"], gr["nm"]), np.float64)
    torch.cuda.synchronize()
    h0, d0 = ug.copy_bytes()
    t0 = time.perf_counter()
    for _ in range(args.e2e_steps):
        fast.init()
        lumi = fast.lumiTable(out=lumi_h)
        cs, tot = fast.nucCSYM(out=cs_h)
    t1 = time.perf_counter()
    h1, d1 = ug.copy_bytes()
    ev_h = None
    if nev:
        # events through the host API into a page-locked host array (allocated
        # once, as a caller reusing its buffer would); one untimed call sizes
        # the library's device buffer, then the mean of 3 calls
        evout = ug.pinned_array(nev, ug.EVENT_DTYPE)
        fast.generateEvents(nev, out=evout)
        ev_h0 = ug.copy_bytes()
        te0 = time.perf_counter()
        for _ in range(3):
            fast.generateEvents(nev, out=evout)
        te1 = time.perf_counter()
        ev_h1 = ug.copy_bytes()
        ev_h = {"events_per_s": 3 * nev / (te1 - te0), "d2h_bytes_per_step": (ev_h1[1] - ev_h0[1]) // 3,
                "host_buffer": "page-locked (upcg_host_alloc)"}

    pk_vals, pk_kind = peaks()
    P = FAST_GRID_P
    # the contraction's rows: one cell of each mirror-rapidity pair (the other
    # is a copy); one launch covers up to 2^18 rows
    rows, macs_row = fast.contractWork()
    nlaunch_contract = max(1, -(-rows // 262144))
    # A1 (rows x P) times G - c over the tiles where it can be nonzero, per
    # table (the constant's share, c S0 S1, is a per-cell FP64 product)
    alg_flops = 2.0 * rows * macs_row
    achieved = alg_flops / (ms_contract * 1e-3) / 1e12
    peak = pk_vals.get("bf16_tflops", 1900.0)
    traffic = CONTRACT_DRAM_BYTES_PER_ROW * rows / nlaunch_contract
    ph = runs[-1][3]
    line = {
        "metric": METRIC, "value": value, "unit": "cells/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_tab,
        "higher_is_better": True, "scaling": "strong", "vs_baseline": None, "dtype": "f64+bf16x3",
        "data": "synthetic (the workload is a parameter set)",
        "config": {"workload": workload_name(args.workload, params, g0["nm"], g0["ny"], nev),
                   "lumi_method": f"{args.lumi_method} (tcgen05 3xBF16 contraction)",
                   "l2": "flushed (256 MB write) before each timed phase"},
        "fast_vs_plain": fvp,
        "parity": parity,
        "events_per_s": nev_total / (ms_ev * 1e-3) if nev else None,
        "ms_events": ms_ev, "rejected_per_step": runs[-1][2],
        "sigma_tot_mb": tot,
        "phases_ms": ph, "plain_phases_ms": pruns[-1][3] if pruns else None,
        "e2e": {"value": cells * args.e2e_steps / (t1 - t0), "unit": "cells/s",
                "h2d_bytes_per_step": (h1 - h0) // args.e2e_steps,
                "d2h_bytes_per_step": (d1 - d0) // args.e2e_steps,
                "host_buffers": "page-locked (upcg_host_alloc), allocated once",
                "events": ev_h},
        "roofline": {"kernel": "k_contract_pers (persistent tcgen05.mma kind::f16, 3xBF16)",
                     "bound": "tensor",
                     "achieved": achieved, "peak": peak,
                     "unit": "TFLOP/s", "frac": achieved / peak, "traffic": traffic,
                     "issued_frac": 3.0 * achieved / peak,
                     "note": f"algorithmic 2*rows*MACs = {alg_flops:.3e} FLOP per table over "
                             f"{nlaunch_contract} launch(es), rows = {rows} computed cells (one of "
                             f"each mirror-rapidity pair), {macs_row} multiply-adds per row (the "
                             f"nonzero tiles of G - c: {macs_row / P / P:.3f} of the dense "
                             f"P x P; the hi/lo split issues them 3x: issued_frac); "
                             f"peak = {pk_kind} bf16 burst; traffic = DRAM bytes per launch "
                             f"from an ncu capture, scaled by rows"},
        "roofline_weights": {
            "kernel": "k_fast_weights (the projection's node weights and dense rows)",
            "bound": "hbm",
            "achieved": 8.0 * P * rows / (ms_project * 1e-3) / 1e9 if ms_project else None,
            "peak": pk_vals.get("hbm_gbs", 6800.0), "unit": "GB/s",
            "traffic": WEIGHTS_DRAM_BYTES_PER_ROW * rows / nlaunch_contract,
            "note": "algorithmic bytes = the 8 KB per computed row of dense contraction operands "
                    "written (A1 bf16 hi + lo, A2 FP32) over the kernel's time (events around its "
                    "launch, after the flux tables are joined); peak = "
                    f"{pk_kind} copy rate; traffic = its DRAM bytes per launch from an ncu capture"},
        "cold_first_init_ms": cold_init_ms,
        "gpu_launches": n_launch,
        "clocks": clk,
    }
    if line["roofline_weights"]["achieved"]:
        line["roofline_weights"]["frac"] = (line["roofline_weights"]["achieved"] /
                                            line["roofline_weights"]["peak"])
    if rank == 0 and args.workload == "c2" and not args.no_files:
        line["event_files"] = event_file_rates(fast)
    if rank == 0 and args.workload == "c2" and not args.no_scan:
        # the batched scan (C5) of the same run, beside the headline table
        line["c5_scan"] = scan_c5(ug, torch, steps=5, warmup=2, nev=EVENTS["c5"])
    if rank == 0 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline_sample(args.workload, lf)
    if rank == 0:
        print(json.dumps(line))
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
