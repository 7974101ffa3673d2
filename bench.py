"""Benchmark: two-photon luminosity / cross-section tables and event sampling.

Workload (default): the full-grid Pb-Pb configuration -- Woods-Saxon
form-factor flux (FLUX_POINT 0), gamma-gamma -> tau tau (PROC_ID 15), XNXN
breakup (BREAKUP_MODE 2), m in [3.56, 50] GeV x 1001 bins, y in [-6, 6] x 121
bins, z x 100 bins, pT > 1 GeV and |eta| < 2.4, 1e7 accepted events.
Synthetic in the only sense that applies: the inputs are these parameters.

One step = the complete table build of UpcGenerator::init on the GPU (form
factor, G_AA and breakup tables, the 121,121-cell luminosity, the nuclear
cross section and the sampling CDFs), timed with CUDA events on the library's
stream; the 1e7-event sampling is timed as a second phase of the same step.
`value` = luminosity cells / second of the table build, `events_per_s` =
accepted events / second.  The L2 (129 MB) is flushed before every timed phase.

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
EVENTS = {"c2": 10_000_000, "c1": 100_000}
METRIC = "gamma-gamma lumi (m,y) cells/s"


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            return json.load(f), "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.rows = []
        self.proc = None
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
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
        sm = [float(r[0]) for r in self.rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4) if "Active" in r[3 + i]})
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(self.rows)}


def run_reference(args):
    """CPU restatement of the reference on all host threads, bounded sample."""
    from oracle.oracle import Oracle
    params = WORKLOADS[args.workload]
    threads = os.cpu_count() or 1
    o = Oracle(params, threads=threads)
    o.init_tables()
    g = o.grid()
    # sample: the first R m-rows (all ny rapidities) -- ~10-30 s of CPU work
    rows = args.ref_rows or (16 if args.workload == "c2" else g["nm"])
    times = []
    for _ in range(max(args.warmup, 0) and 1):
        o.lumi_table(0, 1)
    for _ in range(args.steps):
        t0 = time.perf_counter()
        o.lumi_table(0, rows)
        times.append(time.perf_counter() - t0)
    cells = rows * g["ny"]
    v = cells / float(np.mean(times))
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "cells/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * float(np.mean(times)), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": args.workload, "params": params,
                       "sample": f"first {rows} m-rows x {g['ny']} y-bins = {cells} cells"},
            "cpu_baseline": {"value": v, "unit": "cells/s", "cores": threads, "kind": "port",
                             "sample": f"{cells} cells (first {rows} of {g['nm']} m-rows)"},
            "e2e": {"value": v, "unit": "cells/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def cpu_baseline_sample(workload, seconds=15.0):
    from oracle.oracle import Oracle
    params = WORKLOADS[workload]
    threads = os.cpu_count() or 1
    o = Oracle(params, threads=threads)
    o.init_tables()
    g = o.grid()
    rows, dt = 2, 0.0
    while True:
        t0 = time.perf_counter()
        o.lumi_table(0, rows)
        dt = time.perf_counter() - t0
        if dt > seconds / 4 or rows >= g["nm"]:
            break
        rows = min(g["nm"], rows * 4)
    cells = rows * g["ny"]
    return {"value": cells / dt, "unit": "cells/s", "cores": threads, "kind": "port",
            "sample": f"{cells} cells (first {rows} of {g['nm']} m-rows), one pass"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="c2", choices=sorted(WORKLOADS))
    ap.add_argument("--events", type=int, default=None)
    ap.add_argument("--ref-rows", type=int, default=None)
    ap.add_argument("--no-cpu-baseline", action="store_true")
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
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    params = dict(WORKLOADS[args.workload])
    params["SEED"] = 1 + rank  # independent replicas: weak scaling over ranks
    nev = args.events if args.events is not None else EVENTS[args.workload]
    stream = torch.cuda.Stream()
    gen = ug.UpcGenerator(params)
    gen.setStream(stream.cuda_stream)
    g0 = gen.grid()
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    evbuf = torch.empty(max(nev, 1) * 48, dtype=torch.uint8, device="cuda")

    def flush_l2():
        with torch.cuda.stream(stream):
            flush.add_(1.0)

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    def step():
        s0, s1, s2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
        flush_l2()
        s0.record(stream)
        gen.init()
        s1.record(stream)
        flush_l2()
        e0 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        rej = ug.C.c_int64()
        ug._check(gen._L.upcg_generate_events_device(gen._h, nev, ug.C.c_void_p(evbuf.data_ptr()),
                                                     None, ug.C.byref(rej)))
        s2.record(stream)
        stream.synchronize()
        return s0.elapsed_time(s1), e0.elapsed_time(s2), rej.value

    for _ in range(args.warmup):
        step()
    barrier()
    clocks = ClockSampler(local)
    clocks.start()
    t_tab, t_ev, rejs, phases = [], [], [], []
    for _ in range(args.steps):
        a, b, r = step()
        t_tab.append(a)
        t_ev.append(b)
        rejs.append(r)
        phases.append(gen.timings())
    barrier()
    clk = clocks.stop()
    ms_tab = float(np.mean(t_tab))
    ms_ev = float(np.mean(t_ev))
    if dist is not None:
        t = torch.tensor([ms_tab, ms_ev], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms_tab, ms_ev = float(t[0]), float(t[1])
    cells = g0["nm"] * g0["ny"]
    value = world * cells / (ms_tab * 1e-3)

    # end to end through the public API with host buffers (D2H of the tables
    # and of the events inside the timed region)
    host_ev = np.zeros(nev, dtype=ug.EVENT_DTYPE)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    gen.init()
    lumi = gen.lumiTable()
    cs, tot = gen.nucCSYM()
    t1 = time.perf_counter()
    _, rej_h = gen.generateEvents(nev) if nev else (None, 0)
    t2 = time.perf_counter()
    e2e_cells = cells / (t1 - t0)
    e2e_events = nev / (t2 - t1) if nev else None

    pk, pk_kind = peaks()
    ph = phases[-1]
    line = {
        "metric": METRIC, "value": value, "unit": "cells/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_tab,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (parameter set; no dataset)",
        "config": {"workload": f"{args.workload}: Pb-Pb {g0['nm']}x{g0['ny']} (m,y) cells, "
                               f"FLUX_POINT {params['FLUX_POINT']}, BREAKUP_MODE {params['BREAKUP_MODE']}, "
                               f"PROC_ID {params['PROC_ID']}, {nev} events",
                   "lumi_method": "plain FP64", "l2": "flushed (256 MB write) before each timed phase"},
        "events_per_s": world * nev / (ms_ev * 1e-3) if nev else None,
        "ms_events": ms_ev,
        "rejected_per_step": rejs[-1],
        "sigma_tot_mb": tot,
        "phases_ms": ph,
        "e2e": {"value": e2e_cells, "unit": "cells/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": int(lumi.nbytes + cs.nbytes),
                "events_per_s": e2e_events, "events_d2h_bytes": nev * 48},
        "gpu_launches": None,
        "clocks": clk,
        "peaks": {"source": pk_kind},
    }
    if rank == 0 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline_sample(args.workload)
    if rank == 0:
        print(json.dumps(line))
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
