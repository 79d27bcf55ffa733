"""Benchmark of the energy-representation hot path on GB300.

Metric: solute-solvent molecule energies per second (one unit = one placement x one
solvent molecule energy, computed and binned).  Workload (default): reference-solvent
insertion of a 12-site solute into 33,000 rigid waters in a 99.5 A box, PME 96^3,
order 4, cutoff 12 A, 50,000 insertions per frame, ecorr accumulated.  One step = one
frame: the frame preparation plus all of its insertions.

Lines printed (rank 0, one JSON line):
  value         device-resident inputs (frame coordinates and placements already in
                HBM), CUDA events on the library's stream, L2 flushed between steps;
  e2e           the same steps through the host C ABI (ermod_frame / ermod_placements
                with host arrays, the accumulators read back every step), wall clock;
  roofline      the dominant kernel of the step against the measured HBM copy peak;
  plain_fp64_gpu  the plain FP64 GPU path (one placement at a time) on a sample;
  cpu_baseline  the FP64 CPU oracle on a bounded sample, all host cores.
`--impl reference` times the reference algorithm's CPU restatement (the oracle: the
Fortran reference cannot be built here) on the same workload and metric.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import tempfile
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

SMI_QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="refs_large")
    ap.add_argument("--insertions", type=int, default=None, help="insertions per frame (default: workload's)")
    ap.add_argument("--batch", type=int, default=256, help="placements per PME launch")
    ap.add_argument("--finish-group", type=int, default=0,
                    help="placements per molecule-energy block, 4 or 8 (0: automatic)")
    ap.add_argument("--grid", type=int, default=None, help="PME grid points per axis (default: workload's)")
    ap.add_argument("--cpu-sample", type=int, default=96, help="placements timed on the CPU oracle")
    ap.add_argument("--plain-sample", type=int, default=48, help="placements timed on the plain FP64 GPU path")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-graph", action="store_true",
                    help="solution mode: time ordinary calls instead of one CUDA graph launch per frame")
    return ap.parse_args()


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def frames_of_rank(rank, nsteps):
    """The frames rank `rank` processes (weak scaling: every rank its own nsteps frames,
    the reference's plmode = 2 frame sharding)."""
    return [rank * nsteps + i for i in range(nsteps)]


def merge_ranks(acc, w):
    """engstore's exchange over the ranks (engproc.F90:475-546): rank 0 receives the
    merged, normalised distributions (ermod_engstore_merge); other ranks None."""
    from ermod_gb300 import engstore
    return engstore.merge_distributed(acc, w.params["slttype"], w.params["wgtslf"], w.params["temp"])


class ClockSampler:
    """nvidia-smi samples (200 ms) of one GPU while the timed region runs, written as CSV to
    $ERMOD_CLOCK_LOG_DIR/clocks_<pid>.csv when that variable is set (else a temporary file)."""

    def __init__(self, device_index: int):
        self.dev = device_index
        self.proc = None
        d = os.environ.get("ERMOD_CLOCK_LOG_DIR") or tempfile.gettempdir()
        self.path = os.path.join(d, f"clocks_{os.getpid()}.csv")

    def __enter__(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.dev}", f"--query-gpu={SMI_QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
        try:
            self.f.close()
        except Exception:
            pass

    def summary(self):
        try:
            rows = [r.split(",") for r in open(self.path).read().strip().splitlines()]
        except Exception:
            return None
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            r = [x.strip() for x in r]
            if len(r) < 9:
                continue
            try:
                sm.append(float(r[1]))
                mx = float(r[2])
            except ValueError:
                continue
            for n, v in zip(names, r[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return None
        busy = [s for s in sm if mx and s > 0.5 * mx] or sm
        return {"sm_mhz": statistics.median(busy), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def load_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def make_workload(args):
    from ermod_gb300 import synth
    if args.workload.startswith("uneven_"):  # one system of the uneven set, alone
        w = synth.uneven()[int(args.workload.split("_")[1])]
    else:
        w = synth.WORKLOADS[args.workload]()
    if args.insertions:
        w.ins_per_frame = args.insertions
    if args.grid:
        w.params.update(ms1max=args.grid, ms2max=args.grid, ms3max=args.grid)
    return w


def workload_config(w, args, ws=1):
    """The `config` object of both arms: the same workload named the same way."""
    K = w.params["ms1max"]
    soln = w.mode == "soln"
    return {"workload": f"{w.name}: {w.nwater} waters, {w.box} A box, PME {K}^3 order {w.params['splodr']}, "
                        f"{len(w.solute['charge'])}-site solute, "
                        + ("solution mode" if soln else f"{w.ins_per_frame} insertions/frame")
                        + (", ecorr on" if w.params.get("corrcal") else ""),
            "batch": args.batch, "l2": "flushed between steps (256 MiB write)",
            "parallelism": f"frames sharded over {ws} GPU(s)" if ws > 1 else "1 GPU"}


def cpu_oracle_rate(w, topo, bins, nplace, frame_index=0, want_uvengy=False, placements=None):
    """The FP64 oracle on nplace placements of one frame (the given ones, else the first
    nplace of the frame's own draw), all host cores (solution mode: the frame's own
    solute, once).  Returns (rate, seconds, uvengy or None)."""
    from oracle import oracle as O
    O.build()
    orc = O.Oracle(w.params, topo, bins)
    pos, cell = w.frame(frame_index)
    orc.frame(pos, cell)
    if w.mode == "soln":
        nplace = 1
    if w.mode == "soln":
        pl = None
    elif placements is not None:
        pl = np.ascontiguousarray(placements[:nplace])
    else:
        pl = w.placements(frame_index, w.ins_per_frame)[:nplace]
    tag = np.full(nplace, topo["nummol"], np.int32)
    t0 = time.perf_counter()
    r = orc.placements(tag, pl, want_uvengy=want_uvengy, nthreads=0)
    dt = time.perf_counter() - t0
    orc.close()
    return nplace * w.nwater / dt, dt, (r["uvengy"] if want_uvengy else None)


# The mixed path's stated per-molecule error bound against the FP64 oracle (kcal/mol): the
# band around each bin edge within which a molecule may take the neighbouring bin; for a
# solute of summed absolute charge above 3 e it grows as sqrt(sum|q| / 3 e).
MIXED_BAND = 3e-5


def mixed_band(solute):
    return MIXED_BAND * max(1.0, float(np.sqrt(np.sum(np.abs(solute["charge"])) / 3.0)))


def accuracy_report(u_gpu, u_orc, edges, band=MIXED_BAND):
    """Per-molecule error of the GPU energies against the oracle's on the same placements,
    molecules near a bin edge (within 1e-6 and within the stated band) and molecules that
    the GPU bins elsewhere."""
    ug, uo = u_gpu[:, 1:], u_orc[:, 1:]
    err = np.abs(ug - uo)
    soft = np.abs(uo) < 20.0
    hard = np.abs(uo) >= 1e3
    near6 = near = flips = 0
    for a, b in zip(ug, uo):
        idx = np.searchsorted(edges, b)
        dlo = np.abs(b - edges[np.clip(idx - 1, 0, len(edges) - 1)])
        dhi = np.abs(b - edges[np.clip(idx, 0, len(edges) - 1)])
        d = np.minimum(dlo, dhi)
        near6 += int(np.count_nonzero(d <= 1e-6))
        near += int(np.count_nonzero(d <= band))
        flips += int(np.count_nonzero(np.searchsorted(edges, a, side="left") != np.searchsorted(edges, b, side="left")))
    return {"molecules": int(uo.size), "max_abs_err_below_1e3": float(err[~hard].max()) if (~hard).any() else 0.0,
            "max_abs_err_soft": float(err[soft].max()) if soft.any() else 0.0,
            "max_rel_err_above_1e3": float((err[hard] / np.abs(uo[hard])).max()) if hard.any() else 0.0,
            "max_abs_energy": float(np.abs(uo).max()),
            "self_energy_max_abs_err": float(np.abs(u_gpu[:, 0] - u_orc[:, 0]).max()),
            "band": band, "near_edge_1e-6": near6, "near_edge_band": near, "other_bin": flips}


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    # the topology and bins from the oracle's own restatement of setconf/enginit, so that
    # this arm loads nothing of the GPU library
    from oracle import oracle as O
    w = make_workload(args)
    topo = O.setparam_topology(w.species(), slttype=w.params["slttype"])
    bins = O.enginit_bins(topo["numslv"], w.hist)
    sample = 1 if w.mode == "soln" else max(1, args.cpu_sample // 4)  # solution mode: the frame's solute
    for i in range(args.warmup):
        cpu_oracle_rate(w, topo, bins, max(1, sample // 4), i)
    t_total, units = 0.0, 0
    for i in range(args.steps):
        rate, dt, _ = cpu_oracle_rate(w, topo, bins, sample, i)
        t_total += dt
        units += sample * w.nwater
    value = units / t_total
    cores = os.cpu_count()
    line = {
        "impl": "reference", "metric": "solute-solvent molecule energies/s", "value": value,
        "unit": "molecule-energies/s", "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1000.0 * t_total / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": workload_config(w, args, ws),
        "cpu_baseline": {"value": value, "unit": "molecule-energies/s", "cores": cores, "kind": "port",
                         "sample": f"{sample} insertions of one frame per step x {args.steps} steps, FP64 "
                                   f"oracle restating the Fortran reference (which cannot be built here), "
                                   f"OpenMP over insertions on all {cores} host cores"},
        "e2e": {"value": value, "unit": "molecule-energies/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def run_ours(args):
    import torch
    from ermod_gb300 import build, roofline, setconf
    from ermod_gb300.engproc import EnergyRepresentation

    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    build.build()
    w = make_workload(args)
    topo = setconf.setparam_topology(w.species(), slttype=w.params["slttype"])
    bins = setconf.enginit_bins(topo["numslv"], w.hist)
    nplace = w.ins_per_frame
    nsteps = args.warmup + args.steps
    # frames of this rank (weak scaling: every rank its own frames)
    fidx = frames_of_rank(rank, nsteps)
    frames = [w.frame(i) for i in fidx]
    soln = w.mode == "soln"  # solution mode: the solute is the frame's own molecule
    places = None if soln else [w.placements(i, nplace) for i in fidx]
    tag_h = np.full(nplace, topo["nummol"], np.int32)
    cell = frames[0][1]

    eng = EnergyRepresentation(w.params, topo, bins, precision="mixed", device=local, batch=args.batch,
                               finish_group=args.finish_group)
    stream = torch.cuda.Stream(device=dev)
    eng.set_stream(stream.cuda_stream)
    pos_d = [torch.from_numpy(f[0]).to(dev) for f in frames]
    pl_d = None if soln else [torch.from_numpy(np.ascontiguousarray(p)).to(dev) for p in places]
    tag_d = torch.from_numpy(tag_h).to(dev)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    torch.cuda.synchronize()

    def step(i):
        eng.frame_device(pos_d[i].data_ptr(), frames[i][1])
        eng.placements_device(nplace, tag_d.data_ptr(), 0 if soln else pl_d[i].data_ptr())

    for i in range(args.warmup):
        with torch.cuda.stream(stream):
            flush.fill_(float(i))
        step(i)
        eng.sync()
    # solution mode: a frame is one placement, so a step is a few dozen short kernels and
    # their launches would dominate; the step is captured once into a CUDA graph
    # (ermod_graph_create, the public API) and each frame is its coordinate copy into the
    # graph's input buffer plus one graph launch.  The phase times and launch count come
    # from ordinary steps run untimed before the capture.
    graph = None
    if soln and not args.no_graph:
        from ermod_gb300.multisystem import SystemGraph
        eng.timing(True)
        eng.timing_reset()
        for k in range(args.steps):
            step(args.warmup + k)
        eng.sync()
        phases, launches = eng.timing_get()
        eng.timing(False)
        graph = SystemGraph([eng], [frames[0]], [None], [topo["nummol"]])
        gpos = graph.frame_buffer(0)

        def step(i):  # noqa: F811 -- the graph form of the step
            with torch.cuda.stream(stream):
                gpos.copy_(pos_d[i], non_blocking=True)
            graph.launch_ordered(stream.cuda_stream)

        for i in range(args.warmup):
            with torch.cuda.stream(stream):
                flush.fill_(float(i))
            step(i)
        graph.sync()
    else:
        eng.timing(True)
        eng.timing_reset()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    if ws > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        for k in range(args.steps):
            i = args.warmup + k
            with torch.cuda.stream(stream):
                flush.fill_(float(i))
                ev[k][0].record(stream)
            step(i)
            ev[k][1].record(stream)
        eng.sync()
        torch.cuda.synchronize()
    if ws > 1:
        torch.distributed.barrier()
    ms = sum(a.elapsed_time(b) for a, b in ev)
    if graph is None:
        phases, launches = eng.timing_get()
        eng.timing(False)
    else:
        graph.sync()
    t_local = torch.tensor([ms], device=dev, dtype=torch.float64)
    if ws > 1:
        torch.distributed.all_reduce(t_local, op=torch.distributed.ReduceOp.MAX)
    ms_max = float(t_local.item())
    if ws > 1:  # the path's one exchange: engstore's merge of every rank's accumulators
        merge_ranks(eng.accum(), w)
    units = nplace * w.nwater * args.steps * ws
    value = units / (ms_max / 1000.0)

    # ---- roofline of the dominant kernel ----
    K = w.params["ms1max"]
    nsite_phys = 3 * w.nwater
    per_pl = roofline.bytes_per_placement(K, K, K, nsite_phys, G=min(8, args.batch))
    nbatch = args.steps * ((nplace + args.batch - 1) // args.batch)
    cand = {k: phases.get(k, 0.0) for k in ("spectrum", "fft_c2r", "gather")}
    dom = max(cand, key=cand.get)
    avg_launch_ms = cand[dom] / nbatch
    per_launch = nplace / ((nplace + args.batch - 1) // args.batch)  # placements per PME launch
    bytes_per_launch = per_pl[dom] * per_launch
    peak, peak_kind = load_peaks()
    achieved = bytes_per_launch / (avg_launch_ms / 1000.0) / 1e9
    traffic = pipes = None
    if args.workload == "refs_large":
        traffic = roofline.MEASURED_TRAFFIC_REFS_LARGE[dom] * per_launch
        # the issue / pipe use that bounds the kernel (the HBM fraction alone does not: it
        # waits on barriers and instruction issue), and the fraction it reaches launched alone
        pm = dict(roofline.MEASURED_PIPES_REFS_LARGE[dom])
        alone_gbs = per_pl[dom] * 256 / (pm["standalone_us"] * 1e-6) / 1e9
        pipes = dict(pm, frac_standalone=alone_gbs / peak, source=roofline.PIPES_SOURCE,
                     note="ncu --set full of one 256-placement launch; frac_standalone = algorithmic "
                          "bytes / that launch's duration / peak")
    roof = {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak, "peak_kind": peak_kind, "traffic": traffic,
            "traffic_note": "ncu DRAM read+write per launch (one capture, scaled to the launch's placements)",
            "bytes_per_launch": bytes_per_launch, "avg_launch_ms": avg_launch_ms, "pipes": pipes,
            "phase_ms_per_step": {k: v / args.steps for k, v in phases.items()}}
    clocks = clk.summary()

    # ---- end to end through the host C ABI ----
    e2e = None
    if not args.no_e2e:
        eng2 = EnergyRepresentation(w.params, topo, bins, precision="mixed", device=local, batch=args.batch,
                                   finish_group=args.finish_group)
        pinned_pl = [None] * nsteps if soln else [torch.from_numpy(np.ascontiguousarray(p)).pin_memory().numpy()
                                                  for p in places]
        pinned_pos = [torch.from_numpy(f[0]).pin_memory().numpy() for f in frames]
        for i in range(args.warmup):
            eng2.frame(pinned_pos[i], cell)
            eng2.placements(tag_h, pinned_pl[i])
            eng2.accum()
        t0 = time.perf_counter()
        for k in range(args.steps):
            i = args.warmup + k
            eng2.frame(pinned_pos[i], cell)
            eng2.placements(tag_h, pinned_pl[i])
            acc = eng2.accum()
        dt = time.perf_counter() - t0
        eng2.close()
        h2d = frames[0][0].nbytes + (0 if soln else places[0].nbytes) + tag_h.nbytes
        # the accumulators read back every step (ecorr only when it is on), from the arrays
        d2h = sum(v.nbytes for v in acc.values() if isinstance(v, np.ndarray)) + 5 * 8
        e2e = {"value": nplace * w.nwater * args.steps / dt * ws, "unit": "molecule-energies/s",
               "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h)}
        del acc

    # ---- plain FP64 GPU path (the comparator of the metric) ----
    plain = None
    if rank == 0 and args.plain_sample > 0:
        eng64 = EnergyRepresentation(w.params, topo, bins, precision="fp64", device=local)
        eng64.frame(frames[0][0], cell)
        n = min(args.plain_sample, nplace)
        eng64.placements(tag_h[:4], None if soln else places[0][:4])
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        eng64.placements(tag_h[:n], None if soln else places[0][:n])
        dt = time.perf_counter() - t0
        eng64.close()
        plain = {"value": n * w.nwater / dt, "unit": "molecule-energies/s", "sample": f"{n} placements, frame 0",
                 "dtype": "f64"}

    cpu = accuracy = None
    if rank == 0 and not args.no_cpu:
        ncpu = 1 if soln else args.cpu_sample
        rate, dt, u_orc = cpu_oracle_rate(w, topo, bins, ncpu, fidx[0], want_uvengy=True,
                                          placements=None if soln else places[0])
        cpu = {"value": rate, "unit": "molecule-energies/s", "cores": os.cpu_count(), "kind": "port",
               "sample": f"{ncpu} placements of frame 0 ({dt:.2f} s), FP64 oracle, OpenMP"}
        # the same placements on the mixed path, checked against the oracle's energies
        eng3 = EnergyRepresentation(w.params, topo, bins, precision="mixed", device=local, batch=args.batch,
                                   finish_group=args.finish_group)
        eng3.frame(frames[0][0], cell)
        u_gpu = eng3.placements(tag_h[:ncpu], None if soln else places[0][:ncpu], want_uvengy=True)["uvengy"]
        eng3.close()
        accuracy = accuracy_report(u_gpu, u_orc, bins["uvcrd"], mixed_band(w.solute))
        accuracy["sample"] = f"{ncpu} placements of frame 0 against the FP64 oracle"

    if rank == 0:
        line = {
            "metric": "solute-solvent molecule energies/s", "value": value, "unit": "molecule-energies/s",
            "n_gpus": ws, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_max / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64",
            "data": "synthetic",
            "config": workload_config(w, args, ws),
            "e2e": e2e, "roofline": roof, "cpu_baseline": cpu, "accuracy": accuracy, "plain_fp64_gpu": plain,
            "gpu_launches": int(launches), "clocks": clocks,
        }
        if graph is not None:
            line["launch"] = "one CUDA graph launch per frame (ermod_graph_launch), frame copied into its input"
        print(json.dumps(line))
    if graph is not None:
        graph.close()
    eng.close()
    if ws > 1:
        torch.distributed.destroy_process_group()


def _timed(fn, steps, warmup, stream):
    """CUDA-event time (ms) of `steps` calls of fn(i) after `warmup` calls, on stream."""
    import torch
    for i in range(warmup):
        fn(i)
    torch.cuda.synchronize()
    t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    t0.record(stream)
    for k in range(steps):
        fn(warmup + k)
    t1.record(stream)
    torch.cuda.synchronize()
    return t0.elapsed_time(t1)


def run_uneven(args):
    """16 water systems of uneven size (2k-60k waters), each with its own solute, grid and
    insertion count, one step of all of them replayed as one CUDA graph launch; the batch
    (placements per PME launch) and the finish group (placements per molecule-energy block)
    of every system picked by the autotuner."""
    import torch
    from ermod_gb300 import build, setconf, synth
    from ermod_gb300.engproc import EnergyRepresentation
    from ermod_gb300.multisystem import SystemGraph, autotune_tiles
    build.build()
    torch.cuda.set_device(0)
    systems = synth.uneven()
    engines, tops, frames, places, batches = [], [], [], [], []
    for w in systems:
        topo = setconf.setparam_topology(w.species(), slttype=2)
        bins = setconf.enginit_bins(topo["numslv"], w.hist)
        f0, f1 = w.frame(0), w.frame(1)
        p0, p1 = w.placements(0), w.placements(1)
        B, G, _ = autotune_tiles(w.params, topo, bins, f0, p0[:1024], topo["nummol"])
        eng = EnergyRepresentation(w.params, topo, bins, precision="mixed", batch=B, finish_group=G)
        eng.frame(*f0)
        eng.placements(np.full(len(p0), topo["nummol"], np.int32), p0)
        engines.append(eng)
        tops.append(topo)
        frames.append(f1)
        places.append(p1)
        batches.append((B, G))
    g = SystemGraph(engines, frames, places, [t["nummol"] for t in tops])
    stream = torch.cuda.Stream()

    def step(i):
        g.launch(stream.cuda_stream)

    with ClockSampler(0) as clk:
        ms = _timed(step, args.steps, args.warmup, stream)
    g.sync()
    units = sum(w.ins_per_frame * w.nwater for w in systems) * args.steps
    cpu = accuracy = None
    if not args.no_cpu:  # one system of the set (the median size) on the oracle, and the GPU on the same sample
        k = int(np.argsort([w.nwater for w in systems])[len(systems) // 2])
        w, topo = systems[k], tops[k]
        bins = setconf.enginit_bins(topo["numslv"], w.hist)
        n = max(8, args.cpu_sample // 4)
        rate, dt, u_orc = cpu_oracle_rate(w, topo, bins, n, 1, want_uvengy=True, placements=places[k])
        cpu = {"value": rate, "unit": "molecule-energies/s", "cores": os.cpu_count(), "kind": "port",
               "sample": f"system {k} ({w.nwater} waters, PME {w.params['ms1max']}^3): {n} placements ({dt:.2f} s), "
                         f"FP64 oracle, OpenMP"}
        eng = EnergyRepresentation(w.params, topo, bins, precision="mixed", batch=batches[k][0],
                                   finish_group=batches[k][1])
        eng.frame(*frames[k])
        u_gpu = eng.placements(np.full(n, topo["nummol"], np.int32), places[k][:n], want_uvengy=True)["uvengy"]
        eng.close()
        accuracy = accuracy_report(u_gpu, u_orc, bins["uvcrd"], mixed_band(w.solute))
        accuracy["sample"] = cpu["sample"]
    line = {"metric": "solute-solvent molecule energies/s", "value": units / (ms / 1e3),
            "unit": "molecule-energies/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32+f64", "data": "synthetic",
            "config": {"workload": "uneven: 16 systems, 2k-60k waters, own solutes (6-40 sites), grids and "
                                   "1k-20k insertions, one CUDA graph launch per step",
                       "systems": [{"waters": w.nwater, "K": w.params["ms1max"], "insertions": w.ins_per_frame,
                                    "solute_sites": len(w.solute["charge"]), "batch": b[0], "finish_group": b[1]}
                                   for w, b in zip(systems, batches)]},
            "clocks": clk.summary(), "cpu_baseline": cpu, "accuracy": accuracy}
    print(json.dumps(line))
    g.close()
    for e in engines:
        e.close()


def run_adjoint(args):
    """Solution mode of 8,000 waters with a 16-site solute (PME 64^3): frames per second of
    the energies plus the bin-resolved derivatives for all 48 solute parameters."""
    import torch
    from ermod_gb300 import build, setconf, synth
    from ermod_gb300.engproc import EnergyRepresentation
    build.build()
    torch.cuda.set_device(0)
    w = synth.soln_adjoint(frames=args.warmup + args.steps)
    topo = setconf.setparam_topology(w.species(), slttype=1)
    bins = setconf.enginit_bins(topo["numslv"], w.hist)
    dev = torch.device("cuda", 0)
    nsteps = args.warmup + args.steps
    pos_d = [torch.from_numpy(w.frame(i)[0]).to(dev) for i in range(nsteps)]
    cell = w.frame(0)[1]
    tag_d = torch.tensor([topo["nummol"]], dtype=torch.int32, device=dev)
    rates = {}
    for adj in (False, True):
        eng = EnergyRepresentation(w.params, topo, bins, precision="mixed")
        if adj:
            eng.adjoint_enable()
        stream = torch.cuda.Stream()
        eng.set_stream(stream.cuda_stream)

        def step(i):
            eng.frame_device(pos_d[i].data_ptr(), cell)
            eng.placements_device(1, tag_d.data_ptr())

        graph = None
        if not args.no_graph:  # one CUDA graph launch per frame, as in solution mode of run_ours
            from ermod_gb300.multisystem import SystemGraph
            step(0)
            eng.sync()
            graph = SystemGraph([eng], [w.frame(0)], [None], [topo["nummol"]])
            gpos = graph.frame_buffer(0)

            def step(i):  # noqa: F811 -- the graph form of the step
                with torch.cuda.stream(stream):
                    gpos.copy_(pos_d[i], non_blocking=True)
                graph.launch_ordered(stream.cuda_stream)

        ms = _timed(step, args.steps, args.warmup, stream)
        if graph is not None:
            graph.sync()
            graph.close()
        eng.sync()
        rates[adj] = ms / args.steps
        eng.close()
    units = w.nwater * args.steps
    line = {"metric": "solute-solvent molecule energies/s", "value": units / (rates[True] * args.steps / 1e3),
            "unit": "molecule-energies/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": rates[True], "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32+f64", "data": "synthetic",
            "config": {"workload": "soln_adjoint: 8000 waters, 62 A box, 16-site solute, PME 64^3, "
                                   "48 parameters, one frame per step"},
            "ms_per_frame_without_adjoint": rates[False]}
    if not args.no_graph:
        line["launch"] = "one CUDA graph launch per frame (ermod_graph_launch), frame copied into its input"
    if not args.no_cpu:
        from oracle import oracle as O
        O.build()
        orc = O.Oracle(w.params, topo, bins)
        pos, cl = w.frame(0)
        t0 = time.perf_counter()
        orc.frame(pos, cl)
        u_orc = orc.placements([topo["nummol"]])["uvengy"]
        du = orc.adjoint(topo["nummol"])
        dt = time.perf_counter() - t0
        line["cpu_baseline"] = {"value": w.nwater / dt, "unit": "molecule-energies/s", "cores": os.cpu_count(),
                                "kind": "port", "sample": "1 frame: energies + analytic FP64 derivatives"}
        # the same frame on the GPU: energies, and the bin-resolved derivatives against the
        # oracle's per-molecule derivatives binned by the GPU's energies
        eng = EnergyRepresentation(w.params, topo, bins, precision="mixed")
        eng.adjoint_enable()
        eng.frame(pos, cl)
        u_gpu = eng.placements([topo["nummol"]], want_uvengy=True)["uvengy"]
        grad, wt = eng.adjoint_get()
        eng.close()
        acc = accuracy_report(u_gpu, u_orc, bins["uvcrd"], mixed_band(w.solute))
        edges = np.asarray(bins["uvcrd"])
        b = np.searchsorted(edges, u_gpu[0, 1:-1], side="left") - 1  # the solute itself is the last molecule
        ref = np.zeros_like(grad)
        mag = np.zeros_like(grad)
        np.add.at(ref.T, b, du[:-1])
        np.add.at(mag.T, b, np.abs(du[:-1]))
        C = wt.sum() / max(len(b), 1)  # every molecule's weight: the volume factor
        # error per (parameter, bin) relative to the bin's summed magnitude, on bins holding at
        # least 1e-3 of the parameter's largest bin magnitude (elsewhere the derivatives of a
        # few molecules nearly cancel and only an absolute bound means anything)
        err = np.abs(grad / C - ref)
        big = mag >= 1e-3 * mag.max(axis=1, keepdims=True)
        acc["gradient_max_rel_err"] = float((err[big] / mag[big]).max())
        small = ~big & (mag > 0)
        acc["gradient_max_abs_err_small_bins"] = float(err[small].max()) if np.any(small) else 0.0
        acc["sample"] = "frame 0 against the FP64 oracle (energies and the oracle's analytic gradient)"
        line["accuracy"] = acc
    print(json.dumps(line))


def main():
    args = parse_args()
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "uneven":
        run_uneven(args)
    elif args.workload == "soln_adjoint":
        run_adjoint(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
