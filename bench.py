"""Benchmark of the fastreg registration loop on GB300.

One step = one whole registration (fastreg's FastReg::operator()) of the 182x218x182
synthetic pair for 200 iterations with the reference solver (params.ini values of the
reference: ALPHA=0.004, TAU=0.2, W_REG=0.2, RHO_0=1, p=2, C=0.25), inputs resident
in HBM.  Prints one JSON line.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

--impl reference times the reference algorithm's CPU implementation (the oracle
port, OpenMP over all host cores): one whole registration of the same pair per step;
its line also carries the reference's own CUDA kernels timed on the same pair.
Multi-GPU runs are independent replicas (one pair per rank, no collective on the
data path), and the shared-target cohort is split across the ranks by voxel count, one
batched call per rank; rank 0 prints.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "pairs/s at 182×218×182, 200 its, batched vs plain; warp GB/s vs HBM peak"
DIMS = (182, 218, 182)
ITERS = 200

# algorithmic bytes per interior voxel and launch (packed FP32: vector 12 B, scalar 4 B)
BYTES_LAPLACIAN = 12 + 4 + 16       # psi and T read, (L, T) interleaved written
BYTES_PASS_A = 4 + 12 + 12 + 16 + 4 + 4 + 12 + 12  # rho, v, psi_inv, (L, T) o psi_inv, S; rho, v, psi_inv
BYTES_PASS_B = 12 + 12 + 12         # psi, v o psi gathered, psi written
BYTES_ITER_CANONICAL = 112          # per voxel-iteration with L recomputed from psi (no L round trip)
BYTES_WARP = 12 + 4 + 4 + 2 + 2     # psi, image gathered, out, label gathered, out label


def reference_params(dims=DIMS, iters=ITERS, solver="reference"):
    from fastreg_gb300 import Params
    return Params(volume_dims=dims, volume_size=(1.0, 1.0, 1.0), no_labels=8, max_iter=iters,
                  max_update_norm=-1e-10, rho_0=1.0, tau=0.2, w_reg=0.2, alpha=0.004, p=2.0, C=0.25,
                  reset_iter=-1, verbosity=0, solver=solver, smooth_sigma=1.5, smooth_width=7, damping=0.9,
                  step=0.5)


def load_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            d = json.loads(p.read_text())
            return float(d["hbm_gbs"]), "measured"
        except Exception:
            pass
    return 6800.0, "fallback"


def load_traffic(kernel: str):
    """dram bytes per launch of `kernel` at the bench workload, from the committed ncu
    summary (a line 'dram_bytes_per_launch: <int>'), or None."""
    f = ROOT / "profiles" / f"{kernel}_182x218x182.txt"
    if not f.exists():
        return None
    for line in f.read_text().splitlines():
        if line.startswith("dram_bytes_per_launch:"):
            try:
                return int(float(line.split(":", 1)[1].strip()))
            except ValueError:
                return None
    return None


class ClockSampler:
    """nvidia-smi clock/throttle samples during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.file = None

    def start(self):
        try:
            self.file = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=self.file, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.file.flush()
        rows = []
        with open(self.file.name) as f:
            for line in f:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        os.unlink(self.file.name)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        smax = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": reasons, "samples": len(rows)}


def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("nccl")
    return ws, rank, local


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def allmax(ws, v):
    if ws == 1:
        return v
    from fastreg_gb300.replicas import max_over_ranks
    return max_over_ranks(v)


def cpu_registrations(data, P, n):
    """Time `n` whole registrations of the pair by the oracle port (the reference
    algorithm, FP32, OpenMP over the host cores); returns the seconds of each."""
    from oracle import oracle as O
    times = []
    for _ in range(n):
        t0 = time.perf_counter()
        O.ref_register(P, data["T"], data["labT"], data["S"], data["labS"])
        times.append(time.perf_counter() - t0)
    return times


def reference_cuda_timing(data, reps=3):
    """The reference's own CUDA kernels (compiled unmodified from its sources for sm_103a,
    launched in the order of its host code by the reference runner) on the same pair and
    settings: device time of the whole FastReg::operator() sequence and of estimate_psi
    alone, as the reference app times it (src/apps/demo.cpp:306-310).  None when the
    reference kernels are not built or there is no GPU."""
    try:
        import torch
        from oracle import ref_runner
        if not (torch.cuda.is_available() and ref_runner.available()):
            return None
        P = reference_params()
        runs = [ref_runner.register(P, data["T"], data["labT"], data["S"], data["labS"], timing=True)
                for _ in range(reps + 1)][1:]
    except Exception as e:  # the runner is test infrastructure: report, do not fail the line
        return {"unavailable": f"{type(e).__name__}: {e}"[:200]}
    op = [r["ms_operator"] for r in runs]
    ep = [r["ms_estimate_psi"] for r in runs]
    return {"what": "the reference's CUDA kernels built from its sources for sm_103a (its own nvcc flags), launched "
                    "in its order: 13 launches and 2 host synchronisations per iteration",
            "workload": "one 182x218x182 pair, 200 iterations, reference PDE solver (params.ini values)",
            "ms_operator": statistics.median(op), "ms_estimate_psi": statistics.median(ep),
            "pairs_per_s": 1000.0 / statistics.median(op), "runs": reps, "ms_operator_all": op}


def run_reference_arm(args):
    ws, rank, local = int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")), 0
    if rank != 0:
        return 0
    from fastreg_gb300 import synthetic as sy
    from oracle import build as obuild
    obuild.build()
    cores = os.cpu_count() or 1
    os.environ.setdefault("OMP_NUM_THREADS", str(cores))
    data = sy.make_pair(sy.PAIR_182X218X182)
    P = reference_params()
    # one step = one whole 200-iteration registration of the pair on the host cores
    cpu_registrations(data, P, args.warmup)
    times = cpu_registrations(data, P, args.steps)
    total = sum(times)
    value = args.steps / total
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "pairs/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * total / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": "one 182x218x182 pair, 200 iterations, reference PDE solver (params.ini values)",
                   "solver": "reference", "sample": "each step is one whole 200-iteration registration"},
        "cpu_baseline": {"value": value, "unit": "pairs/s", "cores": cores, "kind": "port",
                         "sample": "CPU oracle (OpenMP, FP32, op-order matched): whole 200-iteration registrations "
                                   "of the 182x218x182 pair, one per step"},
        "e2e": {"value": value, "unit": "pairs/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "step_s": [round(t, 3) for t in times],
    }
    ref_cuda = reference_cuda_timing(data)
    if ref_cuda is not None:
        line["reference_cuda"] = ref_cuda
    print(json.dumps(line))
    return 0


def profile_case(args):
    """The bench workload for ncu captures: one registration that settles the tile shapes
    (the autotuner's launches), then the profiled registration and warp inside the NVTX
    range "profile" (capture with --nvtx --nvtx-include "profile/").  With --solver adjoint:
    the differentiated registration of the 128^3 pair (--iters unrolled iterations,
    checkpoints every 10), once outside and once inside the range."""
    import torch
    if args.solver == "adjoint":
        import ctypes as C
        from fastreg_gb300 import synthetic as sy, _native as N
        lib = N.load()
        dev = torch.device("cuda", 0)
        d = sy.make_pair_torch(sy.PairSpec(dims=(128, 128, 128), n_blobs=40, vel_sigma=4.0, max_disp=4.0,
                                           n_classes=4, seed=4000), dev)
        v0 = (0.05 * torch.randn((3, 128, 128, 128), generator=torch.Generator().manual_seed(4001))).to(dev)
        gv = torch.empty_like(v0)
        P = reference_params(dims=(128, 128, 128), solver="sobolev")
        dims = (C.c_int * 3)(128, 128, 128)
        loss, gl = C.c_double(), C.c_double()
        for rep in range(2):
            if rep:
                torch.cuda.synchronize()
                torch.cuda.nvtx.range_push("profile")
            N.check(lib.fr_sobolev_loss_grad(d["T"].data_ptr(), d["S"].data_ptr(), dims, v0.data_ptr(), 0.2,
                                             args.iters, 10, P.damping, P.step, P.smooth_sigma, P.smooth_width,
                                             C.byref(loss), gv.data_ptr(), C.byref(gl), None), None,
                    "fr_sobolev_loss_grad")
            torch.cuda.synchronize()
        torch.cuda.nvtx.range_pop()
        print(f"profile case: adjoint, {args.iters} iterations, J {loss.value:.6g}, dJ/dlambda {gl.value:.6g}")
        return 0
    from fastreg_gb300 import FastReg, synthetic as sy, warp, _native as N
    dev = torch.device("cuda", 0)
    data = sy.make_pair(sy.PAIR_182X218X182)
    P = reference_params(DIMS, args.iters, solver=args.solver)
    P.staging = args.staging
    fr = FastReg(P)
    fresh = lambda: [torch.from_numpy(data[k]).to(dev) for k in ("T", "labT", "S", "labS")]  # noqa: E731
    fr(*fresh())
    bufs = fresh()
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_push("profile")
    fr(*bufs)
    psi = fr.get_field(N.FR_FIELD_PSI)
    img = torch.from_numpy(data["S"]).to(dev)
    lab = torch.from_numpy(data["labS"]).to(dev)
    warp(psi, img, lab)
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_pop()
    st = fr.stats()
    print(f"profile case: {args.solver} solver, {st.iterations} iterations, e_data {st.e_data:.6g}, "
          f"staging {fr.tile_staging()}, shapes {fr.tile_shapes()}")
    fr.close()
    return 0


def adjoint_timing(dev, stream, reps=3):
    import ctypes as C
    import torch
    from fastreg_gb300 import synthetic as sy, _native as N
    lib = N.load()
    spec = sy.PairSpec(dims=(128, 128, 128), n_blobs=40, vel_sigma=4.0, max_disp=4.0, n_classes=4, seed=4000)
    d = sy.make_pair_torch(spec, dev)
    g = torch.Generator(device="cpu").manual_seed(4001)
    v0 = (0.05 * torch.randn((3, 128, 128, 128), generator=g)).to(dev)
    gv = torch.empty_like(v0)
    dims = (C.c_int * 3)(128, 128, 128)
    loss, gl = C.c_double(), C.c_double()
    P = reference_params(dims=(128, 128, 128), solver="sobolev")
    times = []
    for rep in range(reps + 1):
        t0 = time.perf_counter()
        rc = lib.fr_sobolev_loss_grad(d["T"].data_ptr(), d["S"].data_ptr(), dims, v0.data_ptr(), 0.2, 50, 10,
                                      P.damping, P.step, P.smooth_sigma, P.smooth_width, C.byref(loss),
                                      gv.data_ptr(), C.byref(gl), stream.cuda_stream)
        N.check(rc, None, "fr_sobolev_loss_grad")
        if rep:
            times.append(time.perf_counter() - t0)
    return {"config": "128^3 pair, 50 unrolled sobolev iterations, gradient w.r.t. v0 (3x128^3) and lambda, "
                      "checkpoints every 10", "ms_forward_and_adjoint": 1000.0 * min(times),
            "loss": loss.value, "grad_lambda": gl.value}


def small_pair_timing(dev, stream, reps=5):
    """Registrations per second of the 64^3 pair (200 iterations), reference and sobolev
    solvers, inputs resident; after warm-up registrations (which also tune the shapes)."""
    import torch
    from fastreg_gb300 import FastReg, synthetic as sy
    d = sy.make_pair_torch(sy.PAIR_64CUBE, dev)
    pristine = [d[k] for k in ("T", "labT", "S", "labS")]
    work = [t.clone() for t in pristine]
    out = {"dims": list(sy.PAIR_64CUBE.dims), "iterations": ITERS}
    for solver in ("reference", "sobolev"):
        fr = FastReg(reference_params(dims=sy.PAIR_64CUBE.dims, solver=solver))
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            for rep in range(3 + reps):
                if rep == 3:
                    e0.record(stream)
                for w, p in zip(work, pristine):
                    w.copy_(p, non_blocking=True)
                fr(*work, stream=stream, sync=False)
            e1.record(stream)
        stream.synchronize()
        ms = e0.elapsed_time(e1) / reps
        out[solver] = {"pairs_per_s": 1000.0 / ms, "ms_per_pair": ms, "tile_shapes": fr.tile_shapes()}
        fr.close()
    return out


def hypergradient_cohort(dev, stream, n_pairs=32):
    """The shared-target cohort (32 x 160x192x160): each pair's W_REG tuned by 5
    hypergradient steps through a 30-iteration unrolled sobolev registration (adjoint
    kernels, checkpoints every 10), then one 200-iteration batched sobolev registration
    with the per-pair weights; Dice per class averaged over the pairs."""
    import numpy as np
    import torch
    from fastreg_gb300 import FastReg, synthetic as sy
    from fastreg_gb300.hypertune import register_cohort_tuned
    pairs = sy.shared_target_cohort(n_pairs, device=dev)
    work = [(d["T"].clone(), d["labT"].clone(), d["S"].clone(), d["labS"].clone()) for d in pairs]
    dims = tuple(reversed(work[0][0].shape))
    P = reference_params(dims=dims, solver="sobolev")
    P.no_labels = 8
    fr = FastReg(P)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    weights = register_cohort_tuned(fr, work, P, steps=5, iters=30, checkpoint_every=10, stream=stream)
    stream.synchronize()
    t_all = time.perf_counter() - t0
    dice = np.array([[fr.stats(k).dice[l] for l in range(1, 8)] for k in range(n_pairs)], np.float64)
    out = {"cohort": f"{n_pairs} sources of {dims[0]}x{dims[1]}x{dims[2]} to one shared target, sobolev solver",
           "tuning": "5 hypergradient steps per pair through a 30-iteration unrolled registration (checkpoints every "
                     "10), then one 200-iteration batched registration with the per-pair W_REG",
           "seconds_total": t_all, "w_reg_min": min(weights), "w_reg_max": max(weights),
           "dice_per_class_mean": [float(v) for v in np.nanmean(dice, 0)],
           "e_data_mean": float(np.mean([fr.stats(k).e_data for k in range(n_pairs)]))}
    fr.close()
    return out


def batched_vs_plain(dev, stream, pristine, solver, what, reps=2):
    """One fr_register_batch over a cohort against one fr_register per pair (a handle per
    pair size), same data and iterations: one warm-up and `reps` timed runs of each mode
    (CUDA events on `stream`, fastest run kept).  Then, untimed, every pair is registered
    alone once more and compared with its batched result: psi, both warped images and
    both warped label maps bit for bit, and the final SSD."""
    import torch
    from fastreg_gb300 import FastReg, _native as N
    n = len(pristine)
    work = [tuple(t.clone() for t in q) for q in pristine]
    dims = [tuple(reversed(q[0].shape)) for q in pristine]

    def restore(k=None):
        for j in (range(n) if k is None else [k]):
            for a_, b_ in zip(work[j], pristine[j]):
                a_.copy_(b_, non_blocking=True)

    frb = FastReg(reference_params(dims=dims[0], solver=solver))
    plain = {d: FastReg(reference_params(dims=d, solver=solver)) for d in sorted(set(dims))}
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    tb, tp = [], []
    with torch.cuda.stream(stream):
        for rep in range(reps + 1):
            restore()
            e0.record(stream)
            frb.register_batch(work, stream=stream, sync=False)
            e1.record(stream)
            stream.synchronize()
            if rep:
                tb.append(e0.elapsed_time(e1))
        out_b = [(frb.get_field(N.FR_FIELD_PSI, pair=k),) + tuple(t.clone() for t in work[k]) for k in range(n)]
        ssd_b = [frb.stats(k).e_data for k in range(n)]
        for rep in range(reps + 1):
            restore()
            e0.record(stream)
            for k in range(n):
                plain[dims[k]](*work[k], stream=stream, sync=False)
            e1.record(stream)
            stream.synchronize()
            if rep:
                tp.append(e0.elapsed_time(e1))
        names = ("psi", "T o psi_inv", "labels T", "S o psi", "labels S")
        mismatch = {}
        ssd_rel = []
        for k in range(n):  # every pair alone, against its batched result
            restore(k)
            fr = plain[dims[k]]
            fr(*work[k], stream=stream, sync=False)
            stream.synchronize()
            got = (fr.get_field(N.FR_FIELD_PSI),) + tuple(work[k])
            for nm, x, y in zip(names, got, out_b[k]):
                if not torch.equal(x, y):
                    mismatch.setdefault(nm, []).append(k)
            e = fr.stats().e_data
            ssd_rel.append(abs(ssd_b[k] - e) / max(abs(e), 1e-30))
    for fr in plain.values():
        fr.close()
    frb.close()
    t_b, t_p = min(tb), min(tp)
    voxels = sum(d[0] * d[1] * d[2] for d in dims)
    return {"cohort": what, "solver": solver, "pairs": n, "voxels": voxels, "iterations": ITERS,
            "batched_pairs_per_s": n / (t_b / 1000.0), "plain_pairs_per_s": n / (t_p / 1000.0),
            "ratio": t_p / t_b, "batched_ms": t_b, "plain_ms": t_p, "timed_runs": reps,
            "bitexact_batched_vs_plain": not mismatch, "compared": "psi, both warped images and both warped label "
                                                                  "maps of every pair",
            "mismatches": mismatch, "max_final_ssd_rel_diff": max(ssd_rel)}


def staging_variants(dev, stream, pristine, iters=20):
    """Per-kernel times of both solvers on the bench pair with each staging forced
    (STAGING=1: per-thread cp.async, STAGING=2: TMA tensor copies where a kernel has
    them), each with its own autotuned tile shapes: CUDA events around every launch of
    `iters` iterations (fr_time_kernels), after one registration."""
    import ctypes as C
    from fastreg_gb300 import FastReg, _native as N
    names = {"reference": ["ref_laplacian_kernel", "ref_pass_a_kernel", "ref_pass_b_kernel"],
             "sobolev": ["sob_grad_kernel", "sob_smooth3_kernel", "sob_pass_b_kernel"]}
    out = {}
    work = [t.clone() for t in pristine]
    for solver in ("reference", "sobolev"):
        for staging in (1, 2):
            P = reference_params(solver=solver)
            P.staging = staging
            fr = FastReg(P)
            for w, p in zip(work, pristine):
                w.copy_(p)
            fr(*work, stream=stream)
            fr.begin([tuple(work)], stream=stream)
            ms = (C.c_float * 8)()
            nk = C.c_int()
            N.check(fr.lib.fr_time_kernels(fr.h, iters, ms, C.byref(nk), stream.cuda_stream), fr.h,
                    "fr_time_kernels")
            stream.synchronize()
            out[f"{solver}_staging{staging}"] = {
                "kernels_ms": {n: ms[k] for k, n in enumerate(names[solver])},
                "staging": fr.tile_staging(), "tile_shapes": fr.tile_shapes()}
            fr.close()
    return out


def sharded_cohort(dev, stream, ws, rank, reps=2):
    """Replicas over several GPUs: the shared-target cohort (32 x 160x192x160, sobolev
    solver) split across the ranks by voxel count (replicas.shard_pairs), one
    fr_register_batch per rank over its pairs; the job's time is the slowest rank's
    (barrier before, max over ranks after); per-pair statistics gathered on rank 0."""
    import torch
    from fastreg_gb300 import FastReg, synthetic as sy
    from fastreg_gb300.replicas import gather_to_rank0, shard_pairs
    n, dims = 32, (160, 192, 160)
    mine = shard_pairs([dims[0] * dims[1] * dims[2]] * n, ws)[rank]
    cohort = sy.shared_target_cohort(n, dims=dims, device=dev)
    pristine = [(cohort[k]["T"], cohort[k]["labT"], cohort[k]["S"], cohort[k]["labS"]) for k in mine]
    work = [tuple(t.clone() for t in q) for q in pristine]
    fr = FastReg(reference_params(dims=dims, solver="sobolev"))
    times = []
    with torch.cuda.stream(stream):
        for rep in range(reps + 1):
            for w, p in zip(work, pristine):
                for a_, b_ in zip(w, p):
                    a_.copy_(b_, non_blocking=True)
            stream.synchronize()
            barrier(ws)
            t0 = time.perf_counter()
            fr.register_batch(work, stream=stream, sync=False)
            stream.synchronize()
            dt = allmax(ws, time.perf_counter() - t0)
            if rep:
                times.append(dt)
    stats = gather_to_rank0([(k, fr.stats(j).e_data) for j, k in enumerate(mine)])
    fr.close()
    t = min(times)
    return {"cohort": f"{n} sources of 160x192x160 to one shared target, sobolev solver, {ITERS} iterations",
            "ranks": ws, "pairs_per_rank": [len(x) for x in shard_pairs([1] * n, ws)], "seconds": t,
            "pairs_per_s": n / t, "e_data": sorted(x for r in (stats or []) for x in r) if stats else None}


def cohort_blocks(dev, stream):
    """The two cohorts with a batched target: the 16 uneven pairs and the 32 sources of
    160x192x160 registered to one shared target, each with both solvers."""
    from fastreg_gb300 import synthetic as sy
    specs = sy.cohort_specs(16)
    mixed = []
    for sp in specs:
        d = sy.make_pair_torch(sp, dev)
        mixed.append((d["T"], d["labT"], d["S"], d["labS"]))
    shared = [(d["T"], d["labT"], d["S"], d["labS"]) for d in sy.shared_target_cohort(32, device=dev)]
    w_mixed = ("16 pairs, dims per pair from {96,128,160,192}x{112,160,224}x{96,128,192}, max displacement "
               "2-6 voxels")
    w_shared = ("32 sources of 160x192x160 to one shared target (velocity sigma 5, max displacement 5, N(0,0.02) "
                "noise, 8 classes)")
    out = {}
    for solver in ("sobolev", "reference"):
        out[f"mixed_{solver}"] = batched_vs_plain(dev, stream, mixed, solver, w_mixed)
        out[f"shared_target_{solver}"] = batched_vs_plain(dev, stream, shared, solver, w_shared)
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-extras", action="store_true", help="skip the sobolev/warp/kernel/CPU measurements")
    ap.add_argument("--profile", action="store_true",
                    help="one registration of the bench pair with --iters iterations and one standalone warp, "
                         "for ncu (no timing, no JSON line)")
    ap.add_argument("--iters", type=int, default=ITERS, help="iterations of the --profile registration")
    ap.add_argument("--solver", default="reference", choices=["reference", "sobolev", "adjoint"],
                    help="solver of the --profile registration")
    ap.add_argument("--staging", type=int, default=0, choices=[0, 1, 2],
                    help="STAGING of the --profile registration (0: the autotuner's choice, 1: cp.async, 2: TMA)")
    args = ap.parse_args()
    if args.profile:
        return profile_case(args)
    if args.warmup < 3 and not args.profile:
        args.warmup = 3

    if args.impl == "reference":
        return run_reference_arm(args)

    ws, rank, local = dist_setup()
    import numpy as np
    import torch
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    from fastreg_gb300 import FastReg, synthetic as sy, warp, _native as N
    import ctypes as C

    spec = sy.PAIR_182X218X182
    if ws > 1:
        spec = sy.PairSpec(**{**spec.__dict__, "seed": spec.seed + rank})
    data = sy.make_pair(spec)
    P = reference_params()
    fr = FastReg(P)
    stream = torch.cuda.Stream(device=dev)
    pristine = [torch.from_numpy(data[k]).to(dev) for k in ("T", "labT", "S", "labS")]
    work = [t.clone() for t in pristine]

    def step():
        for w, p in zip(work, pristine):
            w.copy_(p, non_blocking=True)
        fr(*work, stream=stream, sync=False)

    # the first registration of a size class also runs the autotuner (a few tile shapes
    # per kernel, timed once and cached); it is part of the warm-up, timed on its own
    with torch.cuda.stream(stream):
        t_first = time.perf_counter()
        step()
        stream.synchronize()
        t_first = time.perf_counter() - t_first
        for _ in range(max(args.warmup - 2, 0)):  # first + these + the next one = warmup
            step()
        stream.synchronize()
        t_next = time.perf_counter()
        step()
        stream.synchronize()
        t_next = time.perf_counter() - t_next
    shapes_ref = fr.tile_shapes()

    sampler = ClockSampler(local)
    barrier(ws)
    torch.cuda.synchronize()
    sampler.start()
    time.sleep(0.3)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with torch.cuda.stream(stream):
        e0.record(stream)
        for _ in range(args.steps):
            step()
        e1.record(stream)
    stream.synchronize()
    torch.cuda.synchronize()
    clocks = sampler.stop()
    barrier(ws)
    ms = e0.elapsed_time(e1)
    ms_max = allmax(ws, ms)
    value = ws * args.steps / (ms_max / 1000.0)
    st = fr.stats()

    # end to end through the public API with host buffers: H2D of the inputs, the
    # registration, D2H of the warped images/labels and of the statistics
    host_in = [t.cpu().pin_memory() for t in pristine]
    host_out = [torch.empty_like(t).pin_memory() for t in host_in]
    h2d = sum(t.numel() * t.element_size() for t in host_in)
    d2h = h2d + C.sizeof(N.fr_stats)
    e2e_steps = max(1, args.steps)

    def e2e_step():
        for w, h in zip(work, host_in):
            w.copy_(h, non_blocking=True)
        fr(*work, stream=stream, sync=False)
        for h, w in zip(host_out, work):
            h.copy_(w, non_blocking=True)
        stream.synchronize()
        fr.stats()

    with torch.cuda.stream(stream):
        e2e_step()
        barrier(ws)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        e0.record(stream)
        step_ms = []
        for _ in range(e2e_steps):
            ts = time.perf_counter()
            e2e_step()
            step_ms.append(round((time.perf_counter() - ts) * 1e3, 3))
        e1.record(stream)
        stream.synchronize()
        t_e2e = time.perf_counter() - t0
    e2e_max = allmax(ws, t_e2e)
    e2e_value = ws * e2e_steps / e2e_max

    line = {
        "metric": METRIC, "value": value, "unit": "pairs/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded: 400 Gaussian blobs + N(0,0.01), smooth velocity sigma 6, max disp 6, 8 classes)",
        "config": {"workload": "one 182x218x182 pair, 200 iterations, reference PDE solver (params.ini values)",
                   "solver": "reference", "voxels": int(np.prod(DIMS)), "iterations": ITERS,
                   "other_solver": "the workload's Gaussian-smoothed (sobolev) settings -- width 7, sigma 1.5, "
                                   "damping 0.9, step 0.5 -- are timed on the same pair in the 'sobolev' block",
                   "parallelism": f"replicas x{ws}" if ws > 1 else "single GPU",
                   "l2": "working set ~0.7 GB per pair, larger than L2 (no flush needed)"},
        "voxel_iters_per_s": value * int(np.prod(DIMS)) * ITERS,
        "e2e": {"value": e2e_value, "unit": "pairs/s", "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                "steps": e2e_steps, "step_ms": step_ms},
        "gpu_launches": args.steps * (2 + 3 * ITERS),
        "clocks": clocks,
        "result": {"iterations": st.iterations, "e_data": st.e_data, "e_reg": st.e_reg, "folds": st.folds,
                   "dice_all": st.dice_all},
        "tile_shapes": {"kernels": ["ref_laplacian_kernel", "ref_pass_a_kernel", "ref_pass_b_kernel"],
                        "slices_and_blocks_per_sm": shapes_ref,
                        "autotune_s": max(0.0, t_first - t_next)},
    }

    if ws > 1 and not args.no_extras:
        # every rank takes part: its share of the shared-target cohort in one batched call
        line["cohort_replicas"] = sharded_cohort(dev, stream, ws, rank)

    if rank == 0 and not args.no_extras and not args.profile:
        peak, peak_kind = load_peaks()
        # per-kernel durations (CUDA events around each launch on `stream`)
        fr.begin([tuple(work)], stream=stream)
        ms_k = (C.c_float * 8)()
        nk = C.c_int()
        N.check(fr.lib.fr_time_kernels(fr.h, 20, ms_k, C.byref(nk), stream.cuda_stream), fr.h, "fr_time_kernels")
        stream.synchronize()
        ni = (DIMS[0] - 2) * (DIMS[1] - 2) * (DIMS[2] - 2)
        kern = {"ref_laplacian_kernel": (ms_k[0], BYTES_LAPLACIAN * ni),
                "ref_pass_a_kernel": (ms_k[1], BYTES_PASS_A * ni),
                "ref_pass_b_kernel": (ms_k[2], BYTES_PASS_B * ni)}
        top = max(kern, key=lambda k: kern[k][0])
        t_top, b_top = kern[top]
        achieved = b_top / (t_top * 1e-3) / 1e9
        traffic = load_traffic(top)
        line["roofline"] = {"bound": "hbm", "kernel": top, "achieved": achieved, "peak": peak, "unit": "GB/s",
                            "frac": achieved / peak, "traffic": traffic, "peak_kind": peak_kind,
                            "algorithmic_bytes_per_launch": b_top}
        line["kernels_ms"] = {k: v[0] for k, v in kern.items()}
        line["kernels_gbs"] = {k: v[1] / (v[0] * 1e-3) / 1e9 for k, v in kern.items()}
        iter_ms = sum(v[0] for v in kern.values())
        line["iteration"] = {"ms": iter_ms, "canonical_bytes_per_voxel": BYTES_ITER_CANONICAL,
                             "effective_gbs": BYTES_ITER_CANONICAL * int(np.prod(DIMS)) / (iter_ms * 1e-3) / 1e9}

        # standalone warp (apply): S o psi with the final psi of the registration
        psi = fr.get_field(N.FR_FIELD_PSI)
        img, lab = pristine[2], pristine[3]
        out, out_lab = torch.empty_like(img), torch.empty_like(lab)
        with torch.cuda.stream(stream):
            for _ in range(3):
                warp(psi, img, lab, stream=stream, out=out, out_lab=out_lab)
            w0, w1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            w0.record(stream)
            for _ in range(20):
                warp(psi, img, lab, stream=stream, out=out, out_lab=out_lab)
            w1.record(stream)
        stream.synchronize()
        wms = w0.elapsed_time(w1) / 20
        wgbs = BYTES_WARP * int(np.prod(DIMS)) / (wms * 1e-3) / 1e9
        line["warp"] = {"ms": wms, "gbs": wgbs, "frac_of_peak": wgbs / peak, "bytes_per_voxel": BYTES_WARP}

        # the sobolev solver (SSD + Gaussian-smoothed gradient + momentum) on the same pair
        Ps = reference_params(solver="sobolev")
        frs = FastReg(Ps)
        with torch.cuda.stream(stream):
            for _ in range(2):
                for w, p in zip(work, pristine):
                    w.copy_(p, non_blocking=True)
                frs(*work, stream=stream, sync=False)
            s0, s1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            s0.record(stream)
            for _ in range(3):
                for w, p in zip(work, pristine):
                    w.copy_(p, non_blocking=True)
                frs(*work, stream=stream, sync=False)
            s1.record(stream)
        stream.synchronize()
        sms = s0.elapsed_time(s1) / 3
        ss = frs.stats()
        frs.begin([tuple(work)], stream=stream)
        N.check(frs.lib.fr_time_kernels(frs.h, 20, ms_k, C.byref(nk), stream.cuda_stream), frs.h, "fr_time_kernels")
        stream.synchronize()
        sob_k = {"sob_grad_kernel": ms_k[0], "sob_smooth3_kernel": ms_k[1], "sob_pass_b_kernel": ms_k[2]}
        line["sobolev"] = {"value": 1000.0 / sms, "unit": "pairs/s", "ms_per_pair": sms, "kernels_ms": sob_k,
                           "tile_shapes": frs.tile_shapes(), "e_data": ss.e_data,
                           "e_data_initial": float(0.5 * ((data["T"].astype(np.float64) -
                                                           data["S"].astype(np.float64)) ** 2).sum()),
                           "folds": ss.folds, "dice_all": ss.dice_all}
        frs.close()

        # each kernel with either staging of its stencil operands (cp.async / TMA)
        line["staging_variants"] = staging_variants(dev, stream, pristine)

        # the 64^3 single-pair workload (the CPU-runnable configuration), both solvers
        line["pair_64cube"] = small_pair_timing(dev, stream)

        # batched cohorts against plain per-pair calls, 200 iterations each, both solvers:
        # 16 uneven pairs, and the shared-target cohort the batched target is quoted on
        # (32 x 160x192x160)
        line["batched"] = cohort_blocks(dev, stream)
        # the same cohort with per-pair weights tuned by hypergradients (adjoint kernels)
        line["hypergradient_cohort"] = hypergradient_cohort(dev, stream)

        # the differentiated registration: 128^3 pair, 50 iterations unrolled, gradient of
        # J = SSD + 0.1 |m_K|^2 with respect to v0 and lambda, checkpoints every 10
        line["adjoint"] = adjoint_timing(dev, stream)

        # CPU baseline: the oracle port on the host cores, bounded sample of two whole
        # registrations (about 15 s of CPU work)
        cores = os.cpu_count() or 1
        os.environ.setdefault("OMP_NUM_THREADS", str(cores))
        ct = cpu_registrations(data, P, 2)
        line["cpu_baseline"] = {"value": len(ct) / sum(ct), "unit": "pairs/s", "cores": cores, "kind": "port",
                                "sample": "CPU oracle (OpenMP, FP32) on the 182x218x182 pair: two whole "
                                          f"200-iteration registrations ({', '.join(f'{t:.2f}' for t in ct)} s)"}

    if rank == 0:
        print(json.dumps(line))
    fr.close()
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
