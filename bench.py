#!/usr/bin/env python3
"""Benchmark: pair evaluations/s of the GB300 pair counter on the reference's headline workload.

Workload (one step = one full countpairs() call: device gridlink, device worklist, pair kernel,
histogram read-back): DD(r) cross-correlation with pair_product weights, N1 = N2 = 2,000,000
clustered points (80% in Gaussian blobs of sigma 2, Poisson occupancy 80; 20% uniform) in a
periodic L = 1000 box, 25 log bins 0.1-50, float64 positions, FP32 classification + FP64 edge
re-evaluation.  Seeded synthetic inputs stand in for a survey catalogue.

Units: pair evaluations = candidate pairs of the *reference's* lattice (computed by
cf_reference_candidate_pairs, a restatement of the reference's gridlink + cell-pair list), so
the number does not depend on how the GPU tiles the work.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line.  With --gpus N > 1 (launched by torchrun) every rank runs an independent
replica of the workload on its own GPU ("replicas only": the path needs no collective).
"""
import argparse
import atexit
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "pair evaluations/sec (reference-lattice candidate pairs), DD cross-correlation"
UNIT = "pairs/s"
WORKLOADS = {
    "cfg2": dict(workload="theory DD cross-correlation with pair_product weights, N1=N2=2,000,000 clustered "
                          "points, periodic L=1000, 25 log bins 0.1-50, float64",
                 n1=2_000_000, n2=2_000_000, boxsize=1000.0, nbins=25, rmin=0.1, rmax=50.0, seeds=[1, 2],
                 weights="U[0.5,1.5]", kind="clustered", autocorr=0),
    "northstar": dict(workload="theory DD auto-correlation, N=1,000,000 uniform points, periodic L=420, "
                               "20 log bins 0.1-25, float64",
                      n1=1_000_000, n2=0, boxsize=420.0, nbins=20, rmin=0.1, rmax=25.0, seeds=[0],
                      weights=None, kind="uniform", autocorr=1),
}
WORKLOADS["cfg5"] = dict(workload="batched DD cross-correlations: 64 clustered catalogues of 50,000-500,000 points "
                                   "(log-uniform sizes) against one 5,000,000-point uniform catalogue, periodic "
                                   "L=1000, 20 log bins 0.1-25, float32 positions, pair_product weights U[0.5,1.5]",
                          nbatch=64, nmin=50_000, nmax=500_000, n2=5_000_000, boxsize=1000.0, nbins=20, rmin=0.1,
                          rmax=25.0, size_seed=100, seeds="0-63", random_seed=1000, weights="U[0.5,1.5]",
                          kind="batched", autocorr=0)
WORKLOADS["survey"] = dict(workload="DDrppi_mocks auto-correlation of a synthetic redshift survey of 84,383 galaxies "
                                    "(RA 110-266, DEC -4-70, cz 6,000-20,000 km/s, 60% in groups), cosmology 1, "
                                    "pimax 40, 14 log rp bins 0.1-25, pair_product weights, float64",
                           n1=84_383, n2=0, nbins=14, rmin=0.1, rmax=25.0, pimax=40.0, seeds=[5, 6],
                           weights="U[0.5,1.5]", kind="survey", autocorr=1)
WORKLOAD = dict(WORKLOADS["cfg2"])
FLOP_PER_PAIR = 8  # 3 FADD + 1 FMUL + 2 FFMA per 3-D separation
# dram__bytes_read.sum + dram__bytes_write.sum of one FP32 pair-kernel launch per workload and split
# of the j lattice's columns (1: unsplit), from an ncu capture of this kernel on that workload (a
# recorded constant, not measured by this script)
PAIR_KERNEL_TRAFFIC_BYTES = {("cfg2", 1): 829_490_944 + 21_026_816, ("cfg2", 4): 548_401_664 + 9_282_560,
                             ("northstar", 1): 55_271_424 + 2_289_920}
TRAFFIC_SOURCE = ("ncu capture of the pair kernel on this workload (dram__bytes_read.sum + dram__bytes_write.sum "
                  "per launch): a recorded constant, not measured in this run")


def gridlink_roofline(ms, ncells):
    """The lattice build against the HBM copy rate, by the byte count of the path's survey: per
    lattice N (3 + nw) x (input element) read, N (3 + nw) x (4 + 8) written (FP32 cell-local and FP64
    copies), N x 4 x 2 (cell ids written and read) and ncells x 8 x 2 (counts and offsets)."""
    ew = 8 if WORKLOAD.get("dtype", "float64") == "float64" else 4
    nw = 1 if WORKLOAD["weights"] else 0
    sets = [WORKLOAD["n1"]] + ([] if WORKLOAD["autocorr"] else [WORKLOAD["n2"]])
    nbytes = sum(n * (3 + nw) * ew + n * (3 + nw) * 12 + n * 8 + ncells * 16 for n in sets)
    peak = measured_hbm_gbs()
    gbs = nbytes / (ms / 1e3) / 1e9 if ms > 0 else None
    return {"bound": "hbm", "bytes": nbytes, "ms": ms, "achieved": gbs, "peak": peak, "unit": "GB/s",
            "frac": gbs / peak if (gbs and peak) else None,
            "peak_source": "MEASURED_PEAKS.json hbm_gbs" if peak else None,
            "kernels": "k_assign, k_scan_tile / k_scan_add, k_scatter (CUDA events around the lattice build)"}


def measured_hbm_gbs():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"])
    except Exception:
        return None


def _rank_env():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("LOCAL_RANK", "0"))


def max_over_ranks(seconds, world, device):
    """Replicas only: every rank times its own copy of the workload; the job's time is the
    slowest rank's (all ranks take part in the reduction)."""
    if world <= 1:
        return seconds
    import torch
    import torch.distributed as dist
    t = torch.tensor([seconds], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.barrier()
    return float(t.item())


def replica_throughput(work_per_step, steps, seconds, world):
    """Whole-job throughput of `world` replicas, each doing `work_per_step` per step."""
    return world * work_per_step * steps / seconds


def make_workload(dtype=np.float64):
    from corrfunc_gb300 import catalogs as cat
    L = WORKLOAD["boxsize"]
    gen = cat.clustered_box if WORKLOAD["kind"] == "clustered" else cat.uniform_box
    x1, y1, z1 = gen(WORKLOAD["n1"], L, WORKLOAD["seeds"][0], dtype=dtype)
    w1 = cat.weights(WORKLOAD["n1"], 101, dtype=dtype)
    if WORKLOAD["autocorr"]:
        set2 = (x1, y1, z1, w1)
    else:
        x2, y2, z2 = gen(WORKLOAD["n2"], L, WORKLOAD["seeds"][1], dtype=dtype)
        set2 = (x2, y2, z2, cat.weights(WORKLOAD["n2"], 102, dtype=dtype))
    bins = cat.log_bins(WORKLOAD["rmin"], WORKLOAD["rmax"], WORKLOAD["nbins"])
    return (x1, y1, z1, w1), set2, bins


def options_for(C, L, dtype):
    o = C.get_config_options()
    o.verbose = 0
    o.periodic = 1
    o.boxsize_x = o.boxsize_y = o.boxsize_z = L
    o.float_type = np.dtype(dtype).itemsize
    o.instruction_set = 0
    return o


def extra_for(C, w1, w2):
    if WORKLOAD["weights"] is None:
        return C.get_extra_options()
    e = C.get_extra_options(C.WEIGHT_PAIR_PRODUCT)
    e.weights0.weights[0] = w1
    e.weights1.weights[0] = w2
    e.weights0.num_weights = e.weights1.num_weights = 1
    return e


def reference_work(C, set1, set2, binfile, dtype, boxsize=None):
    """Candidate pairs of the reference's lattice for this count (host-only library: loads no GPU
    code, so the CPU-only reference arm can use it too)."""
    o = options_for(C, WORKLOAD["boxsize"] if boxsize is None else boxsize, dtype)
    auto = 1 if set2[0] is set1[0] else 0
    return C.reference_candidate_pairs(set1, set2, binfile, o, auto)


class ClockSampler:
    """nvidia-smi clocks / throttle reasons, sampled every 50 ms by one process that runs for the
    whole benchmark.  A timed region is bracketed by `window()`; its summary takes the samples
    from 0.3 s before to 0.3 s after the region (the warm-up and end-to-end loops around it keep
    the GPU under load), since a region of a few milliseconds holds no sample of its own."""

    FIELDS = ["clocks.sm", "clocks.max.sm", "power.draw", "clocks_event_reasons.hw_slowdown",
              "clocks_event_reasons.hw_thermal_slowdown", "clocks_event_reasons.sw_thermal_slowdown",
              "clocks_event_reasons.sw_power_cap"]
    MARGIN_S = 0.3
    _running = {}

    def __init__(self, device_index):
        self.dev = device_index
        self.proc = None
        self.lines = []  # (perf_counter time, csv line)

    @classmethod
    def shared(cls, device_index):
        if device_index not in cls._running:
            smp = cls(device_index)
            smp.start()
            cls._running[device_index] = smp
        return cls._running[device_index]

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.dev), "--query-gpu=" + ",".join(self.FIELDS),
                                          "--format=csv,noheader,nounits", "-lms", "50"], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            atexit.register(self.stop)
            t_end = time.perf_counter() + 2.0  # wait for the first sample
            while not self.lines and time.perf_counter() < t_end and self.proc.poll() is None:
                time.sleep(0.01)
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append((time.perf_counter(), ln.strip()))

    def stop(self):
        if self.proc is not None and self.proc.poll() is None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self, t0=None, t1=None):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for t, ln in list(self.lines):
            if t0 is not None and not (t0 - self.MARGIN_S <= t <= t1 + self.MARGIN_S):
                continue
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[3:7]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


class _ClockWindow:
    """`with clock_window(dev) as clocks:` around a timed region; `clocks.summary()` afterwards
    (called after the region and the loops that follow it, so that the trailing margin is in)."""

    def __init__(self, device_index):
        self.smp = ClockSampler.shared(device_index)

    def __enter__(self):
        self.t0 = time.perf_counter()
        return self

    def __exit__(self, *exc):
        self.t1 = time.perf_counter()
        return False

    def summary(self):
        wait = self.t1 + ClockSampler.MARGIN_S + 0.06 - time.perf_counter()
        if wait > 0:
            time.sleep(wait)
        return self.smp.summary(self.t0, self.t1)


def clock_window(device_index):
    return _ClockWindow(device_index)


def flush_l2(torch, dev):
    # write a buffer larger than the 129 MB L2 between timed steps
    if not hasattr(flush_l2, "buf"):
        flush_l2.buf = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=dev)
    flush_l2.buf.fill_(1.0)
    torch.cuda.synchronize(dev)


def cpu_reference_run(set1, set2, bins, nthreads, dtype, frac=1.0):
    """The reference's own countpairs() (oracle/_ref, all host threads) on a subsample keeping a
    fraction `frac` of each catalogue; returns (seconds, reference-lattice candidates)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    from corrfunc_gb300 import _capi as C
    from corrfunc_gb300 import theory
    so = os.path.join(ROOT, "oracle", "_ref", "libcf_ref_DD.so")
    if not os.path.exists(so):
        return None
    ref = C.bind(so)
    n1 = int(len(set1[0]) * frac)
    n2 = int(len(set2[0]) * frac)
    s1 = tuple(np.ascontiguousarray(a[:n1]) for a in set1)
    s2 = tuple(np.ascontiguousarray(a[:n2]) for a in set2)
    wkw = dict(weights1=s1[3], weights2=s2[3], weight_type="pair_product") if WORKLOAD["weights"] else {}
    t0 = time.perf_counter()
    if WORKLOAD["autocorr"]:
        wkw.pop("weights2", None)
        theory.run_DD(ref, 1, nthreads, bins, s1[0], s1[1], s1[2], periodic=True, boxsize=WORKLOAD["boxsize"],
                      isa="fastest", **wkw)
        s2 = s1
    else:
        theory.run_DD(ref, 0, nthreads, bins, s1[0], s1[1], s1[2], X2=s2[0], Y2=s2[1], Z2=s2[2], periodic=True,
                      boxsize=WORKLOAD["boxsize"], isa="fastest", **wkw)
    dt = time.perf_counter() - t0
    with C.BinFile(bins) as bf:
        work = reference_work(C, s1, s2, bf, dtype)
    return dt, work, n1, n2


def _batch_catalogue(args):
    """One clustered float32 catalogue of the batched workload (run in a worker process)."""
    n, L, k = args
    sys.path.insert(0, ROOT)
    from corrfunc_gb300 import catalogs as cat
    x, y, z = cat.clustered_box(int(n), L, k, dtype=np.float32)
    return (x, y, z, cat.weights(int(n), 200 + k, dtype=np.float32))


def make_batch_workload():
    import multiprocessing as mp
    from corrfunc_gb300 import catalogs as cat
    W = WORKLOAD
    rng = np.random.default_rng(W["size_seed"])
    sizes = np.round(np.exp(rng.uniform(np.log(W["nmin"]), np.log(W["nmax"]), W["nbatch"]))).astype(np.int64)
    L = W["boxsize"]
    # worker processes started by spawn (this process may already hold a CUDA context)
    with mp.get_context("spawn").Pool(min(16, os.cpu_count() or 1)) as pool:
        cats = pool.map(_batch_catalogue, [(int(n), L, k) for k, n in enumerate(sizes)])
    x, y, z = cat.uniform_box(W["n2"], L, W["random_seed"], dtype=np.float32)
    rand = (x, y, z, cat.weights(W["n2"], 2000, dtype=np.float32))
    bins = cat.log_bins(W["rmin"], W["rmax"], W["nbins"])
    return cats, rand, bins


def batch_work(C, cats, rand, binfile):
    """Reference-lattice candidates of every catalogue against the random catalogue (host counter,
    one thread per catalogue: ctypes releases the interpreter lock during the call)."""
    from concurrent.futures import ThreadPoolExecutor
    with ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 1)) as ex:
        return sum(ex.map(lambda c: reference_work(C, c, rand, binfile, np.float32), cats))


def run_batch_workload(args):
    """Configuration 5 as the headline line (``--workload cfg5``)."""
    rank, world, local = _rank_env()
    import torch
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    import corrfunc_gb300
    corrfunc_gb300.set_precision(args.precision)
    rec = batch_record(args, torch, dev, local, world, e2e=True)
    line = {"metric": "pair evaluations/sec (reference-lattice candidate pairs), batched DD cross-correlations",
            "value": rec["value"], "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": max(args.warmup, 3),
            "ms_per_step": rec["ms_per_step"], "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32+f64-refine" if args.precision == "fp32_refine" else "f64",
            "data": "synthetic (seeded clustered and uniform catalogues, numpy PCG64)",
            "config": dict(WORKLOAD, precision=args.precision, l2="flushed between steps (256 MB write)",
                           reference_lattice_candidates=rec["pairs"]["reference_lattice_candidates"],
                           catalogue_points=rec["catalogue_points"])}
    for k in ("roofline", "e2e", "gpu_launches", "batch", "pairs", "clocks"):
        line[k] = rec[k]
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cats, rand, bins = rec.pop("_data")
        r = cpu_batch_reference(cats, rand, bins, os.cpu_count() or 1)
        line["cpu_baseline"] = None if r is None else {
            "value": r[1] / r[0], "unit": UNIT, "cores": os.cpu_count(), "kind": "reference",
            "sample": "the first %d catalogues against the full random catalogue, one run" % r[2], "seconds": r[0]}
    rec.pop("_data", None)
    if rank == 0:
        print(json.dumps(line))


def batch_record(args, torch, dev, local, world=1, e2e=False):
    """Configuration 5: 64 clustered catalogues (50k-500k points) against one 5M-point uniform
    catalogue, all in one replayed CUDA graph (one pair-kernel launch), against the same catalogues
    counted by 64 sequential countpairs() calls (which the batch must equal, catalogue by
    catalogue).  Returns the measurement as a dict (with the data under "_data")."""
    import corrfunc_gb300
    from corrfunc_gb300 import _capi as C
    from corrfunc_gb300 import theory
    saved = dict(WORKLOAD)
    WORKLOAD.clear()
    WORKLOAD.update(WORKLOADS["cfg5"])
    try:
        lib = corrfunc_gb300.library()
        lib.cf_gpu_countpairs_device.argtypes = lib.countpairs.argtypes
        lib.cf_gpu_countpairs_device.restype = ctypes.c_int
        lib.cf_gpu_fp32_peak_tflops.argtypes = [ctypes.POINTER(ctypes.c_double)]
        cats, rand, bins = make_batch_workload()
        L = WORKLOAD["boxsize"]
        binf = C.BinFile(bins)
        binfile = binf.__enter__()
        work = batch_work(C, cats, rand, binfile)
        dcats = [[torch.from_numpy(a).to(dev) for a in c] for c in cats]
        drand = [torch.from_numpy(a).to(dev) for a in rand]
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        batch = theory.DDCrossBatch(bins, dcats, drand, periodic=True, boxsize=L, weight_type="pair_product",
                                    autotune=True)
        plan_s = time.perf_counter() - t0
        o = options_for(C, L, np.float32)

        def one_plain(k):
            c = dcats[k]
            e = extra_for(C, c[3].data_ptr(), drand[3].data_ptr())
            res = C.ResultsDD()
            rc = lib.cf_gpu_countpairs_device(len(cats[k][0]), *(ctypes.c_void_p(t.data_ptr()) for t in c[:3]),
                                              WORKLOAD["n2"], *(ctypes.c_void_p(t.data_ptr()) for t in drand[:3]), 1,
                                              0, binfile.encode(), ctypes.byref(res), ctypes.byref(o), ctypes.byref(e))
            if rc != 0:
                raise RuntimeError("countpairs on device inputs failed")
            npairs = np.ctypeslib.as_array(res.npairs, shape=(res.nbin,)).copy()
            lib.free_results(ctypes.byref(res))
            return npairs, corrfunc_gb300.last_stats()

        # parity of the batch against the plain path on every catalogue (outside the timed region)
        first = batch.run()
        for k in range(len(cats)):
            npairs, _ = one_plain(k)
            if not np.array_equal(first[k]["npairs"], npairs[1:]):
                raise RuntimeError("batched counts differ from countpairs() for catalogue %d" % k)

        ClockSampler.shared(local)
        for _ in range(max(args.warmup, 3)):
            batch.run()
            flush_l2(torch, dev)
        gpu_ms, pair_ms, launches, evaluated, refined = [], [], 0, 0, 0
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize(dev)
        with clock_window(local) as clocks:
            for _ in range(args.steps):
                out = batch.run()
                st = corrfunc_gb300.last_stats()
                if not all(np.array_equal(a["npairs"], b["npairs"]) for a, b in zip(out, first)):
                    raise RuntimeError("non-deterministic batched counts")
                gpu_ms.append(st["total_gpu_ms"])
                pair_ms.append(st["pair_kernel_ms"])
                launches += st["kernel_launches"]
                evaluated += st["pairs_evaluated"]
                refined += st["pairs_refined"]
                flush_l2(torch, dev)
        torch.cuda.synchronize(dev)
        batch_st = st  # the replayed plan's statistics (the calls below overwrite them)
        total_s = max_over_ranks(sum(gpu_ms) / 1e3, world, dev)
        value = replica_throughput(work, args.steps, total_s, world)

        # the same 64 counts as 64 sequential plain calls (device inputs), GPU time per call summed
        seq_ms = []
        for _ in range(2):
            tot = 0.0
            for k in range(len(cats)):
                _, st2 = one_plain(k)
                tot += st2["total_gpu_ms"]
            seq_ms.append(tot)
            flush_l2(torch, dev)

        rec_e2e = None
        if e2e:
            # end to end: copy every catalogue from pinned host memory, replay, read the histograms back
            hcats = [[torch.from_numpy(a).pin_memory() for a in c] for c in cats]
            hrand = [torch.from_numpy(a).pin_memory() for a in rand]
            h2d = sum(t.numel() * t.element_size() for c in hcats for t in c) + sum(t.numel() * t.element_size()
                                                                                  for t in hrand)
            d2h = len(cats) * (WORKLOAD["nbins"] + 1) * 3 * 8
            e2e_t = []
            for _ in range(args.steps):
                flush_l2(torch, dev)
                t0 = time.perf_counter()
                for dc, hc in zip(dcats, hcats):
                    for d, h in zip(dc, hc):
                        d.copy_(h, non_blocking=True)
                for d, h in zip(drand, hrand):
                    d.copy_(h, non_blocking=True)
                torch.cuda.synchronize(dev)
                batch.run()
                e2e_t.append(time.perf_counter() - t0)
            rec_e2e = {"value": world * work * args.steps / sum(e2e_t), "unit": UNIT, "h2d_bytes_per_step": h2d,
                       "d2h_bytes_per_step": d2h, "ms_per_step": 1e3 * sum(e2e_t) / args.steps}

        peak = ctypes.c_double()
        lib.cf_gpu_fp32_peak_tflops(ctypes.byref(peak))
        pair_s = sum(pair_ms) / 1e3 / args.steps
        achieved = work * FLOP_PER_PAIR / pair_s / 1e12
        st = batch_st
        rec = {"workload": WORKLOAD["workload"], "value": value, "unit": UNIT, "ms_per_step": sum(gpu_ms) / args.steps,
               "roofline": {"bound": "fp32", "achieved": achieved, "peak": peak.value, "unit": "TFLOP/s",
                            "frac": achieved / peak.value if peak.value else None, "traffic": None,
                            "kernel": "k_pairs_chunks<weights> (merged form; one launch for all catalogues)",
                            "peak_source": "measured: FP32 FMA calibration kernel (cf_gpu_fp32_peak_tflops) in this run",
                            "flop_per_pair": FLOP_PER_PAIR},
               "e2e": rec_e2e, "gpu_launches": launches,
               "batch": {"graph_ms": sum(gpu_ms) / args.steps, "pair_kernel_ms": sum(pair_ms) / args.steps,
                         "sequential_64_calls_ms": min(seq_ms),
                         "speedup_vs_sequential": min(seq_ms) / (sum(gpu_ms) / args.steps),
                         "plan_s": plan_s, "kernels_per_graph": st["kernel_launches"],
                         "tuned_layout": {"lane_stride": st["lane_stride"], "warps_per_block": st["warps_per_block"]},
                         "parity": "every catalogue equal to countpairs() on the same device arrays"},
               "pairs": {"reference_lattice_candidates": work, "gpu_evaluated": evaluated // args.steps,
                         "fp64_refined": refined // args.steps,
                         "counted": int(sum(int(a["npairs"].sum()) for a in first))},
               "catalogue_points": int(sum(len(c[0]) for c in cats)),
               "clocks": clocks.summary(), "_data": (cats, rand, bins)}
        batch.close()
        binf.__exit__(None, None, None)
        return rec
    finally:
        WORKLOAD.clear()
        WORKLOAD.update(saved)


def cpu_batch_reference(cats, rand, bins, nthreads, ncat=4):
    """The reference's countpairs() (oracle/_ref) on the first ncat catalogues against the random
    catalogue; returns (seconds, reference-lattice candidates, ncat)."""
    from corrfunc_gb300 import _capi as C
    from corrfunc_gb300 import theory
    so = os.path.join(ROOT, "oracle", "_ref", "libcf_ref_DD.so")
    if not os.path.exists(so):
        return None
    ref = C.bind(so)
    dt, work = 0.0, 0
    with C.BinFile(bins) as bf:
        for c in cats[:ncat]:
            t0 = time.perf_counter()
            theory.run_DD(ref, 0, nthreads, bins, c[0], c[1], c[2], X2=rand[0], Y2=rand[1], Z2=rand[2],
                          weights1=c[3], weights2=rand[3], weight_type="pair_product", periodic=True,
                          boxsize=WORKLOAD["boxsize"], isa="fastest")
            dt += time.perf_counter() - t0
            work += reference_work(C, c, rand, bf, np.float32)
    return dt, work, ncat


def run_reference_arm(args):
    rank, world, _ = _rank_env()
    if rank != 0:
        return
    if WORKLOAD.get("kind") == "survey":
        return run_survey_reference(args)
    if WORKLOAD.get("kind") == "batched":
        cats, rand, bins = make_batch_workload()
        times, works = [], []
        for _ in range(args.steps):
            r = cpu_batch_reference(cats, rand, bins, os.cpu_count() or 1, ncat=8)
            if r is None:
                print(json.dumps({"impl": "reference",
                                  "unavailable": "reference pair counters were not built in oracle/_ref"}))
                return
            times.append(r[0])
            works.append(r[1])
        value = sum(works) / sum(times)
        sample = "the first 8 of the 64 catalogues against the full random catalogue"
        print(json.dumps({"metric": "pair evaluations/sec (reference-lattice candidate pairs), batched DD "
                                    "cross-correlations", "value": value, "unit": UNIT, "n_gpus": args.gpus,
                          "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * sum(times) / len(times),
                          "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
                          "data": "synthetic (seeded clustered and uniform catalogues)",
                          "config": dict(WORKLOAD, sample=sample), "impl": "reference",
                          "cpu_baseline": {"value": value, "unit": UNIT, "cores": os.cpu_count(), "kind": "reference",
                                           "sample": sample},
                          "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}))
        return
    set1, set2, bins = make_workload()
    nthreads = os.cpu_count() or 1
    # size the sample so that one step stays within ~20 s of CPU time
    frac = 1.0
    probe = cpu_reference_run(set1, set2, bins, nthreads, np.float64, frac=0.1)
    if probe is None:
        print(json.dumps({"impl": "reference", "unavailable": "reference pair counters were not built in oracle/_ref"}))
        return
    est_full = probe[0] * 100.0
    if est_full > 20.0:
        frac = max(0.05, (20.0 / est_full) ** 0.5)
    times, works = [], []
    for _ in range(args.warmup if args.warmup < 1 else 1):
        cpu_reference_run(set1, set2, bins, nthreads, np.float64, frac=frac)
    for _ in range(args.steps):
        dt, work, n1, n2 = cpu_reference_run(set1, set2, bins, nthreads, np.float64, frac=frac)
        times.append(dt)
        works.append(work)
    value = sum(works) / sum(times)
    sample = "first %d and %d points of the two catalogues (fraction %.3f of each)" % (n1, n2, frac)
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * sum(times) / len(times), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded clustered catalogues)",
            "config": dict(WORKLOAD, sample=sample), "impl": "reference",
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": nthreads, "kind": "reference",
                             "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


SURVEY_METRIC = "catalogue pairs/sec (N(N-1)/2 per call), DDrppi_mocks auto-correlation"
# FP32 operations of one survey pair in the classification (s, l, s.s, l.l, s.l, rsqrt, pi, s x l,
# |s x l|^2 / |l|^2; an FMA counts two)
SURVEY_FLOP_PER_PAIR = 48


def run_survey_workload(args):
    """DDrppi_mocks (countpairs_mocks) on the survey workload: device time of the count (upload,
    lattice, work list, pair kernel; the RA/DEC/cz -> XYZ conversion is host work, as in the
    reference) and the API call's wall time as e2e; DDsmu_mocks and vpf timed beside it."""
    rank, world, local = _rank_env()
    if rank != 0:
        return
    import torch
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    import corrfunc_gb300 as cf
    from corrfunc_gb300 import catalogs as cat
    from corrfunc_gb300 import mocks, theory
    cf.set_precision(args.precision)
    W = WORKLOAD
    ra, dec, cz = cat.survey(W["n1"], W["seeds"][0], ra=(110.0, 266.0), dec=(-4.0, 70.0), cz=(6000.0, 20000.0))
    w = cat.weights(W["n1"], W["seeds"][1])
    bins = cat.log_bins(W["rmin"], W["rmax"], W["nbins"])

    def call():
        t0 = time.perf_counter()
        r = mocks.DDrppi_mocks(1, 1, 1, W["pimax"], bins, ra.copy(), dec.copy(), cz.copy(), weights1=w,
                               weight_type="pair_product", isa="fallback")
        return r, time.perf_counter() - t0, cf.last_stats()

    ClockSampler.shared(local)  # clock samples from the warm-up on
    for _ in range(max(args.warmup, 3)):
        ref, _, _ = call()
        flush_l2(torch, dev)
    npair = W["n1"] * (W["n1"] - 1) / 2.0
    gpu_ms, pair_ms, walls, launches = [], [], [], 0
    with clock_window(local) as clocks:
        for _ in range(args.steps):
            r, wall, st = call()
            if not np.array_equal(r["npairs"], ref["npairs"]):
                raise RuntimeError("non-deterministic pair counts between steps")
            gpu_ms.append(st["total_gpu_ms"])
            pair_ms.append(st["pair_kernel_ms"])
            walls.append(wall)
            launches += st["kernel_launches"]
            flush_l2(torch, dev)
    peak = ctypes.c_double()
    lib = cf.library()
    lib.cf_gpu_fp32_peak_tflops.argtypes = [ctypes.POINTER(ctypes.c_double)]
    lib.cf_gpu_fp32_peak_tflops(ctypes.byref(peak))
    pair_s = sum(pair_ms) / 1e3 / args.steps
    achieved = st["pairs_evaluated"] * SURVEY_FLOP_PER_PAIR / pair_s / 1e12
    line = {"metric": SURVEY_METRIC, "value": npair * args.steps / (sum(gpu_ms) / 1e3), "unit": "pairs/s",
            "n_gpus": 1, "steps": args.steps, "warmup": max(args.warmup, 3), "ms_per_step": sum(gpu_ms) / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32+f64-refine" if args.precision == "fp32_refine" else "f64",
            "data": "synthetic (seeded survey catalogue, numpy PCG64)",
            "config": dict(W, precision=args.precision, l2="flushed between steps (256 MB write)"),
            "roofline": {"bound": "fp32", "achieved": achieved, "peak": peak.value, "unit": "TFLOP/s",
                         "frac": achieved / peak.value if peak.value else None, "traffic": None,
                         "kernel": "k_pairs_f32<MODE_RPPI_MOCK,false,true>",
                         "peak_source": "measured: FP32 FMA calibration kernel (cf_gpu_fp32_peak_tflops) in this run",
                         "flop_per_pair": SURVEY_FLOP_PER_PAIR, "pairs_evaluated": st["pairs_evaluated"]},
            "e2e": {"value": npair * args.steps / sum(walls), "unit": "pairs/s",
                    "h2d_bytes_per_step": 4 * 8 * W["n1"], "d2h_bytes_per_step": 15 * 41 * 32,
                    "ms_per_step": 1e3 * sum(walls) / args.steps},
            "gpu_launches": launches,
            "kernel_ms": {"pair_kernel": sum(pair_ms) / args.steps, "step_total": sum(gpu_ms) / args.steps},
            "pairs": {"gpu_evaluated": st["pairs_evaluated"], "fp32_slow_path": st["pairs_slow"],
                      "fp64_refined": st["pairs_refined"], "counted": int(np.sum(ref["npairs"]))},
            "clocks": clocks.summary()}
    beside = {}
    for name, fn in [("DDsmu_mocks_ms", lambda: mocks.DDsmu_mocks(1, 1, 1, 1.0, 10, bins, ra.copy(), dec.copy(),
                                                                  cz.copy(), isa="fallback")),
                     ("DDrppi_mocks_rpavg_ms", lambda: mocks.DDrppi_mocks(1, 1, 1, W["pimax"], bins, ra.copy(),
                                                                          dec.copy(), cz.copy(), output_rpavg=True,
                                                                          isa="fallback"))]:
        fn()
        t = []
        for _ in range(3):
            fn()
            t.append(cf.last_stats()["total_gpu_ms"])
        beside[name] = min(t)
    x4, y4, z4 = cat.clustered_box(1_000_000, 420.0, 3)
    theory.vpf(10.0, 10, 100000, 6, -1234, x4, y4, z4, periodic=True, boxsize=420.0)
    beside["vpf_1M_points_1e5_spheres_ms"] = cf.last_stats()["total_gpu_ms"]
    line["beside"] = beside
    if not args.no_cpu_baseline:
        r = survey_reference_run(ra, dec, cz, w, bins)
        if r is not None:
            dt, npairs_ref = r
            if not np.array_equal(np.asarray(npairs_ref), np.asarray(ref["npairs"])):
                raise RuntimeError("the GPU survey counts differ from the reference's countpairs_mocks()")
            line["cpu_baseline"] = {"value": npair / dt, "unit": "pairs/s", "cores": os.cpu_count(), "kind": "reference",
                                    "sample": "the whole survey, one run (reference built against the test-only GSL "
                                              "stand-in)", "seconds": dt}
            line["parity"] = {"checked": True, "npairs_equal": True,
                              "against": "the reference's countpairs_mocks() (oracle/_ref) on the same survey"}
    print(json.dumps(line))


def survey_reference_run(ra, dec, cz, w, bins):
    """The reference's own DDrppi_mocks (oracle/_ref, compiled against the test-only GSL stand-in),
    all host threads, whole survey: (seconds, npairs), or None if not built."""
    from corrfunc_gb300 import _capi as C
    from corrfunc_gb300 import mocks
    so = os.path.join(ROOT, "oracle", "_ref", "libcf_ref_DDrppi_mocks.so")
    if not os.path.exists(so):
        return None
    lib = C.bind(so)
    t0 = time.perf_counter()
    r = mocks.run_DDrppi_mocks(lib, 1, 1, os.cpu_count() or 1, WORKLOAD["pimax"], bins, ra.copy(), dec.copy(),
                               cz.copy(), weights1=w, weight_type="pair_product", isa="fallback")
    return time.perf_counter() - t0, r["npairs"]


def run_survey_reference(args):
    from corrfunc_gb300 import catalogs as cat
    W = WORKLOAD
    ra, dec, cz = cat.survey(W["n1"], W["seeds"][0], ra=(110.0, 266.0), dec=(-4.0, 70.0), cz=(6000.0, 20000.0))
    w = cat.weights(W["n1"], W["seeds"][1])
    bins = cat.log_bins(W["rmin"], W["rmax"], W["nbins"])
    times = []
    for _ in range(args.steps):
        r = survey_reference_run(ra, dec, cz, w, bins)
        if r is None:
            print(json.dumps({"impl": "reference", "unavailable": "reference survey counter not built in oracle/_ref"}))
            return
        times.append(r[0])
    npair = W["n1"] * (W["n1"] - 1) / 2.0
    value = npair * len(times) / sum(times)
    sample = "the whole survey (reference DDrppi_mocks built against the test-only GSL stand-in)"
    print(json.dumps({"metric": SURVEY_METRIC, "value": value, "unit": "pairs/s", "n_gpus": args.gpus,
                      "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * sum(times) / len(times),
                      "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                      "data": "synthetic (seeded survey catalogue)", "config": dict(W, sample=sample),
                      "impl": "reference",
                      "cpu_baseline": {"value": value, "unit": "pairs/s", "cores": os.cpu_count(), "kind": "reference",
                                       "sample": sample},
                      "e2e": {"value": value, "unit": "pairs/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="fp32_refine", choices=["fp32_refine", "fp64"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--extras", action="store_true", help="also time the other counters (DDrppi, wp, DDsmu, "
                                                          "DDtheta, survey counters, vpf)")
    ap.add_argument("--workload", default="cfg2", choices=sorted(WORKLOADS))
    ap.add_argument("--no-batch", action="store_true", help="leave the batched-workload record out of the line")
    args = ap.parse_args()
    WORKLOAD.clear()
    WORKLOAD.update(WORKLOADS[args.workload])
    if args.impl == "reference":
        return run_reference_arm(args)
    if args.workload == "cfg5":
        return run_batch_workload(args)
    if args.workload == "survey":
        return run_survey_workload(args)

    rank, world, local = _rank_env()
    import torch
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")

    import corrfunc_gb300
    from corrfunc_gb300 import _capi as C
    lib = corrfunc_gb300.library()
    lib.cf_gpu_countpairs_device.argtypes = lib.countpairs.argtypes
    lib.cf_gpu_countpairs_device.restype = ctypes.c_int
    lib.cf_gpu_fp32_peak_tflops.argtypes = [ctypes.POINTER(ctypes.c_double)]
    corrfunc_gb300.set_precision(args.precision)

    set1, set2, bins = make_workload()
    binf = C.BinFile(bins)
    binfile = binf.__enter__()
    work = reference_work(C, set1, set2, binfile, np.float64)
    o = options_for(C, WORKLOAD["boxsize"], np.float64)
    counter = DeviceCounter(lib, C, corrfunc_gb300, binfile, o, WORKLOAD["autocorr"])

    # inputs resident in HBM
    d1 = [torch.from_numpy(a).to(dev) for a in set1]
    d2 = [torch.from_numpy(a).to(dev) for a in set2]
    torch.cuda.synchronize(dev)

    def step_device():
        return counter.device(d1, d2)

    # host arrays in pinned memory for the end-to-end leg
    h1 = [torch.from_numpy(a).pin_memory() for a in set1]
    h2 = [torch.from_numpy(a).pin_memory() for a in set2]
    hn1 = [t.numpy() for t in h1]
    hn2 = [t.numpy() for t in h2]

    ClockSampler.shared(local)  # clock samples from the warm-up on
    for _ in range(max(args.warmup, 3)):
        ref_np, ref_wavg, _ = step_device()
        flush_l2(torch, dev)

    gpu_ms, pair_ms, grid_ms, launches, evaluated, refined, wall = [], [], [], 0, 0, 0, []
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize(dev)
    with clock_window(local) as clocks:
        for _ in range(args.steps):
            t0 = time.perf_counter()
            npairs, _wavg, st = step_device()
            wall.append(time.perf_counter() - t0)
            if not np.array_equal(npairs, ref_np):
                raise RuntimeError("non-deterministic pair counts between steps")
            gpu_ms.append(st["total_gpu_ms"])
            pair_ms.append(st["pair_kernel_ms"])
            grid_ms.append(st["gridlink_ms"])
            launches += st["kernel_launches"]
            evaluated += st["pairs_evaluated"]
            refined += st["pairs_refined"]
            flush_l2(torch, dev)
    torch.cuda.synchronize(dev)
    total_s = max_over_ranks(sum(gpu_ms) / 1e3, world, dev)
    value = replica_throughput(work, args.steps, total_s, world)

    # end to end through the public C API with host buffers: pinned (page-locked) and pageable
    # (plain numpy arrays, as a Python caller passes them)
    e2e_value, e2e_ms = end_to_end(counter, hn1, hn2, ref_np, work, world, args.steps, torch, dev)
    e2e_pg_value, e2e_pg_ms = end_to_end(counter, list(set1), list(set2), ref_np, work, world, args.steps, torch, dev)
    nper = 4 if WORKLOAD["weights"] else 3
    h2d = sum(a.nbytes for a in hn1[:nper]) + (0 if WORKLOAD["autocorr"] else sum(a.nbytes for a in hn2[:nper]))
    d2h = (WORKLOAD["nbins"] + 1) * (8 + 8 + 8 + 8)

    peak = ctypes.c_double()
    lib.cf_gpu_fp32_peak_tflops(ctypes.byref(peak))
    pair_s = sum(pair_ms) / 1e3 / args.steps
    achieved = work * FLOP_PER_PAIR / pair_s / 1e12
    achieved_eval = (evaluated / args.steps) * FLOP_PER_PAIR / pair_s / 1e12
    traffic = (PAIR_KERNEL_TRAFFIC_BYTES.get((args.workload, st["column_split"]))
               if args.precision == "fp32_refine" else None)

    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": max(args.warmup, 3), "ms_per_step": sum(gpu_ms) / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64-refine" if args.precision == "fp32_refine" else "f64",
            "data": "synthetic (seeded clustered catalogues, numpy PCG64)",
            "config": dict(WORKLOAD, precision=args.precision, l2="flushed between steps (256 MB write)",
                           reference_lattice_candidates=work),
            "roofline": {"bound": "fp32", "achieved": achieved, "peak": peak.value, "unit": "TFLOP/s",
                         "frac": achieved / peak.value if peak.value else None, "traffic": traffic,
                         "traffic_source": TRAFFIC_SOURCE if traffic else None,
                         "kernel": "%s<MODE_R3,false,%s>" % ("k_pairs_f32" if args.precision == "fp32_refine"
                                                             else "k_pairs_f64",
                                                             "true" if WORKLOAD["weights"] else "false"),
                         "peak_source": "measured: FP32 FMA calibration kernel (cf_gpu_fp32_peak_tflops) in this run",
                         "flop_per_pair": FLOP_PER_PAIR,
                         "work_unit": "reference-lattice candidate pairs",
                         "achieved_gpu_evaluated": achieved_eval,
                         "frac_gpu_evaluated": achieved_eval / peak.value if peak.value else None},
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                    "ms_per_step": e2e_ms, "host_memory": "pinned"},
            "e2e_pageable": {"value": e2e_pg_value, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                             "ms_per_step": e2e_pg_ms, "host_memory": "pageable (numpy arrays)"},
            "gpu_launches": launches,
            "launch": {"blocks_per_sm": st["blocks_per_sm"], "warps_per_block": st["warps_per_block"],
                       "lane_stride": st["lane_stride"], "column_split": st["column_split"]},
            "kernel_ms": {"pair_kernel": sum(pair_ms) / args.steps, "gridlink": sum(grid_ms) / args.steps,
                          "extent_worklist_and_gaps": (sum(gpu_ms) - sum(pair_ms) - sum(grid_ms)) / args.steps,
                          "step_total": sum(gpu_ms) / args.steps, "host_wall": 1e3 * sum(wall) / args.steps},
            "gridlink_roofline": gridlink_roofline(sum(grid_ms) / args.steps, st["num_cells"]),
            "in_range_pairs_per_s": (int(np.sum(ref_np)) // (2 if WORKLOAD["autocorr"] else 1))
                                    / (sum(gpu_ms) / 1e3 / args.steps),
            "pairs": {"reference_lattice_candidates": work, "gpu_evaluated": evaluated // args.steps,
                      "fp32_slow_path": st["pairs_slow"], "fp64_refined": refined // args.steps,
                      "counted": int(np.sum(ref_np))},
            "clocks": clocks.summary()}

    if rank == 0:
        # the same workload with the pair kernel that evaluates every pair in FP64
        line["fp64_form"] = fp64_form(counter, corrfunc_gb300, lambda: step_device(), ref_np, args.precision,
                                      sum(pair_ms) / args.steps, sum(gpu_ms) / args.steps, torch, dev)
        # the same draw as float32 positions and weights
        f1 = [a.astype(np.float32) for a in set1]
        f2 = [a.astype(np.float32) for a in set2]
        line["float32"] = float32_variant(counter, f1, f2, work, args, torch, dev, local)
        # 1M-point periodic DD auto-correlation (20 log bins to 25, L = 420)
        line["northstar"] = northstar_record(lib, C, corrfunc_gb300, args, torch, dev, local, peak.value)
        # 64 catalogues against one 5M-point catalogue in one replayed CUDA graph
        if not args.no_batch:
            rec = batch_record(args, torch, dev, local)
            rec.pop("_data", None)
            line["cfg5"] = rec

    if args.extras and rank == 0:
        line["extras"] = extras(corrfunc_gb300, args)
        corrfunc_gb300.set_precision(args.precision)

    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        # the reference's own countpairs() on the whole workload (all host threads): the CPU
        # baseline and the parity check of this run's counts, float64 and float32 (the reference's
        # double run on the float32 values upcast)
        r = reference_full_run(set1, set2, bins)
        if r is None:
            line["cpu_baseline"] = None
            line["parity"] = {"checked": False, "why": "reference pair counters not built in oracle/_ref"}
        else:
            dt, ref_np_cpu, ref_wavg_cpu = r
            line["cpu_baseline"] = {"value": work / dt, "unit": UNIT, "cores": os.cpu_count(), "kind": "reference",
                                    "sample": "the whole workload, one run", "seconds": dt}
            line["parity"] = parity_record(ref_np, ref_wavg, ref_np_cpu, ref_wavg_cpu)
            r32 = reference_full_run([a.astype(np.float64) for a in f1], [a.astype(np.float64) for a in f2], bins)
            f32 = line["float32"]
            line["float32"]["parity"] = parity_record(f32.pop("_npairs"), f32.pop("_weightavg"), r32[1], r32[2],
                                                      rtol=1e-4)
            line["float32"]["parity"]["against"] = "the reference's double-precision run on the float32 values upcast"
    for k in ("_npairs", "_weightavg"):
        line.get("float32", {}).pop(k, None)
    binf.__exit__(None, None, None)
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()


class DeviceCounter:
    """countpairs() (DD(r)) on device-resident arrays (cf_gpu_countpairs_device) or on host
    arrays (the public countpairs(), host-to-device copies inside the call)."""

    def __init__(self, lib, C, cf, binfile, options, autocorr):
        self.lib, self.C, self.cf = lib, C, cf
        self.binfile, self.o, self.autocorr = binfile, options, autocorr

    def _extra(self, w1, w2):
        C = self.C
        if WORKLOAD["weights"] is None:
            return C.get_extra_options()
        e = C.get_extra_options(C.WEIGHT_PAIR_PRODUCT)
        e.weights0.weights[0] = w1
        e.weights1.weights[0] = w2
        e.weights0.num_weights = e.weights1.num_weights = 1
        return e

    def _finish(self, rc, res, what):
        if rc != 0:
            raise RuntimeError("%s failed" % what)
        npairs = np.ctypeslib.as_array(res.npairs, shape=(res.nbin,)).copy()
        wavg = np.ctypeslib.as_array(res.weightavg, shape=(res.nbin,)).copy()
        self.lib.free_results(ctypes.byref(res))
        return npairs, wavg, self.cf.last_stats()

    def device(self, d1, d2, options=None):
        C = self.C
        o = self.o if options is None else options
        e = self._extra(d1[3].data_ptr() if len(d1) > 3 else None, d2[3].data_ptr() if len(d2) > 3 else None)
        res = C.ResultsDD()
        rc = self.lib.cf_gpu_countpairs_device(len(d1[0]), *(ctypes.c_void_p(t.data_ptr()) for t in d1[:3]),
                                               len(d2[0]), *(ctypes.c_void_p(t.data_ptr()) for t in d2[:3]), 1,
                                               self.autocorr, self.binfile.encode(), ctypes.byref(res),
                                               ctypes.byref(o), ctypes.byref(e))
        return self._finish(rc, res, "countpairs on device inputs")

    def host(self, h1, h2, options=None):
        C = self.C
        o = self.o if options is None else options
        e = self._extra(h1[3].ctypes.data if len(h1) > 3 else None, h2[3].ctypes.data if len(h2) > 3 else None)
        res = C.ResultsDD()
        rc = self.lib.countpairs(len(h1[0]), *(C.ptr(a) for a in h1[:3]), len(h2[0]), *(C.ptr(a) for a in h2[:3]),
                                 1, self.autocorr, self.binfile.encode(), ctypes.byref(res), ctypes.byref(o),
                                 ctypes.byref(e))
        return self._finish(rc, res, "countpairs")


def end_to_end(counter, h1, h2, ref_np, work, world, steps, torch, dev, options=None):
    """Throughput of the public countpairs() on host arrays (uploads and read-back inside)."""
    for _ in range(2):
        counter.host(h1, h2, options)
    ts = []
    for _ in range(steps):
        flush_l2(torch, dev)
        t0 = time.perf_counter()
        npairs_h, _w, _st = counter.host(h1, h2, options)
        ts.append(time.perf_counter() - t0)
        if not np.array_equal(npairs_h, ref_np):
            raise RuntimeError("host-buffer path disagrees with the device-buffer path")
    return world * work * steps / sum(ts), 1e3 * sum(ts) / steps


def fp64_form(counter, cf, step, ref_np, precision, pair_ms_fp32, step_ms_fp32, torch, dev):
    """The same count with the pair kernel that evaluates every pair with the reference's FP64
    formula: timing and identical counts."""
    cf.set_precision("fp64")
    try:
        step()
        flush_l2(torch, dev)
        pm, sm = [], []
        for _ in range(2):
            npairs, _w, st = step()
            if not np.array_equal(npairs, ref_np):
                raise RuntimeError("FP64 form counts differ from the FP32+refine form")
            pm.append(st["pair_kernel_ms"])
            sm.append(st["total_gpu_ms"])
            flush_l2(torch, dev)
    finally:
        cf.set_precision(precision)
    return {"kernel": "k_pairs_f64", "pair_kernel_ms": min(pm), "step_ms": min(sm), "npairs_equal": True,
            "fp32_refine_pair_kernel_ms": pair_ms_fp32, "fp32_refine_step_ms": step_ms_fp32,
            "speedup_pair_kernel": min(pm) / pair_ms_fp32, "speedup_step": min(sm) / step_ms_fp32}


def float32_variant(counter, f1, f2, work, args, torch, dev, local):
    """The workload as float32 positions and weights (device-resident), timed like the main line."""
    from corrfunc_gb300 import _capi as C
    o = options_for(C, WORKLOAD["boxsize"], np.float32)
    d1 = [torch.from_numpy(a).to(dev) for a in f1]
    d2 = [torch.from_numpy(a).to(dev) for a in f2]
    torch.cuda.synchronize(dev)
    for _ in range(max(args.warmup, 3)):
        ref, wavg, _ = counter.device(d1, d2, o)
        flush_l2(torch, dev)
    gpu_ms, pair_ms = [], []
    with clock_window(local) as clocks:
        for _ in range(args.steps):
            npairs, _w, st = counter.device(d1, d2, o)
            if not np.array_equal(npairs, ref):
                raise RuntimeError("non-deterministic float32 counts")
            gpu_ms.append(st["total_gpu_ms"])
            pair_ms.append(st["pair_kernel_ms"])
            flush_l2(torch, dev)
    return {"value": work * args.steps / (sum(gpu_ms) / 1e3), "unit": UNIT, "ms_per_step": sum(gpu_ms) / args.steps,
            "pair_kernel_ms": sum(pair_ms) / args.steps, "h2d_bytes_per_step": 0, "counted": int(np.sum(ref)),
            "clocks": clocks.summary(), "_npairs": ref, "_weightavg": wavg}


def split_form(counter, step, ref, work, peak, steps, torch, dev, split="4,2"):
    """The same count with the j lattice's columns split (CF_COLUMN_SPLIT, read on every call):
    its pair kernel and device step beside the unsplit form the cost model chose."""
    old = os.environ.get("CF_COLUMN_SPLIT")
    os.environ["CF_COLUMN_SPLIT"] = split
    try:
        for _ in range(3):
            npairs, _w, st = step()
            flush_l2(torch, dev)
        pm, sm = [], []
        for _ in range(steps):
            npairs, _w, st = step()
            if not np.array_equal(npairs, ref):
                raise RuntimeError("split columns changed the counts")
            pm.append(st["pair_kernel_ms"])
            sm.append(st["total_gpu_ms"])
            flush_l2(torch, dev)
    finally:
        if old is None:
            os.environ.pop("CF_COLUMN_SPLIT", None)
        else:
            os.environ["CF_COLUMN_SPLIT"] = old
    pair_s = sum(pm) / 1e3 / steps
    ach = work * FLOP_PER_PAIR / pair_s / 1e12
    return {"column_split": st["column_split"], "slab_merge": int(split.split(",")[1]),
            "pair_kernel_ms": sum(pm) / steps, "step_ms": sum(sm) / steps, "npairs_equal": True,
            "gpu_evaluated": st["pairs_evaluated"], "roofline_frac": ach / peak if peak else None}


def northstar_record(lib, C, cf, args, torch, dev, local, peak):
    """1,000,000 uniform points, periodic L = 420, DD auto-correlation, 20 log bins 0.1-25:
    device throughput, its FP32 roofline fraction, end to end, and the FP64 form."""
    from corrfunc_gb300 import catalogs as cat
    W = WORKLOADS["northstar"]
    L = W["boxsize"]
    x, y, z = cat.uniform_box(W["n1"], L, W["seeds"][0])
    s = (x, y, z)
    bins = cat.log_bins(W["rmin"], W["rmax"], W["nbins"])
    saved = dict(WORKLOAD)
    WORKLOAD.clear()
    WORKLOAD.update(W)
    try:
        with C.BinFile(bins) as bf:
            work = reference_work(C, s, s, bf, np.float64)
            o = options_for(C, L, np.float64)
            counter = DeviceCounter(lib, C, cf, bf, o, 1)
            d = [torch.from_numpy(a).to(dev) for a in s]
            torch.cuda.synchronize(dev)
            for _ in range(max(args.warmup, 3)):
                ref, _w, _ = counter.device(d, d)
                flush_l2(torch, dev)
            gpu_ms, pair_ms, evaluated = [], [], 0
            with clock_window(local) as clocks:
                for _ in range(args.steps):
                    npairs, _w, st = counter.device(d, d)
                    if not np.array_equal(npairs, ref):
                        raise RuntimeError("non-deterministic north-star counts")
                    gpu_ms.append(st["total_gpu_ms"])
                    pair_ms.append(st["pair_kernel_ms"])
                    evaluated += st["pairs_evaluated"]
                    flush_l2(torch, dev)
            pair_s = sum(pair_ms) / 1e3 / args.steps
            ach = work * FLOP_PER_PAIR / pair_s / 1e12
            ach_eval = evaluated / args.steps * FLOP_PER_PAIR / pair_s / 1e12
            split = split_form(counter, lambda: counter.device(d, d), ref, work, peak, args.steps, torch, dev)
            hs = [torch.from_numpy(a).pin_memory().numpy() for a in s]
            e2e_v, e2e_ms = end_to_end(counter, hs, hs, ref, work, 1, args.steps, torch, dev)
            f64 = fp64_form(counter, cf, lambda: counter.device(d, d), ref, args.precision,
                            sum(pair_ms) / args.steps, sum(gpu_ms) / args.steps, torch, dev)
    finally:
        WORKLOAD.clear()
        WORKLOAD.update(saved)
    return {"workload": W["workload"], "value": work * args.steps / (sum(gpu_ms) / 1e3), "unit": UNIT,
            "ms_per_step": sum(gpu_ms) / args.steps, "pair_kernel_ms": sum(pair_ms) / args.steps,
            "column_split": st["column_split"],
            "roofline": {"bound": "fp32", "achieved": ach, "peak": peak, "unit": "TFLOP/s",
                         "frac": ach / peak if peak else None, "kernel": "k_pairs_f32<MODE_R3,false,false>",
                         "traffic": PAIR_KERNEL_TRAFFIC_BYTES.get(("northstar", st["column_split"])),
                         "traffic_source": TRAFFIC_SOURCE,
                         "achieved_gpu_evaluated": ach_eval, "frac_gpu_evaluated": ach_eval / peak if peak else None,
                         "target_frac": 0.40},
            "e2e": {"value": e2e_v, "unit": UNIT, "h2d_bytes_per_step": 3 * 8 * W["n1"],
                    "d2h_bytes_per_step": (W["nbins"] + 1) * 32, "ms_per_step": e2e_ms, "host_memory": "pinned"},
            "fp64_form": f64,
            "split_form": split,
            "pairs": {"reference_lattice_candidates": work, "gpu_evaluated": evaluated // args.steps,
                      "counted": int(np.sum(ref))},
            "clocks": clocks.summary()}


def reference_full_run(set1, set2, bins):
    """The reference's countpairs() (oracle/_ref, FALLBACK kernels where only those exist, all
    host threads) on the whole workload: (seconds, npairs, weightavg), or None if not built."""
    from corrfunc_gb300 import _capi as C
    from corrfunc_gb300 import theory
    so = os.path.join(ROOT, "oracle", "_ref", "libcf_ref_DD.so")
    if not os.path.exists(so):
        return None
    ref = C.bind(so)
    wkw = dict(weights1=set1[3], weights2=set2[3], weight_type="pair_product") if WORKLOAD["weights"] else {}
    t0 = time.perf_counter()
    if WORKLOAD["autocorr"]:
        wkw.pop("weights2", None)
        r = theory.run_DD(ref, 1, os.cpu_count() or 1, bins, set1[0], set1[1], set1[2], periodic=True,
                          boxsize=WORKLOAD["boxsize"], isa="fastest", **wkw)
    else:
        r = theory.run_DD(ref, 0, os.cpu_count() or 1, bins, set1[0], set1[1], set1[2], X2=set2[0], Y2=set2[1],
                          Z2=set2[2], periodic=True, boxsize=WORKLOAD["boxsize"], isa="fastest", **wkw)
    dt = time.perf_counter() - t0
    return dt, np.asarray(r["npairs"], np.uint64), np.asarray(r["weightavg"], float)


def parity_record(gpu_np, gpu_wavg, ref_np, ref_wavg, rtol=1e-6):
    """npairs (the C arrays carry the unused bin 0 first) bit-exact, weightavg within rtol."""
    g = np.asarray(gpu_np, np.uint64)[1:]
    gw = np.asarray(gpu_wavg, float)[1:]
    eq = bool(np.array_equal(g, np.asarray(ref_np, np.uint64)))
    m = np.asarray(ref_np) > 0
    rel = float(np.max(np.abs(gw[m] - ref_wavg[m]) / np.abs(ref_wavg[m]))) if m.any() else 0.0
    if not eq or rel > rtol:
        raise RuntimeError("the GPU counts differ from the reference's countpairs() on this workload "
                           "(npairs equal: %s, max rel weightavg %.3g)" % (eq, rel))
    return {"checked": True, "against": "the reference's countpairs() (oracle/_ref) on the same inputs",
            "npairs_equal": eq, "max_rel_weightavg": rel, "rtol": rtol, "bins_compared": int(len(g))}


def extras(cf, args):
    """The other pair counters, timed on the survey's configurations 3 and 4."""
    from corrfunc_gb300 import catalogs as cat
    from corrfunc_gb300 import theory
    out = other_counters(cf, cat, theory)
    cf.set_precision(args.precision)
    return out


def reference_cpu_beside(x, y, z, rp, sb, ra, dec, tb, L):
    """The reference's own DDrppi / wp / DDsmu (oracle/_ref, all host threads, FALLBACK kernels on
    aarch64) on the full configuration-3 workload, and its DDtheta on the first 200,000 points of the
    configuration-4 cap (with the full-size estimate scaled by the number of point pairs)."""
    from corrfunc_gb300 import _capi as C
    from corrfunc_gb300 import mocks, theory
    out = {}
    nt = os.cpu_count() or 1
    libs = {m: os.path.join(ROOT, "oracle", "_ref", "libcf_ref_%s.so" % m) for m in ("DDrppi", "wp", "DDsmu", "DDtheta")}
    if not all(os.path.exists(v) for v in libs.values()):
        return {"reference_cpu": "reference libraries not built in oracle/_ref"}
    runs = {"cfg3_DDrppi": lambda lib: theory.run_DDrppi(lib, 1, nt, 40.0, rp, x, y, z, boxsize=L, isa="fastest"),
            "cfg3_wp": lambda lib: theory.run_wp(lib, L, 40.0, nt, rp, x, y, z, isa="fastest"),
            "cfg3_DDsmu": lambda lib: theory.run_DDsmu(lib, 1, nt, sb, 1.0, 10, x, y, z, boxsize=L, isa="fastest")}
    mod = {"cfg3_DDrppi": "DDrppi", "cfg3_wp": "wp", "cfg3_DDsmu": "DDsmu"}
    for name, fn in runs.items():
        lib = C.bind(libs[mod[name]])
        t0 = time.perf_counter()
        fn(lib)
        out["%s_reference_cpu_s" % name] = {"seconds": time.perf_counter() - t0, "cores": nt, "sample": "full workload"}
    n = 200_000
    lib = C.bind(libs["DDtheta"])
    t0 = time.perf_counter()
    mocks.run_DDtheta_mocks(lib, 1, nt, tb, ra[:n].copy(), dec[:n].copy(), output_thetaavg=True, isa="fastest")
    dt = time.perf_counter() - t0
    out["cfg4_DDtheta_reference_cpu_s"] = {"seconds": dt, "cores": nt, "sample": "first %d of %d points" % (n, len(ra)),
                                           "full_size_estimate_s": dt * (len(ra) / n) ** 2}
    return out


def other_counters(cf, cat, theory):
    """The other pair counters on the survey's configurations 3 and 4 (timing only; units are the
    GPU's own evaluated pairs and the pairs counted, since the reference-lattice work unit is
    defined for DD): DDrppi, wp and DDsmu on 1M clustered points in L=1000, DDtheta on 1M points
    of a sky cap."""
    from corrfunc_gb300 import mocks
    out = {}
    L = 1000.0
    x, y, z = cat.clustered_box(1_000_000, L, 3)
    rp = cat.log_bins(0.1, 25.0, 14)
    sb = cat.log_bins(0.1, 50.0, 20)
    ra, dec = cat.sky_cap(1_000_000, 4)
    tb = cat.log_bins(0.01, 10.0, 20)
    runs = {
        "cfg3_DDrppi": lambda: theory.DDrppi(1, 1, 40.0, rp, x, y, z, boxsize=L, isa="fallback"),
        "cfg3_wp": lambda: theory.wp(L, 40.0, 1, rp, x, y, z, isa="fallback"),
        "cfg3_DDsmu": lambda: theory.DDsmu(1, 1, sb, 1.0, 10, x, y, z, boxsize=L, isa="fallback"),
        "cfg4_DDtheta": lambda: mocks.DDtheta_mocks(1, 1, tb, ra.copy(), dec.copy(), output_thetaavg=True,
                                                    isa="fallback"),
    }
    # survey catalogue of the reference's mocks tests' size and footprint (84,383 galaxies,
    # RA 110-266, DEC -4-70, cz 6,000-20,000 km/s), pimax 40 and 14 log rp bins 0.1-25
    x4, y4, z4 = cat.clustered_box(1_000_000, 420.0, 3)
    sra, sdec, scz = cat.survey(84383, 5, ra=(110.0, 266.0), dec=(-4.0, 70.0), cz=(6000.0, 20000.0))
    sw = cat.weights(84383, 6)
    runs["mocks_DDrppi_mocks"] = lambda: mocks.DDrppi_mocks(1, 1, 1, 40.0, rp, sra.copy(), sdec.copy(), scz.copy(),
                                                            weights1=sw, weight_type="pair_product",
                                                            output_rpavg=True, isa="fallback")
    runs["mocks_DDsmu_mocks"] = lambda: mocks.DDsmu_mocks(1, 1, 1, 1.0, 10, rp, sra.copy(), sdec.copy(), scz.copy(),
                                                          weights1=sw, weight_type="pair_product", output_savg=True,
                                                          isa="fallback")
    # counts in spheres: 1M clustered points in L=420, spheres up to radius 10, 10 radii, p0..p5
    runs["vpf_1M_nc1e4"] = lambda: theory.vpf(10.0, 10, 10000, 6, -1234, x4, y4, z4, periodic=True, boxsize=420.0)
    runs["vpf_1M_nc1e6"] = lambda: theory.vpf(10.0, 10, 1000000, 6, -1234, x4, y4, z4, periodic=True, boxsize=420.0)
    out.update(reference_cpu_beside(x, y, z, rp, sb, ra, dec, tb, L))
    for name, fn in runs.items():
        for prec in ("fp64", "fp32_refine"):
            cf.set_precision(prec)
            ms = []
            walls = []
            for _ in range(3 if prec == "fp32_refine" else 1):
                t0 = time.perf_counter()
                r = fn()
                walls.append(1e3 * (time.perf_counter() - t0))
                ms.append(cf.last_stats())
            best = min(ms, key=lambda s: s["pair_kernel_ms"])
            out["%s_%s" % (name, prec)] = {"pair_kernel_ms": best["pair_kernel_ms"],
                                          "total_gpu_ms": best["total_gpu_ms"],
                                          "host_wall_ms": min(walls),
                                          "gpu_evaluated_pairs": best["pairs_evaluated"],
                                          "fp32_slow_path": best["pairs_slow"],
                                          "fp64_refined": best["pairs_refined"],
                                          "npairs_sum": int(np.sum(r["npairs"])) if "npairs" in r.dtype.names
                                          else None}
    return out


if __name__ == "__main__":
    main()
