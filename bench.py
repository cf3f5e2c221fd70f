#!/usr/bin/env python3
"""Benchmark of the distance-GEMM hot path on GB300.

Default workload: exact k-NN, L2, nb = 1,000,000 base and nq = 10,000 query
vectors, d = 128, SIFT-like integer-valued float32 data, k = 100 (the k-NN
configuration of the reference's headline metric).  One step = one complete
exact k-NN of all queries (pack, threshold pass, fused BF16 tensor-core
distance + selection pass, exact re-rank / certificate, fallback).

Prints one JSON line (rank 0).  ``value`` is queries/s with the inputs already
resident in HBM; ``e2e`` is the same metric through the drop-in C-ABI call
``knn_full_thread`` with host (pinned) buffers, host<->device copies included.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
os.environ.setdefault("OPENBLAS_NUM_THREADS", "1")

import numpy as np  # noqa: E402

METRIC = "k-means iters/s & exact kNN qps: BF16+rerank vs plain FP32, 1 GB300, exact ids"


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["bf16_tflops"]), float(p["hbm_gbs"]), "measured"
    except Exception:
        return 1900.0, 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi samples (200 ms) during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
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
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def cpu_port_qps(b, q, k, budget_s=10.0, batch=250, max_q=5000):
    """The oracle's restatement of knn_full_thread (BLAS sgemm + yael heap)
    on the host cores, over a bounded sample of the queries."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from _util import knn_port, oracle
    nt = os.cpu_count() or 1
    done, t0 = 0, time.perf_counter()
    while done < min(max_q, q.shape[0]):
        qq = np.ascontiguousarray(q[done:done + batch])
        knn_port(b, qq, k, nt=nt)
        done += qq.shape[0]
        if time.perf_counter() - t0 >= budget_s:
            break
    dt = time.perf_counter() - t0
    return done / dt, nt, done, oracle().oracle_blas_name().decode()


def run_reference(args, world, rank):
    if rank != 0:
        return
    from yael_gb300 import synth
    b = synth.sift_like(args.nb, args.d, seed=1)
    q = synth.sift_like(args.nq, args.d, seed=2)
    vals = []
    nt = os.cpu_count() or 1
    per_step = max(1, args.ref_queries)
    for s in range(args.warmup + args.steps):
        qq = q[(s * per_step) % args.nq:][:per_step]
        t0 = time.perf_counter()
        qps, nt, done, blas = cpu_port_qps(b, qq, args.k, budget_s=1e9, batch=per_step,
                                           max_q=per_step)
        if s >= args.warmup:
            vals.append(qps)
    v = statistics.median(vals)
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "queries/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1000.0 * per_step / v, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": config_of(args),
            "cpu_baseline": {"value": v, "unit": "queries/s", "cores": nt, "kind": "port",
                             "sample": f"{per_step} queries per step vs the full {args.nb}-row "
                                       f"base (knn_full_thread restated, BLAS: {os.path.basename(blas)})"},
            "e2e": {"value": v, "unit": "queries/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# dram__bytes_read.sum + dram__bytes_write.sum of one main-pass launch at the
# default k-NN sizes (one ncu capture of tc_scan_kernel, THRESH mode)
KNN_MAIN_TRAFFIC = 325.835776e6 + 44.952832e6

CLUSTER_CFG = {
    # n, d, k, niter, seed, data
    "kmeans1": dict(n=100_000, d=128, k=256, niter=20, seed=0, comps=256, sigma=0.15, zipf=None),
    "kmeans3": dict(n=10_000_000, d=128, k=65536, niter=10, seed=1, comps=65536, sigma=0.2,
                    zipf=1.1),
    "hkm4": dict(n=2_000_000, d=96, bf=32, nlevel=3, niter=15, comps=4096, sigma=0.1),
}


def flush_l2(dev, nbytes=256 << 20):
    """Writes a buffer larger than the L2 (129 MB) so the next run starts cold."""
    import torch
    buf = getattr(flush_l2, "buf", None)
    if buf is None or buf.device != dev:
        buf = flush_l2.buf = torch.empty(nbytes // 4, dtype=torch.float32, device=dev)
    buf.fill_(1.0)


def cluster_data(name, c, dev):
    """The configuration's points: a seeded Gaussian mixture.  The large one is
    drawn on the device (5 GB; the host copy only of the CPU sample)."""
    import torch
    from yael_gb300 import synth
    w = synth.zipf_weights(c["comps"], c["zipf"]) if c.get("zipf") else None
    if c["n"] <= 2_000_000:
        v_h, _, _ = synth.gaussian_mixture(c["n"], c["d"], c["comps"], c["sigma"], seed=11,
                                           weights=w)
        return torch.from_numpy(v_h).to(dev), v_h
    g = torch.Generator(device=dev)
    g.manual_seed(11)
    centres = torch.randn((c["comps"], c["d"]), device=dev, generator=g)
    p = torch.ones(c["comps"], device=dev) if w is None else torch.from_numpy(w).to(dev)
    lab = torch.multinomial(p, c["n"], replacement=True, generator=g)
    v = torch.empty((c["n"], c["d"]), device=dev)
    step = 1 << 20
    for s0 in range(0, c["n"], step):
        e = min(c["n"], s0 + step)
        v[s0:e] = centres[lab[s0:e]] + c["sigma"] * torch.randn((e - s0, c["d"]), device=dev,
                                                                generator=g)
    return v, None


def kmeans_record(name, args, local):
    """One k-means configuration (kmeans1 / kmeans3) on GB300: Lloyd iterations
    per second of the chosen form (16-bit tensor-core pass + exact re-rank)
    with the points resident in HBM, the plain FP32 path beside it, the
    drop-in kmeans() end to end from host buffers, the oracle's FP64 check of
    the assignment of every iteration, and the reference algorithm (the
    oracle's port) on the host cores."""
    import torch
    import yael_gb300 as yg
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from _util import assign_mismatches, objective64, oracle, ptr
    dev = torch.device("cuda", local)
    L = yg.lib()
    c = dict(CLUSTER_CFG[name])
    if args.niter:
        c["niter"] = args.niter
    if args.n:
        c["n"] = args.n
    dv, v_h = cluster_data(name, c, dev)
    n, d = dv.shape
    k, niter, seed = c["k"], c["niter"], c["seed"]
    C = torch.empty((k, d), device=dev)
    dis = torch.empty(n, device=dev)
    assign = torch.empty(n, dtype=torch.int32, device=dev)
    flags = yg.KMEANS_QUIET | yg.KMEANS_INIT_RANDOM
    stream = torch.cuda.current_stream(dev)
    libc = ctypes.CDLL(None)
    libc.srand48.argtypes = [ctypes.c_long]
    nt = os.cpu_count() or 1

    def run(prec, it=niter, probe=None):
        # seed 0 draws the k-means seed from lrand48(): the same state for every run
        libc.srand48(0)
        o = yg.KmeansOpts(prec, 1, ctypes.c_void_p(stream.cuda_stream))
        if probe:
            for key, val in probe.items():
                setattr(o, key, val)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        q = L.yael_gpu_kmeans_ex(d, n, k, it, dv.data_ptr(), flags, seed, 1, C.data_ptr(),
                                 dis.data_ptr(), assign.data_ptr(), None, ctypes.byref(o))
        e1.record(stream)
        torch.cuda.synchronize(dev)
        if o.status != 0:
            raise RuntimeError(yg.last_error())
        return q, e0.elapsed_time(e1), o

    prec = yg.PREC_BF16 if args.prec == "bf16" else yg.PREC_FP32
    run(prec)  # warm-up: kernel attributes, the chunk tuner's trials
    runs = max(1, args.cluster_runs if n <= 200_000 else 1)
    ms_tot, iters, ms_assign = 0.0, 0, 0.0
    l0 = L.yael_gpu_launch_count()
    with ClockSampler(local) as clk:
        for _ in range(runs):
            flush_l2(dev)
            q, ms, o = run(prec)
            ms_tot += ms
            iters += o.iterations
            ms_assign += o.ms_assign
    launches = L.yael_gpu_launch_count() - l0
    prec_used = {0: "f32", 1: "bf16", 2: "bf16x3", 3: "f16"}.get(o.prec_used, "?")
    a_ch = assign.cpu().numpy().copy()
    rec = {"metric": METRIC, "value": 1e3 * iters / ms_tot, "unit": "iterations/s",
           "ms_per_step": ms_tot / iters, "steps": iters, "warmup": 1, "runs": runs,
           "higher_is_better": True, "dtype": prec_used,
           "config": {"workload": f"k-means n={n} d={d} k={k} niter={niter} seed={seed}, "
                                  f"Gaussian mixture ({c['comps']} comps, sigma={c['sigma']}"
                                  + (f", Zipf({c['zipf']}) weights" if c.get('zipf') else "")
                                  + "), random init", "n": n, "d": d, "k": k,
                      "l2": ("flushed between runs (256 MB written); the 51 MB of points "
                             "stay in L2 across one run's iterations" if 4 * n * d < 100e6
                             else "inputs larger than L2")},
           "qerr": q, "assign_ms_per_iter": ms_assign / iters,
           "update_ms_per_iter": (ms_tot - ms_assign) / iters,
           "band_pass_points": int(o.n_band), "split_pass_points": int(o.n_second),
           "fallback_points": int(o.n_fallback), "gpu_launches": launches,
           "clocks": clk.summary()}
    pk_tf, pk_hbm, pk_src = peaks()
    flop = 2.0 * n * k * d
    rec["roofline"] = {"bound": "tensor",
                       "kernel": "assignment step (packing, 16-bit tensor-core pass, exact "
                                 "re-rank), CUDA events per iteration",
                       "achieved": flop / (ms_assign / iters / 1e3) / 1e12, "unit": "TFLOP/s",
                       "peak": pk_tf, "peak_source": pk_src,
                       "algorithmic": f"2*n*k*d = {flop:.4g} flop per iteration",
                       "traffic": None}
    rec["roofline"]["frac"] = rec["roofline"]["achieved"] / pk_tf
    bytes_it = 2.0 * 4 * n * d  # the points read by the assignment and the update
    rec["hbm_view"] = {"achieved_gbs": bytes_it / (ms_tot / iters / 1e3) / 1e9,
                       "peak_gbs": pk_hbm, "frac": bytes_it / (ms_tot / iters / 1e3) / 1e9 / pk_hbm,
                       "algorithmic": "2 x 4*n*d bytes per iteration (assignment + update)"}
    # the plain FP32 path (the drop-in default): the whole run where it takes
    # seconds, its first iteration on the large configuration
    it32 = niter if n <= 200_000 else 1
    flush_l2(dev)
    q32, ms32, o32 = run(yg.PREC_FP32, it32)
    rec["plain_fp32"] = {"value": 1e3 * o32.iterations / ms32, "unit": "iterations/s",
                         "iterations_timed": int(o32.iterations),
                         "assign_ms_per_iter": o32.ms_assign / max(1, o32.iterations)}
    if it32 == niter:
        rec["plain_fp32"]["same_assignments"] = bool((assign.cpu().numpy() == a_ch).all())
    rec["speedup_vs_plain_fp32"] = rec["value"] / rec["plain_fp32"]["value"]
    # parity: the assignment of every iteration against the oracle's FP64
    # nearest centroid (all points on the small configuration, a fixed sample
    # of 100k on the large one), the objective against the FP64 sum
    if not args.no_check:
        nprobe = n if n <= 200_000 else min(n, 100_000)
        rows = (np.arange(n, dtype=np.int64) if nprobe == n else
                np.sort(np.random.default_rng(0).choice(n, nprobe, replace=False)))
        pa = np.empty((niter, nprobe), np.int32)
        pc = np.empty((niter, k, d), np.float32)
        pq = np.zeros(niter, np.float64)
        probe = {"n_probe": nprobe, "probe_rows": rows.ctypes.data, "probe_iters": niter,
                 "probe_assign": pa.ctypes.data, "probe_centroids": pc.ctypes.data,
                 "probe_qerr": pq.ctypes.data}
        _, _, op = run(prec, niter, probe)
        T = int(op.iterations)
        a_fin = assign.cpu().numpy()
        xs = (v_h if v_h is not None else None)
        if xs is None or nprobe != n:
            xs = np.ascontiguousarray(dv[torch.from_numpy(rows).to(dev)].cpu().numpy())
        t0 = time.perf_counter()
        bad = [assign_mismatches(xs, pc[t], pa[t], nt)[0] for t in range(T)]
        vh = v_h if v_h is not None else None
        if vh is None:
            vh = dv.cpu().numpy()
        q64 = objective64(vh, pc[T - 1], a_fin, nt)
        rec["parity"] = {
            "checked_points_per_iteration": nprobe, "iterations_checked": T,
            "assignment_mismatches_vs_fp64_oracle": int(sum(bad)),
            "same_run_as_timed": bool((a_fin == a_ch).all()),
            "objective_last_iteration": float(pq[T - 1]), "objective_fp64": q64,
            "objective_rel_err_vs_fp64": abs(float(pq[T - 1]) - q64) / q64,
            "check_seconds": time.perf_counter() - t0}
        if n <= 200_000:
            # the whole run against the oracle's exact-mode k-means
            Co = np.zeros((k, d), np.float32)
            ao = np.empty(n, np.int32)
            libc.srand48(0)
            qo = oracle().orc_kmeans(d, n, k, niter, ptr(v_h), nt | flags, seed, 1, ptr(Co),
                                     None, ptr(ao), None, 1, None)
            rec["parity"]["oracle_exact_kmeans"] = {
                "assignments_identical": bool((ao == a_fin).all()),
                "centroids_bit_identical": bool((Co == C.cpu().numpy()).all()),
                "qerr_rel_diff": abs(float(qo) - float(q)) / abs(float(qo))}
        del pc
    # end to end: the drop-in kmeans() with host buffers (copies included)
    vh = v_h if v_h is not None else dv.cpu().numpy()
    vp = torch.from_numpy(vh).pin_memory()
    Ch = torch.empty((k, d)).pin_memory()
    dh = torch.empty(n).pin_memory()
    ah = torch.empty(n, dtype=torch.int32).pin_memory()
    nh = torch.empty(k, dtype=torch.int32).pin_memory()
    os.environ["YAEL_GPU_PRECISION"] = args.prec
    libc.srand48(0)
    t0 = time.perf_counter()
    L.kmeans(d, n, k, niter, vp.data_ptr(), flags, seed, 1, Ch.data_ptr(), dh.data_ptr(),
             ah.data_ptr(), nh.data_ptr())
    te = time.perf_counter() - t0
    rec["e2e"] = {"value": (iters / runs) / te, "unit": "iterations/s",
                  "h2d_bytes_per_step": 4 * n * d, "d2h_bytes_per_step": 4 * (k * d + 2 * n + k),
                  "api": "kmeans (drop-in C ABI), pinned host buffers, one whole run per step"}
    del vp
    # the reference algorithm (oracle port) on the host cores: the whole run on
    # the small configuration, one iteration on 1% of the points on the large one
    if not args.no_cpu:
        sub = vh if n <= 200_000 else np.ascontiguousarray(vh[: n // 100])
        it = niter if n <= 200_000 else 1
        Cc = np.zeros((k, d), np.float32)
        libc.srand48(0)
        t0 = time.perf_counter()
        oracle().orc_kmeans(d, sub.shape[0], k, it, ptr(sub), nt | flags, seed, 1, ptr(Cc),
                            None, None, None, 0, None)
        cdt = time.perf_counter() - t0
        rec["cpu_baseline"] = {"value": it * (sub.shape[0] / n) / cdt, "unit": "iterations/s",
                               "cores": nt, "kind": "port",
                               "sample": f"{it} iteration(s) on {sub.shape[0]} points, seed "
                                         f"{seed}, value scaled to the full n"}
    del dv
    torch.cuda.empty_cache()
    return rec


def hkm_record(args, local):
    """Hierarchical k-means (n = 2M, d = 96, bf = 32, 3 levels, 15 iterations)
    through yael_gpu_hkm_learn_ex and the drop-in hkm_learn (both from host
    buffers; the tree is a host-array API), parity on a tenth of the points
    against the oracle's exact-mode tree, the reference algorithm on the host."""
    import torch
    import yael_gb300 as yg
    from yael_gb300 import synth
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from _util import oracle, ptr
    dev = torch.device("cuda", local)
    L = yg.lib()
    c = dict(CLUSTER_CFG["hkm4"])
    if args.niter:
        c["niter"] = args.niter
    if args.n:
        c["n"] = args.n
    v_h, _, _ = synth.gaussian_mixture(c["n"], c["d"], c["comps"], c["sigma"], seed=11)
    n, d = v_h.shape
    nl, bf, niter = c["nlevel"], c["bf"], c["niter"]
    ncent = sum(bf ** (l + 1) for l in range(nl))
    cent = np.empty(ncent * d, np.float32)
    assign = np.empty(n, np.int32)
    it, ms = ctypes.c_long(0), ctypes.c_float(0)
    vp = torch.from_numpy(v_h).pin_memory()
    libc = ctypes.CDLL(None)
    libc.srand48.argtypes = [ctypes.c_long]

    def learn(x, nn):
        libc.srand48(0)
        st = yg.CallStats()
        rc = L.yael_gpu_hkm_learn_ex(nn, d, nl, bf, x, niter, 1, ptr(cent), ptr(assign),
                                     ctypes.byref(it), ctypes.byref(ms))
        assert rc == 0, yg.last_error()
        L.yael_gpu_last_stats(ctypes.byref(st))
        return st

    # the plain FP32 form first (the drop-in default), then the chosen form
    os.environ["YAEL_GPU_PRECISION"] = "fp32"
    learn(vp.data_ptr(), n)
    t0 = time.perf_counter()
    learn(vp.data_ptr(), n)
    dt32 = time.perf_counter() - t0
    os.environ["YAEL_GPU_PRECISION"] = args.prec
    learn(vp.data_ptr(), n)  # warm-up (kernel attributes, packing buffers)
    l0 = L.yael_gpu_launch_count()
    with ClockSampler(local) as clk:
        t0 = time.perf_counter()
        st = learn(vp.data_ptr(), n)
        dt = time.perf_counter() - t0
    launches = L.yael_gpu_launch_count() - l0
    pk_tf, pk_hbm, pk_src = peaks()
    # algorithmic bytes: one read of every active instance's points per
    # iteration (the fused pass reads them once; 4*d bytes a point)
    alg = 4.0 * d * st.point_iterations
    rec = {"metric": METRIC, "value": it.value / dt, "unit": "instance-iterations/s",
           "ms_per_step": 1e3 * dt, "steps": 1, "warmup": 1, "higher_is_better": True,
           "dtype": {0: "f32", 1: "bf16", 3: "f16"}.get(st.prec_used, "?"),
           "config": {"workload": f"hierarchical k-means n={n} d={d} bf={bf} nlevel={nl} "
                                  f"niter={niter}, Gaussian mixture ({c['comps']} comps, "
                                  f"sigma={c['sigma']})", "n": n, "d": d,
                      "l2": "inputs larger than L2"},
           "tree_ms": 1e3 * dt, "gpu_ms": ms.value, "instance_iterations": it.value,
           "level_iterations": int(st.level_iterations), "gpu_launches": launches,
           "assign_ms": st.ms_assign, "update_ms": st.ms_update, "clocks": clk.summary(),
           "roofline": {"bound": "hbm", "kernel": "assignment passes (all levels), CUDA events",
                        "achieved": alg / (st.ms_assign / 1e3) / 1e9 if st.ms_assign > 0 else None,
                        "unit": "GB/s", "peak": pk_hbm, "peak_source": pk_src,
                        "algorithmic": "4*d bytes per point per iteration of its instance "
                                       f"({alg:.4g} bytes in the tree)", "traffic": None}}
    if rec["roofline"]["achieved"]:
        rec["roofline"]["frac"] = rec["roofline"]["achieved"] / pk_hbm
    rec["whole_tree_hbm_frac"] = alg / dt / 1e9 / pk_hbm
    rec["plain_fp32"] = {"value": it.value / dt32, "unit": "instance-iterations/s",
                         "tree_ms": 1e3 * dt32}
    rec["speedup_vs_plain_fp32"] = dt32 / dt
    # end to end: the call above takes the points from (pinned) host memory and
    # returns the tree there; the device time excludes the upload.  (The
    # drop-in hkm_learn stops on this data, as the reference's kmeans assert
    # would: a level-1 child gets fewer points than bf, and small_nodes = 1
    # gives such a node one child per point instead.)
    rec["value"] = it.value / (ms.value / 1e3)
    rec["ms_per_step"] = ms.value  # the tree on the device (the value's time)
    rec["e2e"] = {"value": it.value / dt, "unit": "instance-iterations/s",
                  "h2d_bytes_per_step": 4 * n * d, "d2h_bytes_per_step": 4 * (ncent * d + n),
                  "api": "yael_gpu_hkm_learn_ex (small_nodes = 1), pinned host buffer"}
    nt = os.cpu_count() or 1
    sub = np.ascontiguousarray(v_h[: n // 10])
    if not args.no_check:
        # the tree of a tenth of the points, GPU against the oracle's exact mode
        cg = np.empty_like(cent)
        ag = np.empty(sub.shape[0], np.int32)
        libc.srand48(0)
        rc = L.yael_gpu_hkm_learn_ex(sub.shape[0], d, nl, bf, ptr(sub), niter, 1, ptr(cg),
                                     ptr(ag), None, None)
        co = np.empty_like(cent)
        ao = np.empty(sub.shape[0], np.int32)
        libc.srand48(0)
        t0 = time.perf_counter()
        # exact mode (1) with the small-node rule of the GPU call (0x100)
        ro = oracle().orc_hkm_learn(sub.shape[0], d, nl, bf, ptr(sub), niter, ptr(co), ptr(ao),
                                    1 | 0x100)
        rec["parity"] = {"points": sub.shape[0], "status": [rc, ro],
                         "assignments_identical_to_oracle_exact": bool((ag == ao).all()),
                         "centroids_bit_identical": bool((cg == co).all()),
                         "check_seconds": time.perf_counter() - t0}
    if not args.no_cpu:
        oc = np.empty_like(cent)
        libc.srand48(0)
        t0 = time.perf_counter()
        # port mode (the reference's arithmetic) with the same small-node rule
        oracle().orc_hkm_learn(sub.shape[0], d, nl, bf, ptr(sub), niter, ptr(oc), None, 0x100)
        cdt = time.perf_counter() - t0
        # the tree has the same instances and iterations at n / 10; each
        # instance's work is linear in its points: time x 10 for the full n
        rec["cpu_baseline"] = {"value": it.value / (10 * cdt), "unit": "instance-iterations/s",
                               "seconds_on_tenth": cdt, "cores": nt, "kind": "port",
                               "sample": f"hkm_learn on n/10 = {sub.shape[0]} points, time x 10, "
                                         "the GPU run's instance-iteration count"}
    del vp
    return rec


def run_clustering(args, world, rank, local):
    """--workload kmeans1 | kmeans3 | hkm4: the configuration's record as the line."""
    import torch
    torch.cuda.set_device(local)
    rec = hkm_record(args, local) if args.workload == "hkm4" else kmeans_record(args.workload,
                                                                               args, local)
    rec.update({"n_gpus": world, "scaling": "weak", "vs_baseline": None, "data": "synthetic"})
    if rank == 0:
        print(json.dumps(rec), flush=True)


class _quiet_stdout:
    """Silences the C library's progress lines on file descriptor 1 (the
    reference's k-means / EM / LSH chatter) so that the JSON line stays alone."""

    def __enter__(self):
        sys.stdout.flush()
        self.saved = os.dup(1)
        self.null = os.open(os.devnull, os.O_WRONLY)
        os.dup2(self.null, 1)

    def __exit__(self, *exc):
        ctypes.CDLL(None).fflush(None)
        os.dup2(self.saved, 1)
        os.close(self.saved)
        os.close(self.null)


def run_callers(args, world, rank, local):
    """The path's callers, timed through their drop-in calls with host buffers
    (host <-> device copies included): gmm_learn / gmm_compute_p / gmm_fisher,
    kmlsh_ann_fvec, vlad_compute, knn_full_thread with the L1 / chi2 distances,
    kmeans with KMEANS_L1.
    The CPU figure is the oracle's restatement in the reference's arithmetic on
    a bounded sample, on the host's threads."""
    import torch
    import yael_gb300 as yg
    from yael_gb300 import synth
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    from _util import oracle, ptr
    torch.cuda.set_device(local)
    L = yg.lib()
    for name, (res, argt) in yg.SIGNATURES.items():
        if name.startswith(("gmm_", "kmlsh_", "nnlist_")):
            getattr(L, name).restype = res
            getattr(L, name).argtypes = argt
    os.environ["YAEL_GPU_PRECISION"] = args.prec
    line = {"n_gpus": world, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "data": "synthetic",
            "dtype": "f32" if args.workload in ("gmm", "alt", "kmeans_l1") else args.prec,
            "steps": 1, "warmup": 1}
    if args.workload == "gmm":
        import gmm_oracle as go
        n = args.n or 1_000_000
        d, k, niter = 128, 256, args.niter or 10
        v, _, _ = synth.gaussian_mixture(n, d, k, 0.5, seed=21)
        flags = go.FLAGS_W

        def learn():
            t0 = time.perf_counter()
            with _quiet_stdout():
                gp = L.gmm_learn(d, n, k, niter, ptr(v), 1, 1, 1, flags)
            return gp, time.perf_counter() - t0

        gp, _ = learn()  # warm-up
        L.gmm_delete(gp)
        C = np.zeros((k, d), np.float32)
        t0 = time.perf_counter()
        with _quiet_stdout():
            L.kmeans(d, n, k, niter, ptr(v), 1 | yg.KMEANS_QUIET, 1, 1, ptr(C), None, None, None)
        t_seed = time.perf_counter() - t0
        gp, t_learn = learn()
        p = np.empty((n, k), np.float32)
        t0 = time.perf_counter()
        L.gmm_compute_p(n, ptr(v), gp, ptr(p), flags)
        t_p = time.perf_counter() - t0
        fl = go.FLAGS_W | go.FLAGS_MU | go.FLAGS_SIGMA
        fv = np.empty(L.gmm_fisher_sizeof(gp, fl), np.float32)
        t0 = time.perf_counter()
        L.gmm_fisher(n, ptr(v), gp, fl, ptr(fv))
        t_f = time.perf_counter() - t0
        t_em = max(t_learn - t_seed, 1e-9)
        line.update({"metric": "GMM EM iterations/s (gmm_learn, k-means seeding excluded)",
                     "unit": "EM iterations/s", "value": niter / t_em,
                     "ms_per_step": 1e3 * t_em / niter,
                     "config": {"workload": f"gmm_learn n={n} d={d} k={k} niter={niter} "
                                            f"flags=GMM_FLAGS_W, Gaussian mixture (k comps, "
                                            f"sigma 0.5)", "n": n, "d": d, "k": k},
                     "gmm_learn_seconds": t_learn, "kmeans_seeding_seconds": t_seed,
                     "e2e": {"gmm_compute_p_vectors_per_s": n / t_p,
                             "gmm_fisher_w_mu_sigma_vectors_per_s": n / t_f,
                             "h2d_bytes_per_step": 4 * n * d, "d2h_bytes_per_step": 4 * n * k}})
        L.gmm_delete(gp)
        if not args.no_cpu:
            # one EM iteration of the reference's arithmetic (the oracle's port,
            # bit-identical to the reference library: sgemm forms, nt slices) on
            # n / 10 vectors, scaled to n
            nt = os.cpu_count() or 1
            sub = np.ascontiguousarray(v[: n // 10])
            rng = np.random.default_rng(0)
            mu0 = np.ascontiguousarray(sub[rng.choice(sub.shape[0], k, replace=False)])
            w0 = np.full(k, 1.0 / k, np.float32)
            s0 = np.ones((k, d), np.float32)
            o = oracle()
            o.orc_gmm_em_step.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_int,
                                          ctypes.c_int] + [ctypes.c_void_p] * 3 + [ctypes.c_int] * 2
            t0 = time.perf_counter()
            o.orc_gmm_em_step(sub.shape[0], ptr(sub), d, k, ptr(w0), ptr(mu0), ptr(s0), flags, nt)
            cdt = time.perf_counter() - t0
            line["cpu_baseline"] = {"value": (sub.shape[0] / n) / cdt, "unit": "EM iterations/s",
                                    "cores": nt, "kind": "port",
                                    "sample": f"one EM iteration (posteriors, splits, parameters) "
                                              f"in the reference's arithmetic (BLAS sgemm, {nt} "
                                              f"slices) on {sub.shape[0]} vectors, scaled to n"}
    elif args.workload == "vlad":
        n, d, k = (args.n or 1_000_000), 128, 256
        v = synth.sift_like(n, d, seed=31)
        C = synth.sift_like(k, d, seed=32)
        desc = np.empty((k, d), np.float32)
        L.vlad_compute(k, d, ptr(C), 10_000, ptr(v), ptr(desc))  # warm-up
        t0 = time.perf_counter()
        L.vlad_compute(k, d, ptr(C), n, ptr(v), ptr(desc))
        dt = time.perf_counter() - t0
        line.update({"metric": "VLAD descriptors/s (vlad_compute, host buffers)",
                     "unit": "vectors/s", "value": n / dt, "ms_per_step": 1e3 * dt,
                     "config": {"workload": f"vlad_compute n={n} d={d} k={k}, SIFT-like vectors "
                                            f"and centroids", "n": n, "d": d, "k": k},
                     "e2e": {"value": n / dt, "unit": "vectors/s", "h2d_bytes_per_step": 4 * n * d,
                             "d2h_bytes_per_step": 4 * k * d}})
        if not args.no_cpu:
            nt = os.cpu_count() or 1
            sub = v  # the whole workload: a fraction of a second per million vectors
            o = oracle()
            o.orc_vlad_compute.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p,
                                           ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                                           ctypes.c_int]
            od = np.empty((k, d), np.float32)
            t0 = time.perf_counter()
            o.orc_vlad_compute(k, d, ptr(C), sub.shape[0], ptr(sub), ptr(od), nt)
            cdt = time.perf_counter() - t0
            line["cpu_baseline"] = {"value": sub.shape[0] / cdt, "unit": "vectors/s",
                                    "cores": nt, "kind": "port",
                                    "sample": f"vlad_compute in the reference's arithmetic "
                                              f"(bit-identical to it) on {sub.shape[0]} vectors"}
    elif args.workload == "kmeans_l1":
        n, d, k, niter, seed = (args.n or 100_000), 128, 256, (args.niter or 5), 3
        v = synth.sift_like(n, d, seed=41)
        C = np.zeros((k, d), np.float32)
        flags = yg.KMEANS_QUIET | yg.KMEANS_INIT_RANDOM | yg.KMEANS_L1
        with _quiet_stdout():
            L.kmeans(d, 5000, k, 1, ptr(v), flags, seed, 1, ptr(C), None, None, None)  # warm-up
        t0 = time.perf_counter()
        with _quiet_stdout():
            L.kmeans(d, n, k, niter, ptr(v), flags, seed, 1, ptr(C), None, None, None)
        dt = time.perf_counter() - t0
        line.update({"metric": "L1 k-means iterations/s (kmeans with KMEANS_L1: exhaustive L1 "
                               "assignment, per-coordinate medians)",
                     "unit": "iterations/s", "value": niter / dt, "ms_per_step": 1e3 * dt / niter,
                     "config": {"workload": f"kmeans KMEANS_L1 n={n} d={d} k={k} niter={niter} "
                                            f"seed={seed}, SIFT-like", "n": n, "d": d, "k": k},
                     "e2e": {"value": niter / dt, "unit": "iterations/s",
                             "h2d_bytes_per_step": 4 * n * d // niter,
                             "d2h_bytes_per_step": 4 * k * d // niter}})
        if not args.no_cpu:
            nt = os.cpu_count() or 1
            sub = np.ascontiguousarray(v[: n // 10])
            Cc = np.zeros((k, d), np.float32)
            t0 = time.perf_counter()
            oracle().orc_kmeans(d, sub.shape[0], k, 2, ptr(sub), nt | (flags & ~0xffff), seed, 1,
                                ptr(Cc), None, None, None, 0, None)
            cdt = time.perf_counter() - t0
            line["cpu_baseline"] = {"value": 2 * (sub.shape[0] / n) / cdt,
                                    "unit": "iterations/s", "cores": nt, "kind": "port",
                                    "sample": f"2 iterations of KMEANS_L1 in the reference's "
                                              f"arithmetic (bit-identical to it) on "
                                              f"{sub.shape[0]} points, scaled to n"}
    elif args.workload == "alt":
        nb, nq, d, k = (args.n or 100_000), 1000, 128, 10
        b = synth.sift_like(nb, d, seed=1)
        q = synth.sift_like(nq, d, seed=2)
        idx = np.empty((nq, k), np.int32)
        dis = np.empty((nq, k), np.float32)
        rates = {}
        for t in (1, 3):  # L1, chi2
            L.knn_full_thread(t, 10, nb, d, k, ptr(b), ptr(q), None, ptr(idx), ptr(dis), 1)
            t0 = time.perf_counter()
            L.knn_full_thread(t, nq, nb, d, k, ptr(b), ptr(q), None, ptr(idx), ptr(dis), 1)
            rates[t] = nq / (time.perf_counter() - t0)
        line.update({"metric": "k-NN queries/s with the per-coordinate distances "
                               "(knn_full_thread, L1; chi2 beside it)",
                     "unit": "queries/s", "value": rates[1], "ms_per_step": 1e3 * nq / rates[1],
                     "config": {"workload": f"knn_full_thread distance_type 1 (L1) nb={nb} "
                                            f"nq={nq} d={d} k={k}, SIFT-like", "nb": nb, "nq": nq,
                                "d": d, "k": k},
                     "chi2_queries_per_s": rates[3],
                     "e2e": {"value": rates[1], "unit": "queries/s",
                             "h2d_bytes_per_step": 4 * (nb + nq) * d,
                             "d2h_bytes_per_step": 8 * nq * k}})
        if not args.no_cpu:
            nt = os.cpu_count() or 1
            nqs = nq
            qs = np.ascontiguousarray(q[:nqs])
            oi = np.empty((nqs, k), np.int32)
            od = np.empty((nqs, k), np.float32)
            t0 = time.perf_counter()
            oracle().orc_knn_port(1, nqs, nb, d, k, ptr(b), ptr(qs), None, ptr(oi), ptr(od), nt)
            cdt = time.perf_counter() - t0
            line["cpu_baseline"] = {"value": nqs / cdt, "unit": "queries/s", "cores": nt,
                                    "kind": "port",
                                    "sample": f"knn_full_thread L1 in the reference's arithmetic "
                                              f"(bit-identical to it) for {nqs} queries"}
    else:
        nb, nq, d, k, nhash = (args.n or 1_000_000), 10_000, 128, 100, 4
        b = synth.sift_like(nb, d, seed=1)
        q = synth.sift_like(nq, d, seed=2)

        def ann(bb, qq):
            t0 = time.perf_counter()
            with _quiet_stdout():
                lp = L.kmlsh_ann_fvec(ptr(bb), bb.shape[0], ptr(qq), qq.shape[0], d, k, nhash, 1)
            dt = time.perf_counter() - t0
            nl = ctypes.cast(lp, ctypes.POINTER(ctypes.c_long))
            idx = np.ctypeslib.as_array(ctypes.cast(nl[2], ctypes.POINTER(ctypes.c_int)),
                                        shape=(qq.shape[0] * k,)).reshape(-1, k).copy()
            L.nnlist_delete(lp)
            return idx, dt

        ann(b[:100_000], q[:1000])  # warm-up
        idx, dt = ann(b, q)
        exact = np.empty((nq, k), np.int32)
        dis = np.empty((nq, k), np.float32)
        L.knn_full_thread(2, nq, nb, d, k, ptr(b), ptr(q), None, ptr(exact), ptr(dis), 1)
        recall = float(np.mean([len(np.intersect1d(idx[i], exact[i])) for i in range(nq)]) / k)
        line.update({"metric": "k-means LSH queries/s (kmlsh_ann_fvec: learn, index, search)",
                     "unit": "queries/s", "value": nq / dt, "ms_per_step": 1e3 * dt,
                     "config": {"workload": f"kmlsh_ann_fvec nb={nb} nq={nq} d={d} k={k} "
                                            f"nhash={nhash} (nclust={int(np.sqrt(nb))}), "
                                            f"SIFT-like data", "nb": nb, "nq": nq, "d": d,
                                "k": k},
                     "recall_at_k_vs_exact": recall})
        if not args.no_cpu:
            sb, sq = np.ascontiguousarray(b[:100_000]), np.ascontiguousarray(q[:1000])
            _, gdt = ann(sb, sq)
            o = oracle()
            o.orc_kmlsh_ann.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p,
                                        ctypes.c_int] + [ctypes.c_int] * 6 + [ctypes.c_void_p] * 2
            oi = np.empty((1000, k), np.int32)
            od = np.empty((1000, k), np.float32)
            nt = min(os.cpu_count() or 1, 255)  # KMLSH_NT holds 8 bits
            t0 = time.perf_counter()
            o.orc_kmlsh_ann(ptr(sb), 100_000, ptr(sq), 1000, d, k, nhash, 0, 0, nt, ptr(oi),
                            ptr(od))
            cdt = time.perf_counter() - t0
            line["cpu_baseline"] = {"value": 1000 / cdt, "unit": "queries/s", "cores": nt,
                                    "kind": "port",
                                    "sample": "the reference's algorithm in its own arithmetic "
                                              "(oracle port) at nb=100000 nq=1000; the GPU on "
                                              "the same sample: "
                                              f"{1000 / gdt:.1f} queries/s"}
    if rank == 0:
        print(json.dumps(line), flush=True)


def batch_sizes(npairs, seed):
    """Pair sizes of the batched uneven k-NN configuration: queries log-uniform
    in [1, 8192], base rows log-uniform in [10,000, 2,000,000]."""
    rng = np.random.default_rng(seed)
    nq = np.floor(np.exp(rng.uniform(np.log(1), np.log(8193), npairs))).astype(np.int64)
    nb = np.floor(np.exp(rng.uniform(np.log(1e4), np.log(2e6 + 1), npairs))).astype(np.int64)
    return np.clip(nq, 1, 8192), np.clip(nb, 10_000, 2_000_000)


def run_knn_batch(args, world, rank, local):
    """--workload knn_batch: the batch record as the line."""
    import torch
    torch.cuda.set_device(local)
    line = knn_batch_record(args, local, world, rank)
    if rank == 0:
        print(json.dumps(line), flush=True)


def knn_batch_record(args, local, world=1, rank=0):
    """Batched uneven exact k-NN: 512 independent (queries, base) pairs, d = 128,
    k = 32, unit-normalised Gaussian rows, L2 and inner product, through
    yael_gpu_knn_batch; the plain FP32 per-pair loop beside it; ids of a
    sample of queries from eight pairs against the oracle's FP64 brute force."""
    import torch
    import yael_gb300 as yg
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from _util import knn_port
    dev = torch.device("cuda", local)
    L = yg.lib()
    npairs, d, k = args.pairs, 128, 32
    nq, nb = batch_sizes(npairs, 5 + 1000 * rank)
    gen = torch.Generator(device=dev)
    qs, bs = [], []
    for i in range(npairs):  # seeded per pair, generated and normalised in HBM
        gen.manual_seed(1_000_003 * (rank + 1) + i)
        b = torch.randn((int(nb[i]), d), device=dev, generator=gen)
        b /= b.norm(dim=1, keepdim=True)
        q = torch.randn((int(nq[i]), d), device=dev, generator=gen)
        q /= q.norm(dim=1, keepdim=True)
        bs.append(b)
        qs.append(q)
    idx = [torch.empty((int(n), k), dtype=torch.int32, device=dev) for n in nq]
    dis = [torch.empty((int(n), k), device=dev) for n in nq]
    descs = (yg.KnnPair * npairs)()
    for i in range(npairs):
        descs[i] = yg.KnnPair(int(nq[i]), int(nb[i]), qs[i].data_ptr(), bs[i].data_ptr(),
                              idx[i].data_ptr(), dis[i].data_ptr())
    torch.cuda.synchronize(dev)
    flops = float(np.sum(2.0 * nq * nb * d))

    def batch_call(prec, metric):
        o = yg.KnnOpts(prec, metric, 1, None)
        rc = L.yael_gpu_knn_batch(npairs, ctypes.cast(descs, ctypes.c_void_p), d, k,
                                  ctypes.byref(o))
        if rc != 0:
            raise RuntimeError(yg.last_error())
        return o

    def timed(prec, metric, steps, warmup):
        for _ in range(warmup):
            batch_call(prec, metric)
        torch.cuda.synchronize(dev)
        l0 = L.yael_gpu_launch_count()
        with ClockSampler(local) as clk:
            t0 = time.perf_counter()
            for _ in range(steps):
                o = batch_call(prec, metric)
            torch.cuda.synchronize(dev)
            dt = time.perf_counter() - t0
        return dt / steps, L.yael_gpu_launch_count() - l0, o, clk.summary()

    steps = max(1, args.steps)
    sec, launches, o, clocks = timed(yg.PREC_BF16, 2, steps, args.warmup)
    sec_ip, _, o_ip, _ = timed(yg.PREC_BF16, 16, max(1, steps // 2), 1)
    # parity: up to 32 queries of each of eight pairs (the largest and smallest
    # bases and queries, and four drawn at random) against the FP64 oracle
    check = None
    if not args.no_check:
        from _util import knn_mismatches
        batch_call(yg.PREC_BF16, 2)
        torch.cuda.synchronize(dev)
        sel = {0, int(np.argmax(nb)), int(np.argmin(nb)), int(np.argmax(nq)),
               int(np.argmax(nq * nb))}
        sel |= set(int(x) for x in np.random.default_rng(1).choice(npairs, 4, replace=False))
        nbad, nchk = 0, 0
        for i in sorted(sel):
            m = min(32, int(nq[i]))
            nbad += knn_mismatches(bs[i].cpu().numpy(), qs[i][:m].cpu().numpy(),
                                   idx[i][:m].cpu().numpy(), os.cpu_count() or 1)[0]
            nchk += m
        check = {"pairs": len(sel), "queries": nchk, "queries_with_id_mismatch": nbad}
    # the plain FP32 path, one knn call per pair (the drop-in loop)
    t0 = time.perf_counter()
    for i in range(npairs):
        o32 = yg.KnnOpts(yg.PREC_FP32, 2, 1, None)
        L.yael_gpu_knn_ex(int(nq[i]), int(nb[i]), d, k, bs[i].data_ptr(), qs[i].data_ptr(),
                          idx[i].data_ptr(), dis[i].data_ptr(), ctypes.byref(o32))
    torch.cuda.synchronize(dev)
    sec32 = time.perf_counter() - t0
    # end to end with host buffers for the first pairs (pinned copies of the same data)
    ne = min(npairs, args.e2e_pairs)
    hq = [qs[i].cpu().pin_memory() for i in range(ne)]
    hb = [bs[i].cpu().pin_memory() for i in range(ne)]
    hi = [torch.empty((int(nq[i]), k), dtype=torch.int32).pin_memory() for i in range(ne)]
    hd = [torch.empty((int(nq[i]), k)).pin_memory() for i in range(ne)]
    hdesc = (yg.KnnPair * ne)()
    for i in range(ne):
        hdesc[i] = yg.KnnPair(int(nq[i]), int(nb[i]), hq[i].data_ptr(), hb[i].data_ptr(),
                              hi[i].data_ptr(), hd[i].data_ptr())
    oe = yg.KnnOpts(yg.PREC_BF16, 2, 0, None)
    L.yael_gpu_knn_batch(ne, ctypes.cast(hdesc, ctypes.c_void_p), d, k, ctypes.byref(oe))
    t0 = time.perf_counter()
    rc = L.yael_gpu_knn_batch(ne, ctypes.cast(hdesc, ctypes.c_void_p), d, k, ctypes.byref(oe))
    sec_e2e = time.perf_counter() - t0
    if rc != 0:
        raise RuntimeError(yg.last_error())
    # CPU: the reference algorithm (oracle port) on a bounded sample
    cpu = None
    if not args.no_cpu:
        sel = np.argsort(nb)[:4]
        tq, tt = 0, 0.0
        for i in sel:
            m = min(int(nq[i]), 200)
            bh = bs[i].cpu().numpy()
            qh = qs[i][:m].cpu().numpy()
            t1 = time.perf_counter()
            knn_port(bh, qh, k, nt=os.cpu_count() or 1)
            tt += time.perf_counter() - t1
            tq += m
        cpu = {"value": tq / tt, "unit": "queries/s", "cores": os.cpu_count() or 1,
               "kind": "port",
               "sample": f"<= 200 queries of each of the 4 pairs with the smallest bases "
                         f"(nb {int(nb[sel].min())}..{int(nb[sel].max())}); the whole batch "
                         f"averages nb = {int(nb.mean())}"}
    pk = peaks()
    tot_q = float(np.sum(nq))
    line = {
        "metric": METRIC, "value": world * tot_q / sec, "unit": "queries/s", "n_gpus": world,
        "steps": steps, "warmup": args.warmup, "ms_per_step": 1e3 * sec,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "bf16",
        "data": "synthetic",
        "config": {"workload": f"batched uneven exact k-NN, {npairs} pairs: nq log-uniform "
                               f"[1, 8192], nb log-uniform [1e4, 2e6], d={d}, k={k}, "
                               "unit-normalised Gaussian rows, L2",
                   "pairs": npairs, "sum_nq": int(tot_q), "sum_nb": int(np.sum(nb)),
                   "flop_per_step": flops, "l2": "inputs larger than L2"},
        "inner_product": {"value": world * tot_q / sec_ip, "unit": "queries/s",
                          "ms_per_step": 1e3 * sec_ip, "fallback_queries": o_ip.n_fallback},
        "plain_fp32_per_pair_loop": {"value": tot_q / sec32, "unit": "queries/s",
                                     "ms_per_step": 1e3 * sec32},
        "parity": check,
        "fallback_queries": o.n_fallback, "band_queries": o.n_band,
        "path": ("grouped: one persistent launch per pass over all pairs, waves pipelined"
                 if os.environ.get("YAEL_GPU_BATCH_GROUPED", "1") != "0"
                 else "worker pool, one pipeline per pair"),
        "roofline": {"bound": "tensor", "kernel": "whole batch (all passes)",
                     "achieved": flops / sec / 1e12, "unit": "TFLOP/s", "peak": pk[0],
                     "frac": flops / sec / 1e12 / pk[0], "peak_source": pk[2],
                     "traffic": None},
        "e2e": {"value": float(np.sum(nq[:ne])) / sec_e2e, "unit": "queries/s",
                "h2d_bytes_per_step": int(4 * d * (np.sum(nq[:ne]) + np.sum(nb[:ne]))),
                "d2h_bytes_per_step": int(8 * k * np.sum(nq[:ne])),
                "api": f"yael_gpu_knn_batch with pinned host buffers, first {ne} pairs "
                       "(host arrays: the worker pool)"},
        "gpu_launches": launches, "clocks": clocks,
    }
    if cpu:
        line["cpu_baseline"] = cpu
    del bs, qs, idx, dis
    torch.cuda.empty_cache()
    return line


def config_of(args):
    return {"workload": f"exact kNN L2, SIFT-like float32 (30% zeros, floor|N(0,40)| clipped "
                        f"to 255), nb={args.nb}, nq={args.nq}, d={args.d}, k={args.k}",
            "nb": args.nb, "nq": args.nq, "d": args.d, "k": args.k,
            "precision": args.prec,
            "l2": "inputs larger than L2 (base alone is 4*nb*d bytes)"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=60)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--nb", type=int, default=1_000_000)
    ap.add_argument("--nq", type=int, default=10_000)
    ap.add_argument("--d", type=int, default=128)
    ap.add_argument("--k", type=int, default=100)
    ap.add_argument("--prec", default="bf16", choices=["bf16", "fp32"])
    ap.add_argument("--fp32-steps", type=int, default=2, help="steps of the plain FP32 path")
    ap.add_argument("--e2e-steps", type=int, default=10)
    ap.add_argument("--cpu-budget", type=float, default=10.0)
    ap.add_argument("--ref-queries", type=int, default=500)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-check", action="store_true", help="skip the FP64 spot check")
    ap.add_argument("--niter", type=int, default=0, help="override the clustering iterations")
    ap.add_argument("--n", type=int, default=0,
                    help="override the clustering point count (smaller cases for profiling)")
    ap.add_argument("--cluster-runs", type=int, default=5,
                    help="kmeans1: whole k-means runs timed (L2 flushed between runs)")
    ap.add_argument("--no-workloads", action="store_true",
                    help="default run: only the k-NN line, without the clustering and "
                         "batch records")
    ap.add_argument("--pairs", type=int, default=512, help="knn_batch: number of pairs")
    ap.add_argument("--e2e-pairs", type=int, default=64,
                    help="knn_batch: pairs timed end to end from host buffers")
    ap.add_argument("--workload", default="knn",
                    choices=["knn", "kmeans1", "kmeans3", "hkm4", "knn_batch", "gmm", "kmlsh",
                             "vlad", "alt", "kmeans_l1"],
                    help="knn: the headline configuration; the others are the k-means / hkm "
                         "configurations and the path's callers (gmm, kmlsh, vlad, alt, "
                         "kmeans_l1), reported "
                         "separately")
    args = ap.parse_args()
    world, rank, local = dist_setup()
    if args.impl == "reference" and args.workload != "knn":
        # the reference arm times the headline configuration; every other
        # workload's record carries its own CPU figure
        if rank == 0:
            print(json.dumps({"impl": "reference", "unavailable":
                              "the reference's CPU figure for this workload is the "
                              "cpu_baseline of the ours line (the oracle's port on a "
                              "bounded sample)"}), flush=True)
        return
    if args.workload in ("gmm", "kmlsh", "vlad", "alt", "kmeans_l1"):
        run_callers(args, world, rank, local)
        return
    if args.workload == "knn_batch" and args.impl != "reference":
        run_knn_batch(args, world, rank, local)
        return
    if args.workload not in ("knn", "knn_batch"):
        run_clustering(args, world, rank, local)
        return

    if args.impl == "reference":
        run_reference(args, world, rank)
        return

    import torch
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    import yael_gb300 as yg
    from yael_gb300 import replicas, synth
    L = yg.lib()
    dev = torch.device("cuda", local)

    # the same base on every rank, a different query set per rank (replicas: weak scaling)
    b_h = synth.sift_like(args.nb, args.d, seed=1)
    q_h = synth.sift_like(args.nq, args.d, seed=replicas.query_seed(rank))
    b = torch.from_numpy(b_h).to(dev)
    q = torch.from_numpy(q_h).to(dev)
    idx = torch.empty((args.nq, args.k), dtype=torch.int32, device=dev)
    dis = torch.empty((args.nq, args.k), dtype=torch.float32, device=dev)
    stream = torch.cuda.Stream(device=dev)
    prec = {"bf16": yg.PREC_BF16, "fp32": yg.PREC_FP32}[args.prec]

    def step(p, timing=1):
        o = yg.KnnOpts(p, 2, 1, ctypes.c_void_p(stream.cuda_stream), 0, 0, 0, timing, 0, 0, 0, 0, 0)
        rc = L.yael_gpu_knn_ex(args.nq, args.nb, args.d, args.k, b.data_ptr(), q.data_ptr(),
                               idx.data_ptr(), dis.data_ptr(), ctypes.byref(o))
        if rc != 0:
            raise RuntimeError(yg.last_error())
        return o

    def timed(p, steps, warmup):
        for _ in range(warmup):
            step(p)
        torch.cuda.synchronize(dev)
        if dist:
            dist.barrier()
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        l0 = L.yael_gpu_launch_count()
        scan_ms, scan_n, fb, sample_ms, rr_ms = 0.0, 0, 0, 0.0, 0.0
        with ClockSampler(local) as clk:
            ev0.record(stream)
            for _ in range(steps):
                o = step(p)
                scan_ms += o.ms_scan
                scan_n += o.scan_launches
                fb += o.n_fallback
                sample_ms += o.ms_sample
                rr_ms += o.ms_rerank
            ev1.record(stream)
            torch.cuda.synchronize(dev)
        ms = ev0.elapsed_time(ev1)
        launches = L.yael_gpu_launch_count() - l0
        ms = replicas.max_over_ranks(ms, dist, dev)
        return ms, launches, scan_ms / max(1, scan_n), fb, clk.summary(), sample_ms / steps, rr_ms / steps

    ms, launches, scan_ms, fb, clocks, sample_ms, rr_ms = timed(prec, args.steps, args.warmup)
    qps = replicas.whole_job_rate(args.nq * args.steps, ms / 1e3, world)

    # parity of the timed configuration: every query's ids against the oracle's
    # FP64 brute force (outside the timed region)
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from _util import exact_dist64, knn_mismatches
    parity = None
    if not args.no_check:
        t0 = time.perf_counter()
        gi, gd = idx.cpu().numpy(), dis.cpu().numpy()
        nbad, first = knn_mismatches(b_h, q_h, gi, os.cpu_count() or 1)
        m = min(256, args.nq)
        d64 = exact_dist64(b_h, q_h[:m], gi[:m])
        parity = {"queries_checked": int(args.nq), "queries_with_id_mismatch": nbad,
                  "first_mismatch": first,
                  "distance_max_rel_err_first256": float(
                      np.max(np.abs(gd[:m] - d64) / np.maximum(d64, 1e-30))),
                  "check_seconds": time.perf_counter() - t0}

    # plain FP32 path (the drop-in default) for the speed-up of the chosen form
    fp32 = None
    if args.prec == "bf16" and args.fp32_steps > 0:
        ms32, _, scan32, _, _, _, _ = timed(yg.PREC_FP32, args.fp32_steps, 1)
        fp32 = {"value": world * args.nq * args.fp32_steps / (ms32 / 1e3), "unit": "queries/s",
                "main_pass_ms": scan32}
        step(yg.PREC_FP32, 0)
        i32 = idx.cpu().numpy().copy()
        step(prec, 0)
        fp32["ids_equal_bf16"] = bool((idx.cpu().numpy() == i32).all())

    # end to end through the drop-in C ABI with pinned host buffers
    os.environ["YAEL_GPU_PRECISION"] = args.prec
    bp = torch.from_numpy(b_h).pin_memory()
    qp = torch.from_numpy(q_h).pin_memory()
    ip = torch.empty((args.nq, args.k), dtype=torch.int32).pin_memory()
    dp = torch.empty((args.nq, args.k), dtype=torch.float32).pin_memory()

    def e2e_step():
        L.knn_full_thread(2, args.nq, args.nb, args.d, args.k, bp.data_ptr(), qp.data_ptr(), None,
                          ip.data_ptr(), dp.data_ptr(), os.cpu_count() or 1)

    e2e_s = 0.0
    if args.e2e_steps > 0:
        for _ in range(max(3, args.warmup)):  # includes the chunk tuner's trials of this path
            e2e_step()
        if dist:
            dist.barrier()
        t0 = time.perf_counter()
        for _ in range(args.e2e_steps):
            e2e_step()
        e2e_s = time.perf_counter() - t0
    e2e_s = replicas.max_over_ranks(e2e_s, dist, dev)
    e2e_qps = replicas.whole_job_rate(args.nq * args.e2e_steps, e2e_s, world) if e2e_s > 0 else None

    if rank != 0:
        if dist:
            dist.barrier()
        return

    pk_tf, pk_hbm, pk_src = peaks()
    flops = 2.0 * args.nq * args.nb * args.d
    achieved = flops / (scan_ms / 1e3) / 1e12 if scan_ms > 0 else None
    line = {
        "metric": METRIC, "value": qps, "unit": "queries/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "bf16" if args.prec == "bf16" else "f32", "data": "synthetic",
        "config": config_of(args),
        "parity": parity,
        "fallback_queries_per_step": fb / args.steps,
        "phase_ms": {"threshold_sample_pass": sample_ms, "main_pass": scan_ms, "rerank": rr_ms},
        "roofline": {"bound": "tensor", "kernel": "tc_scan_kernel (THRESH, main pass)",
                     "achieved": achieved, "peak": pk_tf, "unit": "TFLOP/s",
                     "frac": (achieved / pk_tf) if achieved else None,
                     "peak_source": pk_src,
                     "traffic": KNN_MAIN_TRAFFIC if (args.nb, args.nq, args.d, args.k) ==
                     (1_000_000, 10_000, 128, 100) else None,
                     "traffic_unit": "bytes per launch",
                     "algorithmic": f"2*nq*nb*d = {flops:.4g} flop per launch"},
        "e2e": {"value": e2e_qps, "unit": "queries/s",
                "h2d_bytes_per_step": 4 * (args.nb + args.nq) * args.d,
                "d2h_bytes_per_step": 8 * args.nq * args.k,
                "api": "knn_full_thread (drop-in C ABI), pinned host buffers"},
        "gpu_launches": launches,
        "clocks": clocks,
    }
    if fp32:
        line["plain_fp32"] = fp32
        line["speedup_vs_plain_fp32"] = qps / fp32["value"]
    if not args.no_cpu and world >= 1:
        cqps, nt, nq_done, blas = cpu_port_qps(b_h, q_h, args.k, budget_s=args.cpu_budget)
        line["cpu_baseline"] = {"value": cqps, "unit": "queries/s", "cores": nt, "kind": "port",
                                "sample": f"{nq_done} queries vs the full {args.nb}-row base, "
                                          f"knn_full_thread restated (BLAS {os.path.basename(blas)})"}
    if world == 1 and not args.no_workloads:
        # the other configurations of the metric, each a record of its own:
        # k-means (small and large), hierarchical k-means, the batched k-NN
        del b, q, idx, dis, bp, qp, ip, dp
        torch.cuda.empty_cache()
        wl = {}
        for name in ("kmeans1", "kmeans3", "hkm4", "knn_batch"):
            t0 = time.perf_counter()
            try:
                if name == "hkm4":
                    r = hkm_record(args, local)
                elif name == "knn_batch":
                    r = knn_batch_record(args, local)
                else:
                    r = kmeans_record(name, args, local)
            except Exception as e:  # a failed record is reported, not hidden
                r = {"error": f"{type(e).__name__}: {e}"}
            r["record_seconds"] = time.perf_counter() - t0
            wl[name] = r
        line["workloads"] = wl
    print(json.dumps(line), flush=True)
    if dist:
        dist.barrier()


if __name__ == "__main__":
    main()
