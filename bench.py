"""Benchmark: eff_h2 applies/s at bond dimension 1024 (dense ComplexF64 Heisenberg,
63-site binary tree), mixed split-bf16 tcgen05 path vs the plain FP64 GPU path.

One step = one application y = H_eff x of the two-site effective Hamiltonian of the
depth-3 -> depth-2 edge of binary_topology(5) at D = 1024 (Θ legs [8, 8, 2, 128, 2, 1024],
33.6 M complex entries; environments [8,5,8] x2, [128,5,128], [1024,5,1024]; Heisenberg
TTNO, w = 5).  Inputs are seeded synthetic tensors of exactly those shapes.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line.  ``--impl reference`` times the CPU restatement of the reference
path (numpy/OpenBLAS on all host cores) on the same workload.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "graft.jl_gb300")
for _p in (ROOT, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import numpy as np  # noqa: E402

METRIC = "eff_h2 applies/s at D=1024 (bin63 Heisenberg, depth3->depth2 edge), mixed split-product tcgen05"
WORKLOAD = "heisenberg_bin63_d3d2_D1024_eff_h2"
D, W_OP, d = 1024, 5, 2


# ---------------------------------------------------------------------------------------
# workload
# ---------------------------------------------------------------------------------------

WORKLOADS = {
    # name: (topology, node n, bond dim) -- n's parent is m
    "heisenberg_bin63_d3d2_D1024_eff_h2": ("binary", "n3_1", 1024),
    "heisenberg_bin63_d3d2_D256_eff_h2": ("binary", "n3_1", 256),
    "heisenberg_chain63_mid_D1024_eff_h2": ("mps", "site32", 1024),
    # the other D = 256 edge classes of the binary tree that fit one GPU (depth2 -> depth1
    # holds a 64 GiB two-site block at D = 256; at D = 64 it is 1 GiB)
    "heisenberg_bin63_d1root_D256_eff_h2": ("binary", "n1_1", 256),
    "heisenberg_bin63_d4d3_D256_eff_h2": ("binary", "n4_1", 256),
    "heisenberg_bin63_d5d4_D256_eff_h2": ("binary", "n5_1", 256),
    "heisenberg_bin63_d2d1_D64_eff_h2": ("binary", "n2_1", 64),
}


DTYPES = {"bf16x6": "bf16x6 split products on tcgen05, f32 accumulate, c128 in/out",
          "fp16x3": "fp16x3 split products (power-of-two row scales) on tcgen05, f32 accumulate, c128 in/out",
          "bf16x3": "bf16x3 split products on tcgen05, f32 accumulate, c128 in/out"}
PRODUCTS = {"bf16x6": 6, "fp16x3": 3, "bf16x3": 3}


def metric_for(workload):
    """The headline metric for the headline workload; the same quantity, labelled by its
    workload, for the others (both arms use it, so their lines stay comparable)."""
    if workload == WORKLOAD:
        return METRIC
    return f"eff_h2 applies/s ({workload}), mixed split-product tcgen05"


def workload_arrays(name=WORKLOAD, seed=7, bond_dim=None):
    """Labels, order and seeded synthetic statics of one eff_h2 map of the workload table.
    Bond dimensions follow the saturated tree: min(D, product of the legs below); bond_dim
    replaces the table's D (small instances for checks).  On a root edge the root's parent
    leg has dimension 1 and is closed by the ones cap, as eff_h2 does."""
    import grafttn as G
    from grafttn import contractions as GC
    kind, nid, Dm = WORKLOADS[name]
    Dm = bond_dim or Dm
    topo = G.binary_topology(5) if kind == "binary" else G.mps_topology(63)
    n = topo.index[nid]
    m = topo.parent[n]
    rng = np.random.default_rng(seed)

    def crandn(shape):
        return (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)) / np.sqrt(2)

    def env(dim):
        # Hermitian in (ket, bra) for every operator index, like a converged environment
        e = crandn((dim, W_OP, dim)) / np.sqrt(dim)
        return (e + e.conj().transpose(2, 1, 0)) / 2
    below = {}
    for v in topo.postorder():
        below[v] = d * int(np.prod([below[c] for c in topo.children[v]] or [1]))
    bond = {v: min(Dm, below[v]) for v in range(topo.nnodes)}
    Ws = G.ttno_tensors(G.heisenberg(topo))
    k = topo.childslot(m, n)
    root_edge = topo.parent[m] < 0
    x_shape = tuple([bond[c] for c in topo.children[n]] + [d]
                    + [bond[c] for c in topo.children[m] if c != n] + [d, 1 if root_edge else bond[m]])
    pn = topo.nchildren(n) + 1
    labels, order, envs = GC.h2_spec(topo, n, m, len(x_shape), Ws[n].ndim, Ws[m].ndim, pn)
    statics = [Ws[n], Ws[m]] + [env(bond[w] if w != topo.parent[u] else bond[u]) for (w, u) in envs]
    if root_edge:
        statics.append(np.ones((1, 1, 1), dtype=np.complex128))
    theta = crandn(x_shape)
    theta /= np.linalg.norm(theta)
    assert k >= 0
    return x_shape, labels, order, statics, theta


def oracle_flops(x_shape, labels, order, statics):
    from oracle import ttn_oracle as O
    return 8 * O.plan_macs([x_shape] + [s.shape for s in statics], labels, order)


# ---------------------------------------------------------------------------------------
# clocks during the timed region
# ---------------------------------------------------------------------------------------

REASON_BITS = {0x1: "gpu_idle", 0x2: "applications_clocks_setting", 0x4: "sw_power_cap", 0x8: "hw_slowdown",
               0x10: "sync_boost", 0x20: "sw_thermal_slowdown", 0x40: "hw_thermal_slowdown",
               0x80: "hw_power_brake_slowdown", 0x100: "display_clock_setting"}


class ClockSampler:
    def __init__(self, device=0):
        self.device = device
        self.samples = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.device}", "--query-gpu=clocks.sm,clocks.max.sm,clocks_event_reasons.active",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 3:
                try:
                    self.samples.append((float(parts[0]), float(parts[1]), int(parts[2], 16)))
                except ValueError:
                    pass

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [s[0] for s in self.samples]
        reasons = set()
        for s in self.samples:
            for bit, name in REASON_BITS.items():
                if s[2] & bit and name != "gpu_idle":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(s[1] for s in self.samples),
                "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------------------------------
# CPU arm: the oracle restatement of the reference path on the host cores
# ---------------------------------------------------------------------------------------

def cpu_apply_rate(x_shape, labels, order, statics, theta, budget_s=20.0, max_applies=3, warm=False):
    """Applications of the oracle's env-first map per second on the host cores; stops after
    `max_applies` or once `budget_s` is spent (at least one application).  Also returns the
    oracle's output y = H_eff theta, the parity reference of the GPU results."""
    from oracle import ttn_oracle as O
    hm = O.EffMap(labels, order, statics, x_shape)
    if warm:
        hm(theta)
    n, t0 = 0, time.perf_counter()
    y = None
    while n < max_applies:
        y = hm(theta)
        n += 1
        if time.perf_counter() - t0 > budget_s:
            break
    el = time.perf_counter() - t0
    return n / el, n, el, y


def blas_threads():
    try:
        from threadpoolctl import threadpool_info
        info = threadpool_info()
        return max((i.get("num_threads", 1) for i in info), default=os.cpu_count())
    except Exception:
        return os.cpu_count()


def run_reference(args, rank, world):
    """The reference arm: the CPU restatement of the reference path on all host cores.  A
    step is one full application; the timed steps are capped by a 150 s budget (a bounded
    sample of K steps), the count actually timed is reported in `steps`."""
    if rank != 0:
        return
    from oracle import ttn_oracle as O
    x_shape, labels, order, statics, theta = workload_arrays(args.workload)
    flops = oracle_flops(x_shape, labels, order, statics)
    hm = O.EffMap(labels, order, statics, x_shape)
    t_w = time.perf_counter()
    for _ in range(min(args.warmup, 1)):
        hm(theta)
    t_apply = time.perf_counter() - t_w if args.warmup > 0 else None
    steps = args.steps
    if t_apply:
        steps = max(1, min(args.steps, int(150.0 // max(t_apply, 1e-9))))
    t0 = time.perf_counter()
    for _ in range(steps):
        hm(theta)
    total = time.perf_counter() - t0
    value = steps / total
    args = argparse.Namespace(**{**vars(args), "steps": steps})
    cores = blas_threads()
    line = {
        "impl": "reference", "metric": metric_for(args.workload), "value": value, "unit": "applies/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * total / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "c128 (f64)",
        "data": "synthetic (seeded Gaussian tensors of the workload shapes)",
        "config": {"workload": args.workload, "theta_shape": list(x_shape), "bond_dim": WORKLOADS[args.workload][2], "ttno_bond": W_OP,
                   "algorithmic_flops_per_apply": flops},
        "cpu_baseline": {"value": value, "unit": "applies/s", "cores": cores, "kind": "port",
                         "sample": f"{args.steps} full eff_h2 applications (numpy tensordot chain, env-first order)"},
        "e2e": {"value": value, "unit": "applies/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "achieved_tflops": flops * value / 1e12,
    }
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------------------

def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            j = json.load(f)
        return j.get("bf16_tflops"), j.get("hbm_gbs"), "measured"
    return 1900.0, 6800.0, "fallback"


def profile_traffic(kernel, workload):
    """Per-launch DRAM bytes of `kernel` from the committed ncu summary (profiles/traffic.txt)."""
    p = os.path.join(ROOT, "profiles", "traffic.txt")
    if not os.path.exists(p):
        return None
    with open(p) as f:
        for line in f:
            parts = line.split()
            if len(parts) >= 3 and parts[0] == kernel and parts[1] == workload:
                return float(parts[2])
    return None


def _timed(stream, fn, reps):
    import torch
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(reps):
        fn()
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps


def bench_u1(ctx, steps):
    """U(1) Sz-conserving Heisenberg, block-sparse: eff_h2 on the same bin63 depth3->depth2
    edge at total bond dimension 1024 (bond sectors: subtree charge counts, dims binomial
    scaled to the bond dimension and clipped to [4, 256]); all coupled-charge blocks of a
    step in one grouped launch, the application replayed as one CUDA graph."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from u1_cases import h2_u1_case
    from grafttn import blocksparse as B
    from oracle import u1_oracle as U
    xs, labels, order, statics, x = h2_u1_case(5, "n3_1", 1024)
    plan = B.BlockPlan(xs, labels[0], statics, order)
    dx = ctx.upload(x)
    out = {"theta_blocks": len(xs.blocks), "theta_elems": xs.size, "algorithmic_flops_per_apply": plan.flops,
           "static_groups": plan.groups,
           "sector_gemms_mkn_per_step": [sorted([int(g.M), int(g.K), int(g.N)] for g in gm) for _, gm in plan.steps]}
    ys = {}
    for prec in ("bf16x6", "fp16x3", "fp64"):
        bm = B.BlockEffectiveMap(ctx, plan, prec, graph=True)
        dy = ctx.empty((plan.y.size,))
        for _ in range(3):
            bm.apply_into(dx, dy)
        ctx.sync()
        l0 = ctx.launches
        reps = steps if prec != "fp64" else max(2, steps // 4)
        ms = _timed(ctx.stream, lambda: bm.apply_into(dx, dy), reps)
        out[prec] = {"applies_per_s": 1000.0 / ms, "ms_per_apply": ms, "tflops": plan.flops / ms / 1e9,
                     "launches_per_apply": (ctx.launches - l0) / reps}
        ys[prec] = ctx.download(dy)
        out["coupled_charge_problems"] = bm.n_problems
        bm.close()
    y64 = ys["fp64"]
    for prec in ("bf16x6", "fp16x3"):
        out[prec]["rel_err_vs_fp64"] = float(np.linalg.norm(ys[prec] - y64) / np.linalg.norm(y64))
        out[prec]["speedup_vs_fp64"] = out[prec]["applies_per_s"] / out["fp64"]["applies_per_s"]
    # HBM roofline of the block map: the minimal bytes of one application are x read once
    # and y written once (c128), every intermediate coupled-charge output written and read
    # once (c64 in the mixed modes), and every static block read once (c128); the problems
    # are skinny (N of a few to ~200), so bytes, not tensor flops, bound them
    mkn = out["sector_gemms_mkn_per_step"]
    inter = sum(m * n for step in mkn[:-1] for m, _, n in step)
    static_elems = sum(n * k for step in mkn for _, k, n in step)
    hbm = measured_peaks()[1]
    for prec in ("bf16x6", "fp16x3", "fp64"):
        e_mid = 32 if prec == "fp64" else 16
        nbytes = 16 * xs.size + 16 * plan.y.size + e_mid * inter + 16 * static_elems
        gbs = nbytes / (out[prec]["ms_per_apply"] * 1e-3) / 1e9
        out[prec]["hbm_roofline"] = {"algorithmic_bytes": int(nbytes), "achieved_gbs": gbs, "peak_gbs": hbm,
                                     "frac": gbs / hbm if hbm else None}
    blocks = [U.blocks_from_flat(xs, x)] + [U.blocks_from_flat(T, d) for T, _, d in statics]
    t0 = time.perf_counter()
    y_cpu = U.flat_from_blocks(plan.y, U.ncon_blocks(blocks, labels, order))
    el = time.perf_counter() - t0
    out["cpu_baseline"] = {"applies_per_s": 1.0 / el, "kind": "port (per-sector block tensordot, numpy)",
                           "cores": blas_threads(), "sample": "1 application"}
    out["fp64_vs_cpu_rel_err"] = float(np.linalg.norm(y64 - y_cpu) / np.linalg.norm(y_cpu))
    return out


def bench_batched(ctx, steps):
    """64 independent eff_h1 maps with uneven bond dimensions in [16, 256] (chain nodes with
    two bonds, tree nodes with three bonds <= 48): grouped launches per step replayed as one
    CUDA graph, against 64 sequential single-map applications."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from test_gpu_batched import make_batch
    from grafttn.contractions import MapBatch
    rng = np.random.default_rng(64)
    maps, xs, refs = make_batch(ctx, rng, 64, 16, 256, "bf16x6")
    ys = [ctx.empty(m.y_shape) for m in maps]
    b = MapBatch(maps, xs, ys, graph=True)
    for _ in range(3):
        b.run()
    ctx.sync()
    l0 = ctx.launches
    ms_b = _timed(ctx.stream, b.run, steps)
    launches = (ctx.launches - l0) / steps

    def seq():
        for m, x, y in zip(maps, xs, ys):
            m.apply_into(x, y)
    seq()
    ms_s = _timed(ctx.stream, seq, max(2, steps // 2))
    err = max(float(np.linalg.norm(ctx.download(y) - r) / np.linalg.norm(r)) for y, r in zip(ys, refs))
    flops = sum(m.flops for m in maps)
    b.close()
    for m in maps:
        m.close()
    return {"instances": 64, "ms_batched_graph": ms_b, "ms_sequential": ms_s, "speedup": ms_s / ms_b,
            "launches_per_batched_apply": launches, "tflops_batched": flops / ms_b / 1e9, "max_rel_err_vs_oracle": err}


def run_ours(args, rank, world):
    import torch
    import grafttn as G
    from grafttn.contractions import EffectiveMap
    if world > 1:
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", rank)))
    dev = torch.cuda.current_device()
    ctx = G.default_context(dev)
    x_shape, labels, order, statics, theta = workload_arrays(args.workload)
    dstat = [ctx.upload(s) for s in statics]
    x = ctx.upload(theta)
    hm = EffectiveMap(ctx, x_shape, labels, order, dstat, args.precision)
    y = ctx.empty(hm.y_shape)
    flops = hm.flops  # algorithmic flop of the env-first chain (8 per complex MAC)
    stream = ctx.stream

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()

    for _ in range(args.warmup):
        hm.apply_into(x, y)
    ctx.sync()
    barrier()
    torch.cuda.synchronize()
    l0 = ctx.launches
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(dev) as clk:
        time.sleep(0.3)
        ev0.record(stream)
        for _ in range(args.steps):
            hm.apply_into(x, y)
        ev1.record(stream)
        torch.cuda.synchronize()
        time.sleep(0.2)
    ctx.sync()
    launches = ctx.launches - l0
    ms = ev0.elapsed_time(ev1)
    if world > 1:
        import torch.distributed as dist
        t = torch.tensor([ms], dtype=torch.float64, device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    barrier()
    value = world * args.steps / (ms / 1000.0)
    # accuracy of the mixed apply against the FP64 apply of the same map
    y64 = ctx.empty(hm.y_shape)
    hm.apply_into(x, y64, precision=0)
    ctx.sync()
    diff = ctx.empty(hm.y_shape)
    ctx.axpby(1.0, y, 0.0, diff)
    ctx.axpby(-1.0, y64, 1.0, diff)
    mixed_rel_err = ctx.norm(diff) / ctx.norm(y64)

    if rank != 0:
        return
    # FP64 GPU path on the same map (a bounded sample: each apply takes ~2 s on GB300)
    fp64_steps = max(1, min(2, args.steps))
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(fp64_steps):
        hm.apply_into(x, y64, precision=0)
    e1.record(stream)
    torch.cuda.synchronize()
    fp64_rate = fp64_steps / (e0.elapsed_time(e1) / 1000.0)

    # per-launch timing of one application (CUDA events on the launching stream)
    recs = hm.apply_profiled(x, y)
    by = {}
    for name, t, f in recs:
        a = by.setdefault(name, [0, 0.0, 0.0])
        a[0] += 1
        a[1] += t
        a[2] += f
    tot = sum(v[1] for v in by.values())
    kernels = {k: {"launches": v[0], "ms": round(v[1], 4), "share": round(v[1] / tot, 4)} for k, v in by.items()}
    tc = by.get("tc_gemm", [1, 1e-9, 0.0])
    exec_flops = sum(v[2] for v in by.values())           # flops of the executed (grouped) chain
    bf16_peak, hbm_peak, peak_kind = measured_peaks()
    # roofline of the dominant kernel: the env-first chain's algorithmic flops of one
    # application (8 per complex MAC) over the tc_gemm launches' event time of one application
    achieved = flops / (tc[1] / 1000.0) / 1e12
    # the tensor pipe's executed work: flops of the executed tc steps times the slice products
    executed = tc[2] * PRODUCTS[args.precision] / (tc[1] / 1000.0) / 1e12
    traffic = profile_traffic("tc_gemm", args.workload)

    # end to end through the C ABI with host buffers (page-locked): every step moves x from
    # and y to host memory inside the timed region
    xh = torch.from_numpy(theta.copy()).pin_memory()
    yh = torch.empty(hm.y_shape, dtype=torch.complex128).pin_memory()
    import ctypes as C
    from grafttn._lib import check
    e2e_steps = max(2, min(5, args.steps))
    hm.ctx.lib.gtn_map_apply_host(hm.h, C.c_void_p(xh.data_ptr()), C.c_void_p(yh.data_ptr()))
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        check(hm.ctx.lib.gtn_map_apply_host(hm.h, C.c_void_p(xh.data_ptr()), C.c_void_p(yh.data_ptr())), ctx.h)
    e2e_rate = e2e_steps / (time.perf_counter() - t0)
    # the host link alone: the same bytes copied between the page-locked buffers and HBM
    # (copies in the same direction saturate the link whatever the number of streams)
    dxc = torch.empty(xh.shape, dtype=xh.dtype, device="cuda")
    dyc = torch.empty(yh.shape, dtype=yh.dtype, device="cuda")
    link = {}
    for name, fn, nbytes in (("h2d_gbs", lambda: dxc.copy_(xh, non_blocking=True), xh.numel() * 16),
                             ("d2h_gbs", lambda: yh.copy_(dyc, non_blocking=True), yh.numel() * 16)):
        fn()
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        for _ in range(3):
            fn()
        torch.cuda.synchronize()
        link[name] = 3 * nbytes / (time.perf_counter() - t1) / 1e9
    del dxc, dyc

    # CPU baseline: the oracle on the host cores, bounded sample of the same workload; the
    # oracle's count of the chain's flop checks the library's
    cpu_rate, cpu_n, cpu_el, y_oracle = cpu_apply_rate(x_shape, labels, order, statics, theta, budget_s=20.0,
                                                        max_applies=2)
    oflops = oracle_flops(x_shape, labels, order, statics)
    assert abs(flops - oflops) / oflops < 1e-12, (flops, oflops)
    del statics
    # parity of the headline map itself: the GPU's FP64 and mixed outputs against the
    # oracle's output for the same theta (complex128 numpy tensordot chain)
    y64_h, ymix_h = ctx.download(y64), ctx.download(y)
    ref_norm = float(np.linalg.norm(y_oracle))
    fp64_vs_oracle = float(np.linalg.norm(y64_h - y_oracle) / ref_norm)
    mixed_vs_oracle = float(np.linalg.norm(ymix_h - y_oracle) / ref_norm)
    del y64_h, ymix_h, y_oracle
    parity_ok = fp64_vs_oracle <= 1e-12 and mixed_vs_oracle <= 2e-5

    segment = None
    if not args.skip_extra and not args.no_dmrg_segment:
        try:
            segment = dmrg_segment(ctx, args.segment_steps, args.precision)
        except Exception as exc:  # reported, never hides the headline
            segment = {"error": f"{type(exc).__name__}: {exc}"}
    gradient = None
    if not args.skip_extra:
        try:
            gradient = grad_segment(ctx, args.grad_D, tuple(args.grad_precisions.split(",")))
        except Exception as exc:  # reported, never hides the headline
            gradient = {"error": f"{type(exc).__name__}: {exc}"}

    extra = {}
    alt = {}
    for prec in [p for p in ("bf16x6", "fp16x3") if p != args.precision]:
        try:
            hm2 = EffectiveMap(ctx, x_shape, labels, order, dstat, prec)
            y2 = ctx.empty(hm2.y_shape)
            for _ in range(2):
                hm2.apply_into(x, y2)
            a0, a1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a0.record(stream)
            for _ in range(args.steps):
                hm2.apply_into(x, y2)
            a1.record(stream)
            torch.cuda.synchronize()
            ctx.axpby(1.0, y2, 0.0, diff)
            ctx.axpby(-1.0, y64, 1.0, diff)
            alt[prec] = {"value": args.steps / (a0.elapsed_time(a1) / 1000.0), "unit": "applies/s",
                         "rel_err_vs_fp64": ctx.norm(diff) / ctx.norm(y64)}
            hm2.close()
            del y2
        except Exception as exc:
            alt[prec] = {"error": f"{type(exc).__name__}: {exc}"}
    extra["other_mixed_modes"] = alt
    # the grouping choice: the same map compiled as the plain env-first chain (no
    # pre-contracted static groups), timed the same way
    try:
        os.environ["GTN_STATIC_GROUPING"] = "0"
        hm3 = EffectiveMap(ctx, x_shape, labels, order, dstat, args.precision)
        os.environ.pop("GTN_STATIC_GROUPING", None)
        y3 = ctx.empty(hm3.y_shape)
        for _ in range(2):
            hm3.apply_into(x, y3)
        b0, b1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        b0.record(stream)
        for _ in range(args.steps):
            hm3.apply_into(x, y3)
        b1.record(stream)
        torch.cuda.synchronize()
        recs3 = hm3.apply_profiled(x, y3)
        extra["grouping_ab"] = {"grouped_ms_per_apply": ms / args.steps,
                                "env_first_ms_per_apply": b0.elapsed_time(b1) / args.steps,
                                "env_first_executed_flops": sum(f for _, _, f in recs3),
                                "grouped_executed_flops": exec_flops, "algorithmic_flops": flops,
                                "env_first_tc_launches": sum(1 for k, _, _ in recs3 if k == "tc_gemm")}
        hm3.close()
        del y3
    except Exception as exc:
        os.environ.pop("GTN_STATIC_GROUPING", None)
        extra["grouping_ab"] = {"error": f"{type(exc).__name__}: {exc}"}
    if not args.skip_extra:
        for name, fn in (("u1_blocksparse", bench_u1), ("batched_eff_h1", bench_batched)):
            try:
                extra[name] = fn(ctx, args.steps)
            except Exception as exc:  # reported, never hides the headline
                extra[name] = {"error": f"{type(exc).__name__}: {exc}"}

    clocks = clk.summary()
    from grafttn import _lib as GL
    tuning = GL.tc_tune_report()
    line = {
        "metric": metric_for(args.workload), "value": value, "unit": "applies/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": DTYPES[args.precision],
        "data": "synthetic (seeded Gaussian tensors of the workload shapes)",
        "config": {"workload": args.workload, "theta_shape": list(x_shape), "bond_dim": WORKLOADS[args.workload][2], "ttno_bond": W_OP,
                   "algorithmic_flops_per_apply": flops, "l2": "inputs larger than L2 (Θ and intermediates exceed 129 MB)",
                   "parallelism": "replicas" if world > 1 else "single GPU"},
        "fp64_gpu": {"value": fp64_rate, "unit": "applies/s", "speedup_mixed_vs_fp64": value / world / fp64_rate,
                     "samples": fp64_steps},
        "mixed_vs_fp64_rel_err": mixed_rel_err,
        "fp64_vs_oracle_rel_err": fp64_vs_oracle,
        "mixed_vs_oracle_rel_err": mixed_vs_oracle,
        "parity_ok": parity_ok,
        "algorithmic_tflops": flops * value / world / 1e12,
        "kernels": kernels,
        "roofline": {"bound": "tensor", "kernel": "tc_gemm", "achieved": achieved, "peak": bf16_peak,
                     "unit": "TFLOP/s", "frac": achieved / bf16_peak, "peak_kind": f"bf16 dense burst ({peak_kind})",
                     "achieved_definition": ("algorithmic flops of one application (8 x complex MACs of the "
                                             "reference's env-first chain) / the tc_gemm launches' event time "
                                             "of one application"),
                     "tc_ms_per_apply": tc[1], "executed_macs_ratio": exec_flops / flops,
                     "executed_tensor_tflops": executed, "frac_executed": executed / bf16_peak,
                     "traffic": traffic},
        "cpu_baseline": {"value": cpu_rate, "unit": "applies/s", "cores": blas_threads(), "kind": "port",
                         "sample": f"{cpu_n} eff_h2 application(s) of the same workload, {cpu_el:.1f} s"},
        "e2e": {"value": e2e_rate, "unit": "applies/s", "h2d_bytes_per_step": int(theta.size * 16),
                "d2h_bytes_per_step": int(np.prod(hm.y_shape) * 16),
                "path": "gtn_map_apply_host (C ABI), page-locked host buffers: H2D copy, apply, D2H copy",
                "host_link": link,
                "copy_ms_per_step": 1e3 * (xh.numel() * 16 / link["h2d_gbs"] + yh.numel() * 16 / link["d2h_gbs"]) / 1e9},
        "gpu_launches": launches,
        "clocks": clocks,
        "tc_tile_choices": tuning,
    }
    if segment is not None:
        line["dmrg_segment"] = segment
    if gradient is not None:
        line["gradient"] = gradient
    line.update(extra)
    print(json.dumps(line), flush=True)
    if not parity_ok:
        sys.exit(f"parity failure: fp64 vs oracle {fp64_vs_oracle:.3e} (bound 1e-12), "
                 f"mixed vs oracle {mixed_vs_oracle:.3e} (bound 2e-5)")


def dmrg_segment(ctx, steps, precision, D=1024, refine_tol=1e-8):
    """The DMRG half of the metric, bounded: `steps` consecutive two-site dmrg2 steps in the
    middle of the dense Heisenberg chain mps_topology(63) at bond dimension D (Θ = [D,2,2,D]),
    from one seeded random state (seed 7, bonds min(D, 2^k)), once in the mixed mode and once
    in FP64 on the same state.  A step is the reference's local update (GroundState.jl:102-143):
    gauge move, merge, eff_h2 build, Lanczos (krylovdim 20, tol 1e-10), truncated SVD split at
    maxdim D.  In the mixed arm the Lanczos vector is then refined with FP64-accurate residuals
    (gtn_lanczos_refine) until |H v - E v| <= refine_tol * |E|, and its energy is the FP64
    Rayleigh quotient; the FP64-accurate work of that arm (residuals, environment rebuilds)
    runs on the tensor cores in GTN_PREC_FP64E (an FP64E twin of the map).  The FP64 arm is
    the plain FP64 GPU path: FP64 maps, FP64 environments.  The environments of the first
    step are built before the clock starts (the same for both arms); environment rebuilds
    after each split are timed."""
    import torch
    import grafttn as G
    from grafttn.contractions import EnvCache, eff_h2
    from grafttn.networks import move_center, split_two_site, two_site_tensor
    from grafttn.solvers import refine_local
    L = 63
    topo = G.mps_topology(L)
    H = G.TTNO.from_hamiltonian(G.heisenberg(topo), ctx)
    bond = {}
    for c in range(topo.nnodes):
        if topo.parent[c] >= 0:
            below = len(topo.subtree_nodes(c, topo.parent[c]))
            bond[c] = int(min(D, 2 ** min(below, 40), 2 ** min(L - below, 40)))
    psi0 = G.random_ttns(np.random.default_rng(7), topo, 2, bond, ctx=ctx)
    n0 = topo.index["site31"]
    cache0 = EnvCache(topo)
    move_center(psi0, n0, cache0)
    eff_h2(cache0, psi0, H, n0, topo.parent[n0], G._lib.PREC_FP64).close()  # builds the step-1 envs
    ctx.sync()
    trunc = G.TruncationScheme(maxdim=D)
    out = {"workload": f"mps63 Heisenberg (XX+YY+ZZ, Pauli), dense c128, D={D}, middle bonds site31->site32..",
           "steps": steps, "krylovdim": 20, "lanczos_tol": 1e-10, "refine_tol_rel": refine_tol, "runs": {}}
    for prec in (precision, "fp64"):
        psi, cache = psi0.copy(), cache0.copy()
        pcode = G._lib.PRECISIONS[prec]
        mixed = pcode != G._lib.PREC_FP64
        if mixed:  # the FP64-accurate work on the tensor cores, as dmrg2(fp64e=True) runs it
            cache.precision = G._lib.PREC_FP64E
        old_linalg = ctx.linalg_precision(G._lib.PREC_FP64E if mixed else G._lib.PREC_FP64)
        n = n0
        recs = []
        if pcode != G._lib.PREC_FP64:
            # a sweep has chosen its tile shapes long before: measure this bond's problem
            # classes once (a throw-away application of both maps on a copy) before the clock
            wpsi = psi.copy()
            wc = cache.copy()
            move_center(wpsi, n, wc)
            wth = two_site_tensor(wpsi, n, topo.parent[n])
            for wp in (pcode, G._lib.PREC_FP64E):
                wm = eff_h2(wc, wpsi, H, n, topo.parent[n], wp)
                wm(wth)
                wm.close()
            # and the split's factorisations of the same shapes (the solver library loads its
            # kernels on first use; a sweep pays that once, at its first step)
            split_two_site(wpsi, wth, n, topo.parent[n], trunc, "m")
            del wpsi, wc, wth
            torch.cuda.synchronize()
        for _ in range(steps):
            m = topo.parent[n]
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            move_center(psi, n, cache)
            theta = two_site_tensor(psi, n, m, precision=G._lib.PREC_FP64E if mixed else G._lib.PREC_FP64)
            h2 = eff_h2(cache, psi, H, n, m, pcode)
            h2e = None
            if pcode != G._lib.PREC_FP64:
                h2e = eff_h2(cache, psi, H, n, m, G._lib.PREC_FP64E)
                h2.set_fp64_map(h2e)
            E, v, info = h2.lanczos_min(theta, krylovdim=20, tol=1e-10, maxiter=100)
            rstats = {}
            if pcode != G._lib.PREC_FP64:
                E, v = refine_local(h2, E, v, refine_tol, stats=rstats)
            h2.close()
            if h2e is not None:
                h2e.close()
            cache.invalidate_edge(n, m)
            split_two_site(psi, v, n, m, trunc, "m")
            torch.cuda.synchronize()
            recs.append({"bond": [topo.ids[n], topo.ids[m]], "s": time.perf_counter() - t0, "energy": E,
                         "matvecs": info["matvecs"], "converged": info["converged"],
                         "refine_fp64_matvecs": rstats.get("refine_fp64_matvecs", 0),
                         "refine_mixed_matvecs": rstats.get("refine_mixed_matvecs", 0)})
            n = m
        ctx.linalg_precision(old_linalg)
        out["runs"][prec] = {"step_s": [r["s"] for r in recs], "energies": [r["energy"] for r in recs],
                             "matvecs": [r["matvecs"] for r in recs], "total_s": sum(r["s"] for r in recs),
                             "refine_fp64_matvecs": [r["refine_fp64_matvecs"] for r in recs],
                             "refine_mixed_matvecs": [r["refine_mixed_matvecs"] for r in recs]}
        if prec == precision:
            # the environment update after the split (the next step's env of the updated
            # site), on this state in both precisions: time and agreement
            nb = topo.parent[n0]
            envs = {}
            for eprec in ("fp64", "fp64e"):
                ec = cache.copy()
                ec.precision = G._lib.PRECISIONS[eprec]
                ec.env(psi, H, n0, nb).shape  # warm-up (packing, arena growth)
                ec.invalidate_edge(n0, nb)
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                E = ec.env(psi, H, n0, nb)
                torch.cuda.synchronize()
                envs[eprec] = (time.perf_counter() - t0, ctx.download(E))
            e64, ee = envs["fp64"][1], envs["fp64e"][1]
            out["env_update"] = {"env": f"E({topo.ids[n0]}->{topo.ids[nb]}) [ket, op, bra] = {list(e64.shape)}",
                                 "fp64_s": envs["fp64"][0], "fp64e_s": envs["fp64e"][0],
                                 "speedup_fp64e": envs["fp64"][0] / envs["fp64e"][0],
                                 "rel_diff": float(np.linalg.norm(ee - e64) / np.linalg.norm(e64))}
    r64 = out["runs"]["fp64"]
    rm = out["runs"][precision]
    out["rel_energy_vs_fp64"] = [abs(a - b) / abs(b) for a, b in zip(rm["energies"], r64["energies"])]
    out["time_ratio_fp64_over_mixed"] = r64["total_s"] / rm["total_s"]
    return out


def run_dmrg(args):
    """Two-site DMRG sweeps (dmrg2!) of the dense Heisenberg chain mps_topology(63) at bond
    dimension --dmrg-D, from one seeded random state, for each precision: wall time per
    sweep, matvecs and the final energy (mixed energies are FP64 Rayleigh quotients)."""
    import torch
    import grafttn as G
    ctx = G.default_context(0)
    L, D = args.dmrg_sites, args.dmrg_D
    topo = G.mps_topology(L) if args.dmrg_topology == "mps" else G.binary_topology(int(np.log2(L + 1)) - 1)
    H = G.TTNO.from_hamiltonian(G.heisenberg(topo), ctx)
    bond = {}
    for c in range(topo.nnodes):
        if topo.parent[c] >= 0:
            below = len(topo.subtree_nodes(c, topo.parent[c]))
            bond[c] = int(min(D, 2 ** min(below, 40), 2 ** min(L - below, 40)))
    psi0 = G.random_ttns(np.random.default_rng(7), topo, 2, bond, ctx=ctx)
    out = {"metric": "DMRG sweep time", "unit": "s/sweep", "topology": f"{args.dmrg_topology}{L}", "bond_dim": D,
           "model": "Heisenberg XX+YY+ZZ (Pauli), dense ComplexF64", "krylovdim": 20, "runs": {}}
    for label in args.dmrg_precisions.split(","):
        # "fp16x3+fp64e": the mixed maps with FP64-grade tensor-core environments, Rayleigh
        # quotients and refinement residuals; "+refine": FP64-residual refinement of every
        # local eigenvector (gtn_lanczos_refine)
        prec = label.split("+")[0]
        fp64e = "+fp64e" in label
        refine = "all" if ("+refine" in label or fp64e) and prec != "fp64" else "off"
        psi = psi0.copy()
        stats = {"timing": True}
        times, energies = [], []
        for sweep in range(args.dmrg_sweeps):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            _, Es = G.dmrg2(psi, H, G.TruncationScheme(maxdim=D), nsweeps=1, precision=prec, lanczos_tol=1e-10,
                            stats=stats, refine=refine, fp64e=fp64e)
            torch.cuda.synchronize()
            times.append(time.perf_counter() - t0)
            energies.append(Es[-1])
            print(f"dmrg {label} sweep {sweep + 1}: {times[-1]:.3f} s, E = {Es[-1]:.12f}, "
                  f"matvecs so far {stats.get('matvecs')}", file=sys.stderr, flush=True)
        out["runs"][label] = {"sweep_s": times, "energies": energies, "matvecs": stats.get("matvecs"),
                             "steps": stats.get("steps"),
                             "phase_s": {k[2:]: round(v, 3) for k, v in stats.items() if k.startswith("t_")}}
    runs = out["runs"]
    if "fp64" in runs and len(runs) > 1:
        e64 = runs["fp64"]["energies"][-1]
        for p, r in runs.items():
            if p != "fp64":
                r["rel_energy_vs_fp64"] = abs(r["energies"][-1] - e64) / abs(e64)
                r["sweep_speedup_vs_fp64"] = float(np.mean(runs["fp64"]["sweep_s"]) / np.mean(r["sweep_s"]))
    print(json.dumps(out), flush=True)


def run_lanczos(args):
    """One Lanczos solve in the middle of the dense Heisenberg chain mps_topology(63) at bond
    dimension --dmrg-D (Θ = [D,2,2,D]): the time of one map application against the time of
    one Lanczos iteration (application + Gram-Schmidt + coefficient read-back), krylovdim 20,
    two restarts (28 matvecs), from a seeded random start.  The solve runs inside the NVTX
    range "lanczos" so that a profiler can select its launches."""
    import torch
    import grafttn as G
    from grafttn.contractions import EnvCache, eff_h2
    from grafttn.networks import move_center, two_site_tensor
    ctx = G.default_context(0)
    L, D = 63, args.dmrg_D
    topo = G.mps_topology(L)
    H = G.TTNO.from_hamiltonian(G.heisenberg(topo), ctx)
    bond = {}
    for c in range(topo.nnodes):
        if topo.parent[c] >= 0:
            below = len(topo.subtree_nodes(c, topo.parent[c]))
            bond[c] = int(min(D, 2 ** min(below, 40), 2 ** min(L - below, 40)))
    psi = G.random_ttns(np.random.default_rng(7), topo, 2, bond, ctx=ctx)
    n = L // 2
    m = topo.parent[n]
    cache = EnvCache(topo)
    move_center(psi, n, cache)
    theta = two_site_tensor(psi, n, m)
    rng = np.random.default_rng(3)
    x0 = ctx.upload((rng.standard_normal(theta.shape) + 1j * rng.standard_normal(theta.shape)).astype(np.complex128))
    torch.cuda.synchronize()
    out = {"metric": "Lanczos iteration time", "unit": "ms", "topology": f"mps{L}", "bond_dim": D,
           "theta_shape": list(theta.shape), "krylovdim": 20, "runs": {}}
    for prec in args.dmrg_precisions.split(","):
        h2 = eff_h2(cache, psi, H, n, m, G._lib.PRECISIONS[prec])
        y = h2(theta)
        for _ in range(3):
            h2.apply_into(theta, y)
        ctx.sync()
        t0 = time.perf_counter()
        for _ in range(20):
            h2.apply_into(theta, y)
        ctx.sync()
        apply_ms = (time.perf_counter() - t0) / 20 * 1e3
        h2.lanczos_min(x0, krylovdim=20, tol=1e-14, maxiter=1)  # warm the basis allocation
        ctx.sync()
        torch.cuda.nvtx.range_push("lanczos")
        t0 = time.perf_counter()
        _, _, info = h2.lanczos_min(x0, krylovdim=20, tol=1e-14, maxiter=2)
        ctx.sync()
        torch.cuda.nvtx.range_pop()
        solve_s = time.perf_counter() - t0
        out["runs"][prec] = {"apply_ms": apply_ms, "solve_s": solve_s, "matvecs": info["matvecs"],
                             "iteration_ms": solve_s / info["matvecs"] * 1e3}
        h2.close()
    print(json.dumps(out), flush=True)


def run_svd(args):
    """Truncated SVD of one 8192 x 8192 complex matrix at maxdim 64, the shape of a two-site
    split on a depth-2 edge of the 63-site binary tree at D = 64: the subspace-iteration
    route against the Gram route (GTN_SVD_SUBSPACE=0).  The matrix is X Y with X = 8192 x 512
    Gaussian columns scaled by 0.9^i and Y = 512 x 8192 Gaussian (seeded, built on the
    device), so its spectrum decays like a DMRG two-site block's."""
    import torch
    import grafttn as G
    ctx = G.default_context(0)
    g = torch.Generator(device="cuda").manual_seed(3)
    n, r = 8192, 512
    sc = 0.9 ** torch.arange(r, device="cuda", dtype=torch.float64)
    A = ((torch.randn(n, r, dtype=torch.complex128, device="cuda", generator=g) * sc)
         @ torch.randn(r, n, dtype=torch.complex128, device="cuda", generator=g)).contiguous()
    torch.cuda.synchronize()
    out = {"metric": "truncated SVD time", "unit": "s", "shape": [n, n], "maxdim": 64, "routes": {}}
    old = os.environ.get("GTN_SVD_SUBSPACE")
    try:
        for route, flag in (("subspace", "1"), ("gram", "0")):
            os.environ["GTN_SVD_SUBSPACE"] = flag
            ts = []
            for _ in range(3):
                ctx.sync()
                t0 = time.perf_counter()
                _, S, _, disc = ctx.svd_trunc(A, maxdim=64)
                ctx.sync()
                ts.append(time.perf_counter() - t0)
            out["routes"][route] = {"s": ts, "best_s": min(ts[1:]), "sigma_0": float(S[0]),
                                    "sigma_63": float(S[63]), "discarded": disc}
    finally:
        if old is None:
            os.environ.pop("GTN_SVD_SUBSPACE", None)
        else:
            os.environ["GTN_SVD_SUBSPACE"] = old
    print(json.dumps(out), flush=True)


def grad_segment(ctx, D=128, precisions=("fp64", "fp16x3")):
    """Gradient workload: XXZ (Delta = 0.7) on binary_topology(4) (31 sites) at bond
    dimension D with per-edge couplings theta_e ~ U(0.5, 1.5): wall time of the gradient with
    respect to every site tensor (one eff_h1 application per node) and every coupling, the
    latter both through the adjoint of the TTNO operand (gtn_contract_vjp, chain rule through
    W(theta)) and as two-site expectation values; the identities <A_n, g_n> = E and
    sum_e theta_e dE/dtheta_e = E; central finite differences (h = 1e-6) on a sample."""
    import torch
    import grafttn as G
    from grafttn import gradients as GR
    topo = G.binary_topology(4)
    rng = np.random.default_rng(11)
    theta = {e: float(rng.uniform(0.5, 1.5)) for e in topo.edges()}
    S = G.spin_ops()
    terms = {e: [(1.0, S["X"], S["X"]), (1.0, S["Y"], S["Y"]), (0.7, S["Z"], S["Z"])] for e in topo.edges()}
    dco = {e: [1.0, 1.0, 0.7] for e in topo.edges()}

    def ttno(th):
        return G.TTNO.from_hamiltonian(G.xxz(topo, th, 0.7), ctx)
    Hnn = G.xxz(topo, theta, 0.7)
    H = G.TTNO.from_hamiltonian(Hnn, ctx)
    bond = {}
    for c in range(topo.nnodes):
        if topo.parent[c] >= 0:
            below = len(topo.subtree_nodes(c, topo.parent[c]))
            bond[c] = int(min(D, 2 ** below, 2 ** (topo.nnodes - below)))
    psi = G.random_ttns(rng, topo, 2, bond, ctx=ctx)
    E = GR.energy(psi, H).real
    out = {"workload": f"binary31 XXZ Delta=0.7, theta_e ~ U(0.5,1.5), D={D}, random normalised state",
           "energy": E, "site_gradients": {}}
    for prec in precisions:
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        grads = GR.site_gradients(psi, H, precision=prec)
        torch.cuda.synchronize()
        t_sites = time.perf_counter() - t0
        closure = max(abs(ctx.dot(psi.tensors[n], grads[n]) - E) for n in range(topo.nnodes)) / abs(E)
        out["site_gradients"][prec] = {"s": t_sites, "max_rel_closure": closure}
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    g_adj = GR.coupling_gradients_adjoint(psi, H, Hnn, dco)
    torch.cuda.synchronize()
    out["coupling_gradients_adjoint_s"] = time.perf_counter() - t0
    t0 = time.perf_counter()
    g_theta = GR.coupling_gradients(psi, terms)
    torch.cuda.synchronize()
    out["coupling_gradients_expectation_s"] = time.perf_counter() - t0
    out["adjoint_vs_expectation_max_rel"] = max(abs(g_adj[e] - g_theta[e]) / max(1.0, abs(g_theta[e])) for e in theta)
    out["linearity_rel_err"] = abs(sum(theta[e] * g_adj[e] for e in theta) - E) / abs(E)
    h, fd_err = 1e-6, 0.0
    for e in list(topo.edges())[:3]:
        tp, tm = dict(theta), dict(theta)
        tp[e] += h
        tm[e] -= h
        fd = (GR.energy(psi, ttno(tp)).real - GR.energy(psi, ttno(tm)).real) / (2 * h)
        fd_err = max(fd_err, abs(fd - g_adj[e]) / max(1.0, abs(g_adj[e])))
    grads = GR.site_gradients(psi, H)
    for n in [0, topo.nnodes - 1]:
        A = psi.tensors[n]
        Dn = ctx.upload((rng.standard_normal(tuple(A.shape)) + 1j * rng.standard_normal(tuple(A.shape))) / 2)
        pp, pm = psi.copy(), psi.copy()
        pp.tensors[n] = ctx.axpby(h, Dn, 1.0, A.clone())
        pm.tensors[n] = ctx.axpby(-h, Dn, 1.0, A.clone())
        fd = (GR.energy(pp, H).real - GR.energy(pm, H).real) / (2 * h)
        an = 2 * ctx.dot(Dn, grads[n]).real
        fd_err = max(fd_err, abs(fd - an) / max(1.0, abs(an)))
    out["max_fd_rel_err"] = fd_err
    out["fd_sample"] = "3 couplings (h = 1e-6) and 2 site tensors along random directions"
    return out


def run_u1(args):
    """The U(1) block-sparse map alone (see bench_u1)."""
    import grafttn as G
    ctx = G.default_context(0)
    out = {"metric": "U(1) eff_h2 applies/s", "unit": "applies/s"}
    out.update(bench_u1(ctx, args.steps))
    print(json.dumps(out), flush=True)


def run_grad(args):
    """The gradient workload alone at --grad-D (see grad_segment)."""
    import grafttn as G
    ctx = G.default_context(0)
    out = {"metric": "gradient time", "unit": "s", "bond_dim": args.grad_D}
    out.update(grad_segment(ctx, args.grad_D, tuple(args.grad_precisions.split(","))))
    print(json.dumps(out), flush=True)


def run_cbe(args):
    """TDVP1_CBE workload: TFI (-1.0 ZZ, -0.9 X) on the complete 4-ary tree of depth 3
    (85 sites); initial state the one-site DMRG ground state at bond --cbe-maxdim / 2 (the
    two-site blocks of the root edges, D^7 d^2 elements, do not fit for two-site DMRG at
    these bonds) with X applied on one leaf; dz = -0.05i, PredictorCBE(max_add=16) growing
    the bonds up to --cbe-maxdim, maps in --cbe-precision: wall time per step, achieved
    bond dimensions, norm and energy drift."""
    import torch
    import grafttn as G
    from grafttn import gradients as GR
    from grafttn.cbe import TDVP1_CBE, PredictorCBE
    ctx = G.default_context(0)
    topo = G.kary_topology(4, 3)
    H = G.TTNO.from_hamiltonian(G.tfi(topo, J=1.0, g=0.9), ctx)
    psi = G.random_ttns(np.random.default_rng(1), topo, 2, max(1, args.cbe_maxdim // 2), ctx=ctx)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    _, Es = G.dmrg1(psi, H, nsweeps=args.cbe_dmrg_sweeps, precision=args.cbe_precision, lanczos_tol=1e-10)
    dims0 = psi.bond_dims()
    torch.cuda.synchronize()
    t_dmrg = time.perf_counter() - t0
    leaf = topo.nnodes - 1
    X = ctx.upload(G.spin_ops()["X"])
    psi.tensors[leaf] = ctx.contract([psi.tensors[leaf].contiguous(), X], [[1, -2], [-1, 1]])
    E0 = GR.energy(psi, H).real
    ev = TDVP1_CBE(PredictorCBE(max_add=16), maxdim=args.cbe_maxdim, precision=args.cbe_precision)
    times = []
    for _ in range(args.cbe_steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ev.step(psi, H, -0.05j)
        torch.cuda.synchronize()
        times.append(time.perf_counter() - t0)
    E1 = GR.energy(psi, H).real
    dims = psi.bond_dims()
    out = {"metric": "TDVP1_CBE step time", "unit": "s/step", "topology": "kary4_depth3 (85 sites)",
           "model": "TFI -1.0 ZZ -0.9 X", "dz": "-0.05i", "maxdim": args.cbe_maxdim, "precision": args.cbe_precision,
           "dmrg_groundstate": {"sweeps": args.cbe_dmrg_sweeps, "energies": Es, "seconds": t_dmrg},
           "step_s": times, "mean_step_s": float(np.mean(times[1:] if len(times) > 1 else times)),
           "bond_dims_start": {"max": int(max(dims0)), "mean": float(np.mean(dims0))},
           "bond_dims": {"max": int(max(dims)), "mean": float(np.mean(dims))},
           "norm": psi.norm(), "energy_drift_rel": abs(E1 - E0) / abs(E0)}
    print(json.dumps(out), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default=WORKLOAD, choices=sorted(WORKLOADS))
    ap.add_argument("--skip-extra", action="store_true", help="only the headline workload")
    ap.add_argument("--precision", default="fp16x3", choices=sorted(DTYPES), help="mixed mode of the headline map")
    ap.add_argument("--no-dmrg-segment", action="store_true",
                    help="leave out the bounded D=1024 dmrg2 segment (mixed vs FP64) of the default line")
    ap.add_argument("--segment-steps", type=int, default=1)
    ap.add_argument("--tc-tuning", default="measured",
                    choices=["measured", "ladder", "ps128", "ps128x2", "ps256", "pair256", "persist128", "persist256"],
                    help="tile shapes of the tcgen05 steps: timed per problem class (default), the fixed "
                         "ladder, or one variant for every step (fixed launch sequences, for profiler captures)")
    ap.add_argument("--dmrg", action="store_true", help="measure DMRG sweeps instead of map applications")
    ap.add_argument("--dmrg-topology", default="mps", choices=["mps", "binary"])
    ap.add_argument("--dmrg-sites", type=int, default=63)
    ap.add_argument("--dmrg-D", type=int, default=256)
    ap.add_argument("--dmrg-sweeps", type=int, default=2)
    ap.add_argument("--dmrg-precisions", default="bf16x6,fp64")
    ap.add_argument("--svd", action="store_true",
                    help="time one 8192 x 8192 truncated SVD at maxdim 64, subspace route against Gram route")
    ap.add_argument("--lanczos", action="store_true",
                    help="time one mid-chain Lanczos solve of mps63 at --dmrg-D against one map application")
    ap.add_argument("--grad", action="store_true", help="measure the gradient workload (bin31 XXZ)")
    ap.add_argument("--grad-D", type=int, default=128)
    ap.add_argument("--grad-precisions", default="fp64,fp16x3")
    ap.add_argument("--u1", action="store_true",
                    help="measure only the U(1) block-sparse eff_h2 map (bin63-derived block tree, D=1024)")
    ap.add_argument("--cbe", action="store_true", help="measure TDVP1_CBE steps (85-site 4-ary TFI)")
    ap.add_argument("--cbe-maxdim", type=int, default=32)
    ap.add_argument("--cbe-steps", type=int, default=5)
    ap.add_argument("--cbe-dmrg-sweeps", type=int, default=4)
    ap.add_argument("--cbe-precision", default="bf16x6")
    args = ap.parse_args()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        backend = "gloo" if args.impl == "reference" else "nccl"
        if args.impl != "reference":
            import torch
            torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", rank)))
        dist.init_process_group(backend)
    if args.impl != "reference" and args.tc_tuning != "measured":
        from grafttn import _lib as GL
        GL.tc_tuning(args.tc_tuning)
    try:
        if args.dmrg or args.grad or args.cbe or args.lanczos or args.svd or args.u1:
            if rank == 0:
                (run_dmrg if args.dmrg else run_lanczos if args.lanczos else run_svd if args.svd
                 else run_grad if args.grad else run_u1 if args.u1 else run_cbe)(args)
        elif args.impl == "reference":
            run_reference(args, rank, world)
        else:
            run_ours(args, rank, world)
    finally:
        if world > 1:
            import torch.distributed as dist
            dist.destroy_process_group()


if __name__ == "__main__":
    main()
