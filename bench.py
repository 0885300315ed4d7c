#!/usr/bin/env python
"""Benchmark: FEDDLib's element-assembly hot path on GB300.

Default workload: P2-P1 Taylor-Hood Navier-Stokes Newton Jacobian + residual
(rho = 1, nu = 0.01) on the 48^3 x 6 = 663,552-tet unit-cube mesh, velocity =
seeded sum of 8 Fourier modes, pressure uniform[-1, 1] (synthetic, seeded).
One step = one full Jacobian (blocks (0,0), (0,1), (1,0)) + residual
assembly into FP64 CSR values.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--workload NAME]
    python bench.py --impl reference ...   (CPU arm: the FP64 restatement of
                                            the reference's algorithm, all cores)

Prints one JSON line.  Multi-GPU (torchrun): independent replicas, one per
rank; value = elements of all ranks / max over ranks of the timed time.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "elements/s Jacobian+residual into CSR, % HBM roofline; surrogate vs plain law"

WORKLOADS = {
    "ns48": dict(kind="ns", M=48, seed=3,
                 desc="P2-P1 Taylor-Hood Navier-Stokes Newton Jacobian + residual, rho=1, nu=0.01, "
                      "48^3x6 = 663,552 tets, 15-pt (A,N,W) / 5-pt (B) rules"),
    "ns24": dict(kind="ns", M=24, seed=3,
                 desc="P2-P1 Taylor-Hood Navier-Stokes Newton Jacobian + residual, 24^3x6 tets (profiling size)"),
    "nh32": dict(kind="nh", M=32, seed=4,
                 desc="compressible neo-Hooke (skr1) P2 tangent + residual, 32^3x6 tets (profiling size)"),
    "ns64": dict(kind="ns", M=64, seed=3,
                 desc="P2-P1 Taylor-Hood Navier-Stokes Newton Jacobian + residual, 64^3x6 tets"),
    "elas32": dict(kind="elas", M=32, seed=2,
                   desc="P2 linear elasticity stiffness (skr1 at u=0), E=1000, nu=0.3, 32^3x6 tets, 4-pt rule"),
    "nh64": dict(kind="nh", M=64, seed=4,
                 desc="compressible neo-Hooke (skr1) P2 tangent + residual, mu=1, lambda=10, 64^3x6 tets, 4-pt"),
    "aniso64": dict(kind="aniso", M=64, seed=4,
                    desc="two-fibre exponential law (+-40 deg, k1=2, k2=1, skr1 matrix) P2 tangent + residual, "
                         "64^3x6 tets, plain law"),
    "poisson16": dict(kind="poisson", M=16, seed=1,
                      desc="P1 Poisson stiffness + load (f=1), FP64, 16^3x6 tets, 1-pt rule"),
}


def hbm_peak():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


# ------------------------------------------------------------------ clocks --
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1])); smax.append(float(parts[2]))
            except ValueError:
                continue
            for k, nm in enumerate(names):
                if parts[5 + k].lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ----------------------------------------------------------- inputs --------
def make_problem(F, wl, device):
    M, seed, kind = wl["M"], wl["seed"], wl["kind"]
    if kind == "poisson":
        xyz, el = F.structured_mesh(M, 1, seed=seed)
        a = F.Assembler(F.LAPLACE, xyz, el, fe_order=1, source=1.0, device=device)
        return a, dict(xyz=xyz, el=el, u=None, p=None, npe=4, n1=xyz.shape[0])
    xyz2, el2 = F.structured_mesh(M, 2, seed=seed)
    if kind == "ns":
        xyz1, el1 = F.structured_mesh(M, 1, seed=seed)
        u = F.fourier_field(xyz2, seed=seed)
        p = F.uniform_field(seed, xyz1.shape[0])
        a = F.Assembler(F.NAVIER_STOKES, xyz2, el2, elements_p=el1, num_nodes_p=xyz1.shape[0], viscosity=0.01,
                        density=1.0, newton=True, device=device)
        return a, dict(xyz=xyz2, el=el2, el1=el1, u=u, p=p, npe=14, n1=xyz1.shape[0])
    if kind == "elas":
        a = F.Assembler(F.LINEAR_ELASTICITY, xyz2, el2, E=1000.0, poisson_ratio=0.3, device=device)
        return a, dict(xyz=xyz2, el=el2, u=None, p=None, npe=10, n1=(M + 1) ** 3)
    u = F.fourier_field(xyz2, seed=seed, kmin=1, kmax=2, scale=hyper_scale(M))
    prob = F.LINEAR_ELASTICITY if kind == "nh" else F.ANISO_FIBER
    a = F.Assembler(prob, xyz2, el2, E=32.0 / 11.0, poisson_ratio=5.0 / 11.0, k1=2.0, k2=1.0,
                    fiber_angle_deg=40.0, device=device)
    return a, dict(xyz=xyz2, el=el2, u=u, p=None, npe=10, n1=(M + 1) ** 3)


def hyper_scale(M):
    # displacement amplitude that keeps det F in [0.7, 1.4] for the k <= 2
    # field on these meshes (set by the load-step driver's bisection)
    return 0.018


def algorithmic_bytes(a, info, kind):
    """Bytes a step must move at least: FP64 CSR values written once, FP64
    residual written once, int32 connectivity, FP64 vertex coordinates and
    FP64 nodal fields read once."""
    ne = info["el"].shape[0]
    nnz = sum(a.block_info(b)[2] for b in range(a.nblocks))
    res = a.n_u + a.n_p
    fields = 0 if info["u"] is None else 8 * (a.n_u + (a.n_p if info["p"] is not None else 0))
    return 8 * nnz + 8 * res + 4 * info["npe"] * ne + 24 * info["n1"] + fields


def dominant_kernel_bytes(a, kind):
    """Algorithmic bytes of the dominant (row) kernel per launch: the CSR
    values and residual it writes."""
    if kind == "ns":
        return 8 * (a.block_info(0)[2] + a.block_info(1)[2]) + 8 * a.n_u
    return 8 * a.block_info(0)[2] + 8 * a.n_u


# ------------------------------------------------------- CPU baselines ------
def _ref_worker(args):
    M, seed, lo, hi = args
    from oracle import oracle as O
    xyz2, el2, _ = O.mesh(M, 2, seed=seed)
    xyz1, el1, _ = O.mesh(M, 1, seed=seed)
    u = O.field_fourier(xyz2, seed)
    pr = O.field_uniform(seed, xyz1.shape[0])
    t = time.perf_counter()
    O.cpu_baseline_ns(xyz2, el2[lo:hi], el1[lo:hi], u, pr, 0.01, 1.0, xyz1.shape[0])
    return time.perf_counter() - t


def cpu_baseline_single(wl, info):
    """Single-thread reference-shaped FP64 assembly on a bounded sample."""
    from oracle import oracle as O
    ne = info["el"].shape[0]
    sample = min(ne, 60000)
    O.lib()
    t = time.perf_counter()
    O.cpu_baseline_ns(info["xyz"], info["el"][:sample], info["el1"][:sample], info["u"], info["p"], 0.01, 1.0,
                      info["n1"])
    dt = time.perf_counter() - t
    return {"value": sample / dt, "unit": "elements/s", "cores": 1, "kind": "port",
            "sample": f"first {sample:,} of {ne:,} elements of the same mesh and fields; FP64 restatement "
                      "keeping the reference's algorithm shape (per-element table rebuild, heap element matrices, "
                      "per-row insert buffers, sort+merge at fillComplete), Jacobian + residual calls"}


def run_reference(args, wl):
    """--impl reference: the reference's CPU algorithm (oracle port) on all host cores."""
    import multiprocessing as mp
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    if wl["kind"] != "ns":
        print(json.dumps({"impl": "reference", "unavailable": "CPU reference arm implemented for the "
                                                               "Navier-Stokes workload only"}))
        return 0
    cores = os.cpu_count() or 1
    M, seed = wl["M"], wl["seed"]
    ne = 6 * M ** 3
    sample = min(ne, 12000 * cores)
    chunks = [(M, seed, k * sample // cores, (k + 1) * sample // cores) for k in range(cores)]
    ctx = mp.get_context("spawn")
    times = []
    with ctx.Pool(cores) as pool:
        for it in range(args.warmup + args.steps):
            t0 = time.perf_counter()
            pool.map(_ref_worker, chunks)
            dt = time.perf_counter() - t0
            if it >= args.warmup:
                times.append(dt)
    total = sum(times)
    value = sample * len(times) / total
    out = {"impl": "reference", "metric": METRIC, "value": value, "unit": "elements/s", "n_gpus": 0,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / len(times),
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
           "config": {"workload": args.workload, "desc": wl["desc"], "sample_elements_per_step": sample},
           "cpu_baseline": {"value": value, "unit": "elements/s", "cores": cores, "kind": "port",
                            "sample": f"{sample:,} of {ne:,} elements per step, split over {cores} processes "
                                      "(one element range each, as FEDDLib's MPI ranks do); FP64 restatement "
                                      "of the reference's algorithm incl. per-row inserts and fillComplete"},
           "e2e": {"value": value, "unit": "elements/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out))
    return 0


# ----------------------------------------------------------------- main -----
def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--workload", default="ns48", choices=sorted(WORKLOADS))
    ap.add_argument("--impl", default="engine", choices=["engine", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--e2e-steps", type=int, default=3)
    args = ap.parse_args()
    wl = WORKLOADS[args.workload]
    if args.impl == "reference":
        return run_reference(args, wl)
    if args.warmup < 3:
        args.warmup = 3

    import numpy as np
    import torch
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    import feddlib_gb300 as F

    dev = torch.device(f"cuda:{local}")
    a, info = make_problem(F, wl, local)
    kind = wl["kind"]
    ne = info["el"].shape[0]
    nb = a.nblocks
    d_u = None if info["u"] is None else torch.from_numpy(info["u"]).to(dev)
    d_p = None if info["p"] is None else torch.from_numpy(info["p"]).to(dev)
    d_vals = [torch.empty(max(a.block_info(b)[2], 1), dtype=torch.float64, device=dev) for b in range(nb)]
    d_ru = torch.empty(a.n_u, dtype=torch.float64, device=dev)
    d_rp = torch.empty(max(a.n_p, 1), dtype=torch.float64, device=dev) if a.n_p else None
    stream = torch.cuda.current_stream(dev)
    sptr = stream.cuda_stream
    want_res = kind != "elas"
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)  # 256 MiB > 126 MB L2

    def step():
        a.assemble_device(None if d_u is None else d_u.data_ptr(), None if d_p is None else d_p.data_ptr(),
                          [v.data_ptr() for v in d_vals], d_ru.data_ptr(), None if d_rp is None else d_rp.data_ptr(),
                          jacobian=True, residual=want_res, stream=sptr)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize(dev)
    a.check(sptr)

    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    a.set_profiling(True)
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    if dist:
        dist.barrier()
    torch.cuda.synchronize(dev)
    wall0 = time.perf_counter()
    for k in range(args.steps):
        flush.fill_(float(k))  # evict L2 between timed steps (outside the events)
        starts[k].record(stream)
        step()
        ends[k].record(stream)
    torch.cuda.synchronize(dev)
    if dist:
        dist.barrier()
    wall = time.perf_counter() - wall0
    stage_ms = a.stage_times()
    a.set_profiling(False)
    clk = clocks.stop()
    a.check(sptr)
    step_ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    total_s = sum(step_ms) / 1e3
    if dist:
        t = torch.tensor([total_s], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_s = float(t.item())
    launches = a.launch_count() * args.steps
    value = world * ne * args.steps / total_s
    peak, peak_kind = hbm_peak()
    alg = algorithmic_bytes(a, info, kind)
    # dominant kernel: the longest stage
    dom_name, (dom_ms_total, dom_calls) = max(stage_ms.items(), key=lambda kv: kv[1][0])
    dom_ms = dom_ms_total / max(dom_calls, 1)
    dom_bytes = dominant_kernel_bytes(a, kind)
    achieved = dom_bytes / (dom_ms * 1e-3) / 1e9
    traffic = None
    tpath = os.path.join(ROOT, "profiles", "dram_traffic.json")
    if os.path.exists(tpath):
        try:
            traffic = json.load(open(tpath)).get(args.workload, {}).get(dom_name)
        except Exception:
            traffic = None

    # end to end through the C ABI with host buffers (pinned), copies timed
    e2e = None
    if rank == 0 or world > 1:
        h_u = None if info["u"] is None else torch.from_numpy(info["u"]).pin_memory()
        h_p = None if info["p"] is None else torch.from_numpy(info["p"]).pin_memory()
        h_vals = [torch.empty(max(a.block_info(b)[2], 1), dtype=torch.float64).pin_memory() for b in range(nb)]
        h_ru = torch.empty(a.n_u, dtype=torch.float64).pin_memory()
        h_rp = torch.empty(max(a.n_p, 1), dtype=torch.float64).pin_memory() if a.n_p else None
        import ctypes as C
        from feddlib_gb300 import _capi as A

        def host_step():
            what = A.JACOBIAN | (A.RESIDUAL if want_res else 0)
            v = [t.data_ptr() for t in h_vals] + [None] * (3 - nb)
            A.check(A.lib().fedd_assemble(a.h, what, None if h_u is None else h_u.data_ptr(),
                                          None if h_p is None else h_p.data_ptr(), v[0], v[1], v[2],
                                          h_ru.data_ptr() if want_res else None,
                                          None if (h_rp is None or not want_res) else h_rp.data_ptr(), sptr), a.h)
        host_step()
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        for _ in range(args.e2e_steps):
            host_step()
        e2e_s = (time.perf_counter() - t0) / args.e2e_steps
        h2d = 0 if h_u is None else 8 * (a.n_u + (a.n_p if h_p is not None else 0))
        d2h = 8 * sum(a.block_info(b)[2] for b in range(nb)) + (8 * (a.n_u + a.n_p) if want_res else 0)
        e2e = {"value": world * ne / e2e_s, "unit": "elements/s", "h2d_bytes_per_step": h2d,
               "d2h_bytes_per_step": d2h, "ms_per_step": 1e3 * e2e_s,
               "note": "fedd_assemble with pinned host buffers: H2D of u,p, kernels, D2H of all CSR values "
                       "and residuals, synchronised, per step"}

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline and kind == "ns":
        cpu = cpu_baseline_single(wl, info)

    out = {
        "metric": METRIC, "value": value, "unit": "elements/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * total_s / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "fp32 element math, fp64 geometry + CSR values",
        "data": "synthetic (seeded mesh jitter and fields)",
        "config": {"workload": args.workload, "desc": wl["desc"], "elements": ne,
                   "nnz": [a.block_info(b)[2] for b in range(nb)], "rows": [a.block_info(b)[0] for b in range(nb)],
                   "parallelism": f"replicas x{world}" if world > 1 else "1 GPU",
                   "l2": "256 MiB buffer written between timed steps (outside the step events); each step also "
                         "writes > 1 GB", "algorithmic_bytes_per_element": alg / ne,
                   "wall_s_timed_region": wall},
        "step_roofline": {"bound": "hbm", "achieved": alg * args.steps / total_s / 1e9, "peak": peak,
                          "unit": "GB/s", "frac": alg * args.steps / total_s / 1e9 / peak,
                          "peak_source": f"MEASURED_PEAKS.json hbm_gbs ({peak_kind})"},
        "roofline": {"bound": "hbm", "kernel": dom_name, "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic, "bytes_per_launch": dom_bytes,
                     "ms_per_launch": dom_ms, "peak_source": f"MEASURED_PEAKS.json hbm_gbs ({peak_kind})"},
        "stages_ms": {k: v[0] / max(v[1], 1) for k, v in stage_ms.items()},
        "gpu_launches": launches,
        "clocks": clk,
        "e2e": e2e,
        "cpu_baseline": cpu,
    }
    if rank == 0:
        print(json.dumps(out))
    if dist:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
