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
    "gn48": dict(kind="gn", M=48, seed=3,
                 desc="generalized-Newtonian (Carreau-Yasuda, FEDDLib's blood parameters: lambda 1.902, n 0.22, "
                      "eta0 0.056, etaInf 0.00345, a 1.25) P2-P1 Navier-Stokes Newton Jacobian + residual, rho=1, "
                      "48^3x6 tets, same mesh and fields as ns48"),
    "gn24": dict(kind="gn", M=24, seed=3,
                 desc="generalized-Newtonian (Carreau-Yasuda) Navier-Stokes, 24^3x6 tets (profiling size of gn48)"),
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
    "aniso64s": dict(kind="aniso_surr", M=64, seed=4,
                     desc="two-fibre law through the MLP surrogate (invariants->64->64->Psi_fib, softplus, bf16 "
                          "weights, tensor cores) trained by the engine's kernels on 2M quadrature-point samples of "
                          "10 load steps of the plain law; P2 tangent + residual, 64^3x6 tets, 4-pt; plain law timed "
                          "beside it on the same GPU"),
    "aniso32s": dict(kind="aniso_surr", M=32, seed=4,
                     desc="two-fibre law through the MLP surrogate, 32^3x6 tets (profiling size of aniso64s)"),
    "poisson16": dict(kind="poisson", M=16, seed=1,
                      desc="P1 Poisson stiffness + load (f=1), FP64, 16^3x6 tets, 1-pt rule"),
}


# Carreau-Yasuda with FEDDLib's blood parameters (lambda, n, eta0, etaInf, a), shear-rate floor
GN_LAW = (0, [1.902, 0.22, 0.056, 0.00345, 1.25], 1e-12)


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
    if kind in ("ns", "gn"):
        xyz1, el1 = F.structured_mesh(M, 1, seed=seed)
        u = F.fourier_field(xyz2, seed=seed)
        p = F.uniform_field(seed, xyz1.shape[0])
        a = F.Assembler(F.NAVIER_STOKES, xyz2, el2, elements_p=el1, num_nodes_p=xyz1.shape[0], viscosity=0.01,
                        density=1.0, newton=True, device=device)
        if kind == "gn":
            a.set_viscosity_law(GN_LAW[0], GN_LAW[1], gamma_min=GN_LAW[2])
        return a, dict(xyz=xyz2, el=el2, el1=el1, u=u, p=p, npe=14, n1=xyz1.shape[0], gn=kind == "gn")
    if kind == "elas":
        a = F.Assembler(F.LINEAR_ELASTICITY, xyz2, el2, E=1000.0, poisson_ratio=0.3, device=device)
        return a, dict(xyz=xyz2, el=el2, u=None, p=None, npe=10, n1=(M + 1) ** 3)
    prob = F.LINEAR_ELASTICITY if kind == "nh" else F.ANISO_FIBER
    kw = dict(E=32.0 / 11.0, poisson_ratio=5.0 / 11.0, k1=2.0, k2=1.0, fiber_angle_deg=40.0, device=device)
    a = F.Assembler(prob, xyz2, el2, **kw)
    u, scale, jrange = F.detF_scaled_field(a, xyz2, seed)
    info = dict(xyz=xyz2, el=el2, u=u, p=None, npe=10, n1=(M + 1) ** 3,
                field={"amplitude": scale, "detF_min": jrange[0], "detF_max": jrange[1],
                       "rule": "largest amplitude of the seeded k<=2 Fourier field with det F in [0.7, 1.4] at "
                               "every quadrature point (bisection)"})
    if kind == "aniso_surr":
        from feddlib_gb300.surrogate import law_samples, train_surrogate
        t0 = time.perf_counter()
        # training data from the plain law's own kernel at the quadrature points
        # of 10 load steps; the neo-Hooke matrix law (evaluated on a one-element
        # handle: law evaluation needs no mesh) is subtracted
        x1, e1 = F.structured_mesh(1, 2, seed=0)
        mat = F.Assembler(F.LINEAR_ELASTICITY, x1, e1, E=kw["E"], poisson_ratio=kw["poisson_ratio"],
                          device=device)
        inv, psi_f, g_f = law_samples(a, mat, [u * (l / 10) for l in range(1, 11)], n_samples=2_000_000, seed=seed)
        mat.close()
        t1 = time.perf_counter()
        model, rep = train_surrogate(inv, hidden=64, steps=3000, batch=65536, lr=3e-3, lr_final=3e-5,
                                     device=device, targets=(psi_f, g_f))
        surr = F.Assembler(prob, xyz2, el2, surrogate=True, **kw)
        surr.set_surrogate(model, inv_lo=model["inv_lo"], inv_hi=model["inv_hi"])
        info.update(plain=a, model=model, sampling_s=t1 - t0, train=rep)
        a = surr
    return a, info


def algorithmic_bytes(a, info, kind):
    """Bytes a step must move at least: FP64 CSR values written once, FP64
    residual written once, int32 connectivity, FP64 vertex coordinates and
    FP64 nodal fields read once."""
    ne = info["el"].shape[0]
    nnz = sum(a.block_info(b)[2] for b in range(a.nblocks))
    res = a.n_u + a.n_p
    fields = 0 if info["u"] is None else 8 * (a.n_u + (a.n_p if info["p"] is not None else 0))
    return 8 * nnz + 8 * res + 4 * info["npe"] * ne + 24 * info["n1"] + fields


def stage_work(a, info, name):
    """Algorithmic work of one launch of stage `name`: ("hbm", bytes) or
    ("tensor", flops).  Row stages: the FP64 CSR values and residual they
    write once.  Element stages: the stage record they write plus
    connectivity, vertex coordinates and nodal fields read once.  MLP stage:
    the layer-2 contractions on the tensor cores per quadrature point: the
    forward product for 1 + NA channels (NA = inputs with a non-zero scale)
    and the backward product W2^T (w3 * s2), 64 x 64 MACs each, on the bf16 hi
    and lo halves of the activations."""
    ne = info["el"].shape[0]
    nb = lambda b: a.block_info(b)[2]
    fields = 0 if info["u"] is None else 8 * a.n_u
    geo = 4 * info["npe"] * ne + 24 * info["n1"]
    if name == "ns_vel_rows":
        # with the pressure rows assembled by the vertices' velocity-row warps
        # (no separate pressure-row stage) the launch also writes block (1,0)
        # and the pressure residual; a generalized-Newtonian fluid's viscous
        # stage rows are folded in, so that launch also reads them (three
        # padded rows per incidence, 10 incidences per element)
        fused = 8 * nb(2) + 8 * a.n_p if info.get("pressure_rows_fused") else 0
        gn = 10 * 3 * 32 * 4 * ne if info.get("gn") else 0
        return "hbm", 8 * (nb(0) + nb(1)) + 8 * a.n_u + fused + gn
    if name == "ns_pres_rows":
        return "hbm", 8 * nb(2) + 8 * a.n_p
    if name in ("hyper_rows", "lap_rows"):
        return "hbm", 8 * nb(0) + 8 * a.n_u
    if name == "ns_record":
        return "hbm", 512 * ne + geo + fields + 8 * a.n_p
    if name == "hyper_elem":
        return "hbm", 1984 * ne + geo + fields
    if name == "lap_elem":
        return "hbm", 8 * (16 if info["npe"] == 4 else 72) * ne + geo
    if name == "qp_invariants":
        return "hbm", 16 * 4 * ne + geo + fields
    if name == "gn_elem":
        return "hbm", 4 * 932 * ne + geo + fields
    if name == "mlp_qp":
        na = int(sum(1 for v in info["model"]["in_scale"] if v != 0)) if "model" in info else 4
        return "tensor", 2.0 * (1 + na + 1) * 64 * 64 * 2 * 4 * ne
    return "hbm", 0


# ------------------------------------------------------- CPU baselines ------
# The reference's own CPU assembly needs Trilinos, MPI, Boost, HDF5 and
# gfortran and cannot run on this machine; both CPU legs time the oracle's
# reference-shaped FP64 port of the same path (per-element table rebuild,
# heap element matrices, per-row inserts, sort + merge at fillComplete; the
# elasticity port calls the element kernel twice per element when it also
# assembles the residual, as AssembleFE_NonLinElas does).

def _law_spec(O, kind):
    """The oracle law of a workload (E and nu as the engine takes them)."""
    if kind == "elas":
        return O.law_from_E_nu(O.LAW_SKR1, 1000.0, 0.3), 4
    if kind == "nh":
        return O.law_from_E_nu(O.LAW_SKR1, 32.0 / 11.0, 5.0 / 11.0), 4
    return O.LawSpec(O.LAW_ANISO, mu=1.0, lam=10.0, k1=2.0, k2=1.0, angle_deg=40.0), 4


def _port_run(O, kind, xyz, el, el1, u, p, n1):
    """One call of the reference-shaped port over the given elements."""
    if kind in ("ns", "gn"):
        return O.cpu_baseline_ns(xyz, el, el1, u, p, 0.01, 1.0, n1)
    if kind == "poisson":
        rp, ci, v = O.assemble_laplace(1, 1, xyz, el)
        return float(v.sum())
    L, npts = _law_spec(O, kind)
    return O.cpu_baseline_vec(L, npts, xyz, el, u, u is not None)


def cpu_baseline_single(kind, info, sample):
    """Single-thread reference-shaped FP64 port on a bounded sample of the
    workload (the first `sample` elements of the same mesh and fields)."""
    from oracle import oracle as O
    O.lib()
    el = info["el"]
    ne = el.shape[0]
    n = min(ne, sample) if kind != "poisson" else ne
    t = time.perf_counter()
    _port_run(O, kind, info["xyz"], el[:n], None if info.get("el1") is None else info["el1"][:n], info["u"],
              info["p"], info["n1"])
    dt = time.perf_counter() - t
    what = {"ns": "Jacobian + residual calls", "gn": "Jacobian + residual calls (Newtonian port)",
            "poisson": "COO assembly + Tpetra-semantics merge of the whole mesh",
            "elas": "one kernel call per element (Jacobian only)",
            "nh": "two kernel calls per element (Jacobian, residual)",
            "aniso": "two kernel calls per element (Jacobian, residual)",
            "aniso_surr": "two kernel calls per element of the plain law (the reference has no surrogate)"}[kind]
    return {"value": n / dt, "unit": "elements/s", "cores": 1, "kind": "port",
            "sample": f"first {n:,} of {ne:,} elements of the same mesh and fields; FP64 port keeping the "
                      f"reference's algorithm shape (per-element work, heap element matrices, per-row insert "
                      f"buffers, sort+merge at fillComplete); {what}"}


# reference arm workers: the mesh and fields are built once per process (pool
# initialiser), each task times only its own assembly call
_REF = {}


def _ref_init(M, seed, kind, scale):
    from oracle import oracle as O
    O.lib()
    if kind == "poisson":
        xyz, el, _ = O.mesh(M, 1, seed=seed)
        _REF.update(kind=kind, xyz=xyz, el=el, el1=None, u=None, p=None, n1=xyz.shape[0])
        return
    xyz2, el2, _ = O.mesh(M, 2, seed=seed)
    st = dict(kind=kind, xyz=xyz2, el=el2, el1=None, u=None, p=None, n1=0)
    if kind in ("ns", "gn"):
        xyz1, el1, _ = O.mesh(M, 1, seed=seed)
        st.update(el1=el1, u=O.field_fourier(xyz2, seed), p=O.field_uniform(seed, xyz1.shape[0]), n1=xyz1.shape[0])
    elif kind != "elas":
        st.update(u=O.field_fourier(xyz2, seed, kmin=1, kmax=2, scale=scale))
    _REF.update(st)


def _ref_detF(args):
    """det F range of elements [lo, hi) at amplitude s (the pool's field is the unit one)."""
    s, lo, hi = args
    from oracle import oracle as O
    return O.detF_range(4, _REF["xyz"], _REF["el"][lo:hi], _REF["u"] * s)


def _ref_work(args):
    lo, hi = args
    from oracle import oracle as O
    r = _REF
    t = time.perf_counter()
    _port_run(O, r["kind"], r["xyz"], r["el"][lo:hi], None if r["el1"] is None else r["el1"][lo:hi], r["u"], r["p"],
              r["n1"])
    return time.perf_counter() - t


def _ref_scale(ctx, cores, M, seed, kind, lo_j=0.7, hi_j=1.4, iters=24):
    """The hyperelastic field amplitude by bisection on the oracle's FP64 det F
    over all quadrature points (element ranges spread over the host cores)."""
    ne = 6 * M ** 3
    chunks = [(k * ne // cores, (k + 1) * ne // cores) for k in range(cores)]
    with ctx.Pool(cores, initializer=_ref_init, initargs=(M, seed, kind, 1.0)) as pool:
        def jr(s):
            rs = pool.map(_ref_detF, [(s, lo, hi) for lo, hi in chunks])
            return min(r[0] for r in rs), max(r[1] for r in rs)
        lo, hi = 0.0, 1e-3
        while True:
            jmin, jmax = jr(hi)
            if jmin < lo_j or jmax > hi_j:
                break
            lo, hi = hi, 2 * hi
        for _ in range(iters):
            mid = 0.5 * (lo + hi)
            jmin, jmax = jr(mid)
            if jmin < lo_j or jmax > hi_j:
                hi = mid
            else:
                lo = mid
    return lo


def run_reference(args, wl):
    """--impl reference: the reference-shaped FP64 port of the path on all
    host cores, one element range per process as FEDDLib's MPI ranks take
    them; each step is a bounded sample of the workload's elements, and the
    step time is the slowest process's own assembly time."""
    import multiprocessing as mp
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    cores = os.cpu_count() or 1
    M, seed, kind = wl["M"], wl["seed"], wl["kind"]
    port_kind = {"gn": "ns", "aniso_surr": "aniso"}.get(kind, kind)
    ne = 6 * M ** 3
    per_core = {"ns": 12000, "elas": 24000, "nh": 12000, "aniso": 12000, "poisson": ne}[port_kind]
    sample = min(ne, per_core * cores) if port_kind != "poisson" else ne
    ctx = mp.get_context("spawn")
    scale = _ref_scale(ctx, cores, M, seed, port_kind) if port_kind in ("nh", "aniso") else 1.0
    if port_kind == "poisson":
        chunks, procs = [(0, ne)], 1
    else:
        chunks, procs = [(k * sample // cores, (k + 1) * sample // cores) for k in range(cores)], cores
    times = []
    with ctx.Pool(procs, initializer=_ref_init, initargs=(M, seed, port_kind, scale)) as pool:
        for it in range(args.warmup + args.steps):
            worker_s = pool.map(_ref_work, chunks)
            if it >= args.warmup:
                times.append(max(worker_s))
    total = sum(times)
    value = sample * len(times) / total
    what = {"ns": "Navier-Stokes Jacobian + residual", "elas": "linear elasticity Jacobian (skr1 at u = 0)",
            "nh": "neo-Hooke (skr1) Jacobian + residual, two kernel calls per element",
            "aniso": "plain two-fibre law Jacobian + residual, two kernel calls per element",
            "poisson": "P1 Laplace stiffness (COO + Tpetra-semantics merge)"}[port_kind]
    out = {"impl": "reference", "metric": METRIC, "value": value, "unit": "elements/s", "n_gpus": 0,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / len(times),
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
           "config": {"workload": args.workload, "desc": wl["desc"], "sample_elements_per_step": sample,
                      **({"field_amplitude": scale} if port_kind in ("nh", "aniso") else {})},
           "cpu_baseline": {"value": value, "unit": "elements/s", "cores": procs, "kind": "port",
                            "sample": f"{sample:,} of {ne:,} elements per step, split over {procs} processes "
                                      f"(one element range each, as FEDDLib's MPI ranks do); FP64 restatement of "
                                      f"the reference's algorithm ({what}) incl. per-row inserts and "
                                      f"fillComplete; step time = slowest process's own assembly time, mesh and "
                                      f"fields built once per process outside it"},
           "e2e": {"value": value, "unit": "elements/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out))
    return 0


# --------------------------------------------------------------- parity ------
def parity_report(a, info, kind, d_vals, d_ru, d_rp, frac, seed):
    """The checker (oracle, FP64) against the engine's output of the timed
    step: complete rows of a seeded sample of the row nodes rebuilt by the
    oracle from all of their incident elements, relative Frobenius error per
    block (the whole mesh for the small Poisson case)."""
    import numpy as np
    from oracle import oracle as O
    from oracle import parity as P
    vals = [v.cpu().numpy() for v in d_vals]
    ru = d_ru.cpu().numpy() if d_ru is not None else None
    rp = d_rp.cpu().numpy() if d_rp is not None else None
    xyz, el = info["xyz"], info["el"]
    if kind == "poisson":
        orp, oci, ov = O.assemble_laplace(1, 1, xyz, el)
        rp0, ci0, _ = a.pattern(0)
        ob = O.assemble_rhs(1, 1, xyz, el, 1.0)
        return {"pattern_equal": bool(np.array_equal(rp0, orp) and np.array_equal(ci0, oci)),
                "00": float(np.linalg.norm(vals[0][:len(ov)] - ov) / np.linalg.norm(ov)),
                "load": float(np.linalg.norm(ru - ob) / np.linalg.norm(ob)), "rows": "all",
                "tolerance": 1e-12}
    nn = xyz.shape[0]
    if kind in ("ns", "gn"):
        xyz1n = info["n1"]
        inc2 = P.node_elements(el, nn)
        inc1 = P.node_elements(info["el1"], xyz1n)
        vsel = P.sample_nodes(nn, frac, seed=seed)
        psel = P.sample_nodes(xyz1n, frac, seed=seed + 1)
        csr = []
        for b in range(3):
            rpt, ci, _ = a.pattern(b)
            csr.append((rpt, ci, vals[b]))
        law = O.visc_law(GN_LAW[0], GN_LAW[1], GN_LAW[2]) if kind == "gn" else None
        o = P.rows_ns(xyz, el, info["el1"], info["u"], info["p"], 0.01, 1.0, True, inc2, inc1, vsel, psel, law=law)
        out = P.compare_ns(csr, ru, rp, o, vsel, psel)
    else:
        L, npts = _law_spec(O, kind)
        inc = P.node_elements(el, nn)
        sel = P.sample_nodes(nn, frac, seed=seed)
        rpt, ci, _ = a.pattern(0)
        e = P.compare_vec(rpt, ci, vals[0], ru if info["u"] is not None else None,
                          P.rows_vec(1, L, npts, xyz, el, info["u"], inc, sel), sel)
        out = {"00": e["block"], "res_u": e["residual"], "rows_u": e["rows"]}
    out["sample"] = f"complete rows of a seeded {frac:.1%} of the row nodes (and of the pressure nodes)"
    out["tolerance"] = {"blocks": 1e-6, "residuals": 1e-5}
    return out


# ----------------------------------------------------------- Dirichlet -----
def dirichlet_report(a, info, d_vals, d_ru, d_rp, stream, reps=10):
    """Times BCBuilder::setSystem + setRHS on the device (fedd_dirichlet_*)
    with every dof of the cube's boundary nodes Dirichlet, on the step's own
    output buffers.  Algorithmic bytes: the Dirichlet rows' values written
    and column indices read in every block of their block row, their row
    pointers, and the right-hand side entries written."""
    import numpy as np
    import torch
    xyz = info["xyz"]
    bnd = ((np.abs(xyz) < 1e-12) | (np.abs(xyz - 1.0) < 1e-12)).any(axis=1)
    mask = np.repeat(bnd, 3).astype(np.uint8)
    a.set_dirichlet(mask)
    rows = np.nonzero(mask)[0]
    nb = len(d_vals)
    nnz_rows = 0
    for b in range(min(nb, 2)):
        rp, _, _ = a.pattern(b)
        nnz_rows += int((rp[rows + 1] - rp[rows]).sum())
    alg = 12 * nnz_rows + 16 * len(rows) * min(nb, 2) + 8 * len(rows)
    ptrs = [v.data_ptr() for v in d_vals]
    sptr = stream.cuda_stream
    for _ in range(3):
        a.dirichlet_system_device(ptrs, stream=sptr)
        a.dirichlet_rhs_device(d_ru.data_ptr(), stream=sptr)
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for _ in range(reps):
        a.dirichlet_system_device(ptrs, stream=sptr)
        a.dirichlet_rhs_device(d_ru.data_ptr(), stream=sptr)
    ev1.record(stream)
    torch.cuda.synchronize()
    a.check(sptr)
    ms = ev0.elapsed_time(ev1) / reps
    peak, _ = hbm_peak()
    return {"rows": int(len(rows)), "row_entries": nnz_rows, "ms": ms, "bytes": alg,
            "achieved_gbs": alg / (ms * 1e-3) / 1e9, "frac_of_hbm": alg / (ms * 1e-3) / 1e9 / peak,
            "what": "BCBuilder::setSystem + setRHS on the device, all dofs of the cube's boundary nodes"}


def frontend_report(F, wl, info, kind, reps=3):
    """The mesh front end at the workload's size: the structured P2 (+P1)
    mesh made on the device against the host generator, the P2 mesh of the
    P1 mesh built on the device (buildP2ofP1MeshEdge), and the assembler's
    setup (node graph, CSR patterns, vertex map) from a device-resident mesh
    against host arrays.  Wall time around each synchronising call, best of
    `reps`; one-time costs per mesh, outside the step."""
    import numpy as np
    import torch
    M, seed = wl["M"], wl["seed"]
    ne = 6 * M ** 3
    best = lambda f: min(f() for _ in range(reps))

    def timed(fn):
        def run():
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            fn()
            torch.cuda.synchronize()
            return time.perf_counter() - t0
        return run
    out = {"elements": ne}
    out["structured_device_s"] = best(timed(lambda: F.structured_mesh_device(M, 2, seed=seed)))
    out["structured_host_s"] = best(timed(lambda: F.structured_mesh(M, 2, seed=seed)))
    x1d, e1d = F.structured_mesh_device(M, 1, seed=seed)
    out["p2_of_p1_device_s"] = best(timed(lambda: F.p2_of_p1(x1d, e1d)))
    if kind in ("ns", "gn"):
        x2d, e2d = F.structured_mesh_device(M, 2, seed=seed)
        kw = dict(elements_p=e1d, num_nodes_p=x1d.shape[0], viscosity=0.01, density=1.0, newton=True)
        out["setup_device_mesh_s"] = best(timed(lambda: F.Assembler(F.NAVIER_STOKES, x2d, e2d, **kw).close()))
        kw["elements_p"] = info["el1"]
        out["setup_host_mesh_s"] = best(timed(lambda: F.Assembler(F.NAVIER_STOKES, info["xyz"], info["el"],
                                                                   **kw).close()))
        del x2d, e2d
    del x1d, e1d
    torch.cuda.empty_cache()
    out["structured_device_elements_per_s"] = ne / out["structured_device_s"]
    out["what"] = ("one-time mesh front end at the workload's size: device vs host structured generator, "
                   "device P2-of-P1, assembler setup (graph + CSR + vertex map) from device vs host arrays")
    return out


# ------------------------------------------------------ surrogate vs plain --
def surrogate_report(F, surr, info, d_u, d_vals, d_ru, stream, flush, steps, surr_stage_ms):
    """Times the plain two-fibre law on the same mesh, field and buffers as the
    surrogate step just timed, and measures the surrogate against it: stress
    and tangent errors at quadrature points of the load steps, fallback rate,
    tensor-core throughput of the MLP stage, and Newton iteration counts on a
    small load-stepping problem (both laws, same driver)."""
    import numpy as np
    import torch
    from feddlib_gb300.newton import solve_load_steps
    from feddlib_gb300.surrogate import law_samples, sample_F, stress_tangent_errors, train_surrogate
    plain = info["plain"]
    sptr = stream.cuda_stream

    def run(asm):
        asm.assemble_device(d_u.data_ptr(), None, [v.data_ptr() for v in d_vals], d_ru.data_ptr(), None,
                            jacobian=True, residual=True, stream=sptr)

    for _ in range(3):
        run(plain)
    torch.cuda.synchronize()
    plain.set_profiling(True)
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    for k in range(steps):
        flush.fill_(float(k))
        ev[k][0].record(stream)
        run(plain)
        ev[k][1].record(stream)
    torch.cuda.synchronize()
    plain_stages = {k: v[0] / max(v[1], 1) for k, v in plain.stage_times().items()}
    plain.set_profiling(False)
    plain.check(sptr)
    plain_ms = sum(s.elapsed_time(e) for s, e in ev) / steps
    surr_stages = {k: v[0] / max(v[1], 1) for k, v in surr_stage_ms.items()}
    surr_ms = sum(surr_stages.values())
    fb, tot = surr.surrogate_fallbacks()
    u = info["u"]
    Fs = np.concatenate([sample_F(plain, u * (l / 10), 400, seed=l) for l in (4, 7, 10)])
    err = stress_tangent_errors(plain, surr, Fs)
    _, tc_flops = stage_work(surr, info, "mlp_qp")
    mlp_ms = surr_stages.get("mlp_qp")
    # Newton iteration counts: the same workflow on a small mesh (train on the
    # plain law's own iterates, then solve with each law)
    xyz, el = F.structured_mesh(3, 2, seed=4)
    kw = dict(E=32.0 / 11.0, poisson_ratio=5.0 / 11.0, k1=2.0, k2=1.0, fiber_angle_deg=40.0)
    sp = F.Assembler(F.ANISO_FIBER, xyz, el, **kw)
    states = []
    _, its_p4, _ = solve_load_steps(sp, xyz, stretch=0.12, steps=4, tol=1e-4,
                                    on_iterate=lambda s, it, uu: states.append(uu))
    mat = F.Assembler(F.LINEAR_ELASTICITY, xyz, el, E=kw["E"], poisson_ratio=kw["poisson_ratio"])
    inv_s, psi_s, g_s = law_samples(sp, mat, states, n_samples=200000)
    mat.close()
    m_small, _ = train_surrogate(inv_s, hidden=64, steps=4000, batch=16384, lr=3e-3, lr_final=3e-5,
                                 targets=(psi_s, g_s))
    ss = F.Assembler(F.ANISO_FIBER, xyz, el, surrogate=True, **kw)
    ss.set_surrogate(m_small, inv_lo=m_small["inv_lo"], inv_hi=m_small["inv_hi"])
    _, its_s4, _ = solve_load_steps(ss, xyz, stretch=0.12, steps=4, tol=1e-4)
    _, its_p5, _ = solve_load_steps(sp, xyz, stretch=0.12, steps=4, tol=1e-5)
    _, its_s5, _ = solve_load_steps(ss, xyz, stretch=0.12, steps=4, tol=1e-5)
    rep = info["train"]
    return {"plain_ms_per_step": plain_ms, "surrogate_ms_per_step": surr_ms,
            "speedup_vs_plain": plain_ms / surr_ms, "plain_stages_ms": plain_stages, "surrogate_stages_ms": surr_stages,
            "stress_rel_fro": err["stress_rel_fro"], "stress_rel_max": err["stress_rel_max"],
            "tangent_rel_fro": err["tangent_rel_fro"], "error_sample": f"{len(Fs)} quadrature points of load steps "
                                                                        "4, 7, 10 of the workload's deformation",
            "fallbacks": fb, "quadrature_points": tot, "fallback_rate": fb / max(tot, 1),
            "mlp_qp_tensor": {"flops_per_launch": tc_flops, "ms": mlp_ms,
                              "achieved_tflops": None if not mlp_ms else tc_flops / (mlp_ms * 1e-3) / 1e12,
                              "peak_tflops": bf16_peak(), "frac": None if not mlp_ms else
                              tc_flops / (mlp_ms * 1e-3) / 1e12 / bf16_peak()},
            "training": {"samples": rep["samples"], "steps": rep["steps"], "batch": rep["batch"],
                         "seconds": rep["seconds"], "sampling_seconds": info["sampling_s"],
                         "loss_first": rep["loss_history"][0], "loss_last": rep["loss_history"][-1]},
            "newton_iterations": {"problem": "M=3 P2 box, x=0 clamped, x=1 pulled to 12 % in 4 load steps; "
                                             "surrogate trained on the plain law's iterates",
                                  "tol_1e-4": {"plain": its_p4, "surrogate": its_s4},
                                  "tol_1e-5": {"plain": its_p5, "surrogate": its_s5}}}


def stage_frac(a, info, name, ms, hbm):
    bound, work = stage_work(a, info, name)
    if not ms or not work:
        return None
    if bound == "tensor":
        return {"bound": "tensor", "tflops": work / (ms * 1e-3) / 1e12, "frac": work / (ms * 1e-3) / 1e12 / bf16_peak()}
    return {"bound": "hbm", "gbs": work / (ms * 1e-3) / 1e9, "frac": work / (ms * 1e-3) / 1e9 / hbm}


def bf16_peak():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["bf16_tflops"])
    except Exception:
        return 1900.0


# ------------------------------------------------------------- ranks --------
def max_over_ranks(seconds, dist=None, device="cpu"):
    """The timed seconds of the slowest rank (every rank gets the value)."""
    if dist is None:
        return float(seconds)
    import torch
    t = torch.tensor([float(seconds)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_rate(world, units_per_rank, seconds):
    """Whole-job throughput of independent replicas: the units all ranks
    processed over the slowest rank's time (weak scaling)."""
    return world * units_per_rank / seconds


# ----------------------------------------------------------------- main -----
# Sub-records of the default run: every configuration of the metric besides
# the headline, each timed the same way (fewer steps), with its roofline,
# end-to-end figure, bounded CPU baseline and sampled parity.
SUB_WORKLOADS = ["poisson16", "elas32", "nh64", "ns64", "gn48", "aniso64", "aniso64s"]


def measure(F, name, args, local, dist, world, rank, headline):
    """Times `name` on this rank's GPU and returns its JSON record."""
    import numpy as np
    import torch
    wl = WORKLOADS[name]
    kind = wl["kind"]
    steps = args.steps if headline else min(args.steps, args.sub_steps)
    dev = torch.device(f"cuda:{local}")
    a, info = make_problem(F, wl, local)
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
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    if dist and headline:
        dist.barrier()
    torch.cuda.synchronize(dev)
    wall0 = time.perf_counter()
    for k in range(steps):
        flush.fill_(float(k))  # evict L2 between timed steps (outside the events)
        starts[k].record(stream)
        step()
        ends[k].record(stream)
    torch.cuda.synchronize(dev)
    if dist and headline:
        dist.barrier()
    wall = time.perf_counter() - wall0
    clk = clocks.stop()
    a.check(sptr)
    launches = a.launch_count() * steps
    step_ms = [s_.elapsed_time(e_) for s_, e_ in zip(starts, ends)]
    total_s = max_over_ranks(sum(step_ms) / 1e3, dist if headline else None, dev)
    # per-stage times: the same steps once more with stage events (the timed
    # steps above carry no instrumentation)
    a.set_profiling(True)
    for k in range(steps):
        flush.fill_(float(k))
        step()
    torch.cuda.synchronize(dev)
    stage_ms = a.stage_times()
    a.set_profiling(False)
    a.check(sptr)
    info["pressure_rows_fused"] = "ns_vel_rows" in stage_ms and "ns_pres_rows" not in stage_ms
    value = job_rate(world if headline else 1, ne * steps, total_s)
    peak, peak_kind = hbm_peak()
    alg = algorithmic_bytes(a, info, kind)
    dom_name, (dom_ms_total, dom_calls) = max(stage_ms.items(), key=lambda kv: kv[1][0])
    dom_ms = dom_ms_total / max(dom_calls, 1)
    dom_bound, dom_bytes = stage_work(a, info, dom_name)
    if dom_bound == "tensor":
        achieved, dom_peak, dom_unit = dom_bytes / (dom_ms * 1e-3) / 1e12, bf16_peak(), "TFLOP/s"
        dom_src = "MEASURED_PEAKS.json bf16_tflops (burst)"
    else:
        achieved, dom_peak, dom_unit = dom_bytes / (dom_ms * 1e-3) / 1e9, peak, "GB/s"
        dom_src = f"MEASURED_PEAKS.json hbm_gbs ({peak_kind})"
    traffic = None
    tpath = os.path.join(ROOT, "profiles", "dram_traffic.json")
    if os.path.exists(tpath):
        try:
            traffic = json.load(open(tpath)).get(name, {}).get(dom_name)
        except Exception:
            traffic = None

    # end to end through the C ABI with host buffers (pinned), copies timed
    h_u = None if info["u"] is None else torch.from_numpy(info["u"]).pin_memory()
    h_p = None if info["p"] is None else torch.from_numpy(info["p"]).pin_memory()
    h_vals = [torch.empty(max(a.block_info(b)[2], 1), dtype=torch.float64).pin_memory() for b in range(nb)]
    h_ru = torch.empty(a.n_u, dtype=torch.float64).pin_memory()
    h_rp = torch.empty(max(a.n_p, 1), dtype=torch.float64).pin_memory() if a.n_p else None
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
    e2e_steps = args.e2e_steps if headline else min(args.e2e_steps, 2)
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        host_step()
    e2e_s = (time.perf_counter() - t0) / e2e_steps
    h2d = 0 if h_u is None else 8 * (a.n_u + (a.n_p if h_p is not None else 0))
    d2h = 8 * sum(a.block_info(b)[2] for b in range(nb)) + (8 * (a.n_u + a.n_p) if want_res else 0)
    e2e = {"value": (world if headline else 1) * ne / e2e_s, "unit": "elements/s", "h2d_bytes_per_step": h2d,
           "d2h_bytes_per_step": d2h, "ms_per_step": 1e3 * e2e_s,
           "note": "fedd_assemble with pinned host buffers: H2D of the fields, kernels, D2H of all CSR values "
                   "and residuals, synchronised, per step"}
    del h_vals, h_ru, h_rp

    out = {
        "metric": METRIC, "value": value, "unit": "elements/s", "n_gpus": world if headline else 1, "steps": steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * total_s / steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "fp32 element math, fp64 geometry + CSR values",
        "data": "synthetic (seeded mesh jitter and fields)",
        "config": {"workload": name, "desc": wl["desc"], "elements": ne,
                   "nnz": [a.block_info(b)[2] for b in range(nb)], "rows": [a.block_info(b)[0] for b in range(nb)],
                   "parallelism": f"replicas x{world}" if (world > 1 and headline) else "1 GPU",
                   **({"field": info["field"]} if "field" in info else {}),
                   "l2": "256 MiB buffer written between timed steps (outside the step events); each step also "
                         "writes > 1 GB", "algorithmic_bytes_per_element": alg / ne,
                   "wall_s_timed_region": wall,
                   "stages_ms_from": "a second pass of the same steps with stage events"},
        "step_roofline": {"bound": "hbm", "achieved": alg * steps / total_s / 1e9, "peak": peak,
                          "unit": "GB/s", "frac": alg * steps / total_s / 1e9 / peak,
                          "peak_source": f"MEASURED_PEAKS.json hbm_gbs ({peak_kind})"},
        "roofline": {"bound": dom_bound, "kernel": dom_name, "achieved": achieved, "peak": dom_peak,
                     "unit": dom_unit, "frac": achieved / dom_peak, "traffic": traffic,
                     ("flops_per_launch" if dom_bound == "tensor" else "bytes_per_launch"): dom_bytes,
                     "ms_per_launch": dom_ms, "peak_source": dom_src},
        "stage_rooflines": {k: stage_frac(a, info, k, v[0] / max(v[1], 1), peak) for k, v in stage_ms.items()},
        "stages_ms": {k: v[0] / max(v[1], 1) for k, v in stage_ms.items()},
        "gpu_launches": launches,
        "clocks": clk,
        "e2e": e2e,
    }
    # the CPU leg: the reference-shaped port timed on a bounded sample, and the
    # oracle as the checker of the timed step's output (sampled complete rows),
    # before any later report changes the output buffers
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline_single(kind, info, args.cpu_sample if headline else args.cpu_sample // 3)
        if kind in ("ns", "gn", "elas", "nh", "aniso", "poisson"):
            step()
            torch.cuda.synchronize(dev)
            out["parity"] = parity_report(a, info, kind, d_vals, d_ru if want_res else None, d_rp, args.parity_frac,
                                          wl["seed"])
    else:
        out["cpu_baseline"] = None
    if headline and kind in ("ns", "nh", "elas"):
        out["dirichlet"] = dirichlet_report(a, info, d_vals, d_ru, d_rp, stream)
    if headline and kind in ("ns", "gn", "nh", "elas") and not dist:
        out["mesh_frontend"] = frontend_report(F, wl, info, kind)
    if kind == "aniso_surr":
        out["surrogate"] = surrogate_report(F, a, info, d_u, d_vals, d_ru, stream, flush, steps, stage_ms)
    # free the workload's device memory before the next one
    for k_ in ("plain",):
        if k_ in info:
            info[k_].close()
    a.close()
    del d_vals, d_ru, d_rp, d_u, d_p, flush
    torch.cuda.empty_cache()
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--workload", default="ns48", choices=sorted(WORKLOADS))
    ap.add_argument("--impl", default="engine", choices=["engine", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-sub", action="store_true", help="headline workload only (no per-configuration sub-records)")
    ap.add_argument("--sub", default=",".join(SUB_WORKLOADS), help="comma-separated sub-record workloads")
    ap.add_argument("--sub-steps", type=int, default=5)
    ap.add_argument("--e2e-steps", type=int, default=3)
    ap.add_argument("--cpu-sample", type=int, default=60000, help="elements of the single-thread CPU baseline")
    ap.add_argument("--parity-frac", type=float, default=0.005, help="sampled share of row nodes for parity")
    args = ap.parse_args()
    wl = WORKLOADS[args.workload]
    if args.impl == "reference":
        return run_reference(args, wl)
    if args.warmup < 3:
        args.warmup = 3

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

    out = measure(F, args.workload, args, local, dist, world, rank, headline=True)
    if not args.no_sub and world == 1:
        subs = {}
        for name in [x for x in args.sub.split(",") if x and x != args.workload]:
            subs[name] = measure(F, name, args, local, None, 1, rank, headline=False)
        out["workloads"] = subs
    if rank == 0:
        print(json.dumps(out))
    if dist:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
