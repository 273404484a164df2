"""Benchmark of the FE operator hot path on GB300.

Workload (default): P1 variable-coefficient diffusion operator div(kappa grad u)
on a 128^3-cell Kuhn cube (12,582,912 tets, 2,146,689 nodes, 31,802,497 CSR
entries), interior nodes jittered by +-0.25h, elements randomly permuted and
kappa lognormal with sigma 1.5 (seed 3), 4-point quadrature.  One step = FP64
assembly of the operator from device-resident inputs + 100 FP64 CSR SpMVs on a
random vector in [-1, 1].  `value` = tets pushed through that step per second
(tets / step time), summed over replicas.  L2 is flushed (a 256 MB write)
before every step; the SpMV working set (425 MB) is larger than L2 as well.

Also reported (measured after the timed steps, same data): FP32 and native-FP64
assembly, FP32 SpMV, the load vector and the adjoint gradient, each kernel's
achieved GB/s against the measured HBM peak; FP64-PCG vs FP32-refined CG to a
1e-10 relative residual on a system whose exact discrete solution is known
(rhs = A u*), with each solution's error; the end-to-end number through the C
ABI with host buffers (warm: plan resident; cold: from host arrays, mesh and
plan built inside the timed region); the P2 48^3 case (Keast 11-point rule,
mixed vs FP64 CG) as a sub-record; and the oracle (a restatement of the
reference algorithm) timed on one host core as the CPU baseline.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference] [--config 2|3|5]
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "tets assembled/s + SpMV GB/s vs HBM peak; FP32-refined vs FP64 CG time to 1e-10"
N_SPMV = 100
# the P1 workloads: 2 = 64^3 (jitter 0.2h, sigma 1, seed 1), 5 = 128^3 (jitter 0.25h, sigma 1.5, seed 3)
P1_CONFIGS = {2: {"n": 64, "jitter": 0.2, "seed": 1, "sigma": 1.0},
              5: {"n": 128, "jitter": 0.25, "seed": 3, "sigma": 1.5}}


def parse(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--config", type=int, default=5, choices=[2, 3, 5],
                    help="5: P1 128^3 (default); 2: P1 64^3; 3: P2 48^3 mixed-precision vs FP64 CG only")
    ap.add_argument("--n", type=int, default=None, help="cells per cube edge (default: the config's)")
    ap.add_argument("--jitter", type=float, default=None)
    ap.add_argument("--sigma", type=float, default=None)
    ap.add_argument("--seed", type=int, default=None)
    ap.add_argument("--no-cg", action="store_true")
    ap.add_argument("--no-p2", action="store_true", help="skip the P2 48^3 sub-record")
    ap.add_argument("--no-cold", action="store_true", help="skip the cold end-to-end sub-record")
    ap.add_argument("--graph", action="store_true", help="time the step as one CUDA graph replay")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--order", type=int, default=1, choices=[1, 2], help="element order of the --only modes")
    ap.add_argument("--only", default=None,
                    choices=["asm64", "asm32", "spmv64", "spmv32", "cg64", "cg32", "adj", "rhs", "suite", "setup",
                             "lagrange"],
                    help="run warmup + steps launches of one kernel only (for profilers) and print its timing")
    a = ap.parse_args(argv)
    base = P1_CONFIGS.get(a.config, P1_CONFIGS[5])
    for k, v in base.items():
        if getattr(a, k) is None:
            setattr(a, k, v)
    return a


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def workload_config(a, E, N, nnz):
    return {"workload": f"P1 kappa-diffusion operator, {a.n}^3 cells x 6 tets ({E} tets, {N} nodes, {nnz} CSR entries), "
                        f"jitter +-{a.jitter}h, element permutation and lognormal kappa sigma {a.sigma} (seed {a.seed}), "
                        f"4-point rule; step = FP64 assembly + {N_SPMV} FP64 SpMV",
            "n_cells": a.n, "tets": E, "nodes": N, "nnz": nnz, "quadrature": 4,
            "l2": "flushed before every step (256 MB write); the SpMV working set is larger than L2 at 128^3",
            "parallelism": f"replicas x{a.gpus}"}


def profiled_traffic(kernel, n):
    """DRAM bytes per launch of `kernel` at n^3 cells, from the committed ncu summary
    (a line `traffic_bytes_per_launch <kernel> <n> <bytes>`), or None."""
    pdir = os.path.join(ROOT, "profiles")
    try:
        names = sorted(os.listdir(pdir))
    except OSError:
        return None, "no profiles directory"
    for name in names:
        try:
            for line in open(os.path.join(pdir, name)):
                f = line.split()
                if len(f) == 4 and f[0] == "traffic_bytes_per_launch" and f[1] == kernel and f[2] == str(n):
                    return float(f[3]), f"profiles/{name} (ncu dram__bytes_read.sum + dram__bytes_write.sum, one launch)"
        except OSError:
            continue
    return None, f"no committed ncu capture of {kernel} at {n}^3"


def asm_bytes(E, nv, nnz, sv, nb=4):
    """algorithmic bytes of one assembly: E (16 conn + 8 kappa + 4 nb^2 slot map) + 24 n_v + s_v nnz"""
    return E * (16 + 8 + 4 * nb * nb) + 24 * nv + sv * nnz


def adj_bytes(E, nv, ndof, nb=4):
    """E (4*4 connectivity + 8 gradient) + 3*8 n_v + 2*8 ndof (u, lambda).  The kernel reads the plan's
    80-byte per-element geometry cache instead of the coordinates, so it moves more than this."""
    return E * (4 * 4 + 8) + 3 * 8 * nv + 2 * 8 * ndof


def rhs_bytes(E, nv, ndof, nb=4):
    """element pass E (4 element id + 4 nb dofs + 8 cached det + 8 scale + 8 nb out) + 8 ndof (field);
    dof pass 4 (ndof + 1) + 12 E nb (slot + entry) + 8 ndof (b)"""
    return E * (24 + 12 * nb) + 8 * ndof + 4 * (ndof + 1) + 12 * E * nb + 8 * ndof


def spmv_bytes(ndof, nnz, sv):
    """nnz (s_v + 4) + 4 (ndof + 1) + 2 s_v ndof"""
    return nnz * (sv + 4) + 4 * (ndof + 1) + 2 * sv * ndof


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 50 ms while running."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.out = None

    def __enter__(self):
        try:
            self.out = tempfile.TemporaryFile("w+")
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=self.out, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if self.proc is None or self.out is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"], "samples": 0}
        self.out.flush()
        self.out.seek(0)
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.out.read().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for k, nm in enumerate(names):
                if f[5 + k].lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


# --------------------------------------------------------------- reference --
def _ref_worker(args):
    """One host process = one 'MPI rank' of the reference algorithm: assembles
    its slab of elements into CSR (pattern + values, insertion-order sums) and
    applies the result 100 times.  Runs the oracle (CPU restatement)."""
    path, rank, nranks, steps, seed = args
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import numpy as np
    import oracle as orc
    d = np.load(path, mmap_mode="r")
    E = d["conn"].shape[0]
    lo, hi = rank * E // nranks, (rank + 1) * E // nranks
    xyz = np.ascontiguousarray(d["xyz"])
    conn = np.ascontiguousarray(d["conn"][lo:hi])
    kap = np.ascontiguousarray(d["kappa"][lo:hi])
    x = np.random.default_rng(seed).uniform(-1, 1, len(xyz))
    times = []
    for _ in range(steps):
        t0 = time.perf_counter()
        dofs = orc.elem_dofs(1, len(xyz), conn)
        rp, ci = orc.pattern(1, len(xyz), dofs)
        vals = orc.assemble("stiff_kappa", 1, 4, xyz, conn, dofs, rp, ci, kap)
        for _ in range(N_SPMV):
            orc.spmv(rp, ci, vals, x)
        times.append(time.perf_counter() - t0)
    return times, hi - lo


def run_reference(a):
    """The reference algorithm (the oracle, a C restatement; the reference binary
    needs MPI, Boost and Trilinos and does not build here) on all host cores, on
    the same workload as the GPU arm: the elements split over one process per
    core, each assembling its slab (pattern + values) and applying it 100 times."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    import multiprocessing as mp
    import numpy as np
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as orc
    from morganapublic_gb300 import meshgen
    orc.build()
    nproc = os.cpu_count() or 1
    m = meshgen.kuhn_cube(a.n, jitter=a.jitter, seed=a.seed, permute=True)
    kappa = meshgen.lognormal(len(m.conn), a.sigma, a.seed)
    E, N = len(m.conn), len(m.xyz)
    # edges of the Kuhn cube (axis, face-diagonal and body-diagonal ones): nnz = N + 2 n_edges
    n_edges = 3 * a.n * (a.n + 1) ** 2 + 3 * a.n ** 2 * (a.n + 1) + a.n ** 3
    # the full mesh split over all host cores, the warm-up and timed steps asked
    # (a 128^3 step takes ~4 s on 16 host cores: the default 3 + 20 steps ~1.5 min)
    warm, timed = max(0, a.warmup), max(1, a.steps)
    steps = warm + timed
    with tempfile.TemporaryDirectory() as td:
        path = os.path.join(td, "mesh.npz")
        np.savez(path, xyz=m.xyz, conn=m.conn, kappa=kappa)
        del m
        ctx = mp.get_context("spawn")
        with ctx.Pool(nproc) as pool:
            res = pool.map(_ref_worker, [(path, r, nproc, steps, a.seed) for r in range(nproc)])
    per_step = [max(r[0][s] for r in res) for s in range(warm, steps)]
    assert sum(r[1] for r in res) == E
    t = statistics.mean(per_step)
    val = E / t
    line = {"impl": "reference", "metric": METRIC, "value": val, "unit": "tets/s", "n_gpus": a.gpus,
            "steps": timed, "warmup": warm, "ms_per_step": t * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {**workload_config(a, E, N, N + 2 * n_edges),
                       "l2": "host run (no L2 flush)",
                       "parallelism": f"elements split over {nproc} host processes (one per core)"},
            "cpu_baseline": {"value": val, "unit": "tets/s", "cores": nproc, "kind": "port",
                             "sample": f"full {a.n}^3 mesh per step, {warm} warm-up + {timed} timed steps, "
                                       f"{nproc} processes x 1 thread, CPU restatement of the reference algorithm "
                                       "(reference binary not buildable: needs MPI, Boost, Trilinos)"},
            "e2e": {"value": val, "unit": "tets/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def cpu_baseline_port(a, budget_s=12.0):
    """The oracle on one host core, bounded: assembly of a 24^3 mesh repeated."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as orc
    from morganapublic_gb300 import meshgen
    n = min(a.n, 24)
    m = meshgen.kuhn_cube(n, jitter=a.jitter, seed=a.seed, permute=True)
    kappa = meshgen.lognormal(len(m.conn), a.sigma, a.seed)
    t_asm, reps = 0.0, 0
    t_end = time.perf_counter() + budget_s
    while time.perf_counter() < t_end or reps == 0:
        t0 = time.perf_counter()
        dofs = orc.elem_dofs(1, len(m.xyz), m.conn)
        rp, ci = orc.pattern(1, len(m.xyz), dofs)
        orc.assemble("stiff_kappa", 1, 4, m.xyz, m.conn, dofs, rp, ci, kappa)
        t_asm += time.perf_counter() - t0
        reps += 1
    return {"value": reps * len(m.conn) / t_asm, "unit": "tets/s", "cores": 1, "kind": "port",
            "sample": f"{n}^3 mesh ({len(m.conn)} tets) assembled {reps}x (pattern + values, reference algorithm "
                      f"restated in C, -O2), {t_asm:.1f} s"}


# -------------------------------------------------------------------- gb300 --
def run_only(a):
    """warmup + steps launches of a single kernel on the bench workload, L2 flushed
    before each; prints the median launch time and its GB/s."""
    import numpy as np
    import torch
    import morganapublic_gb300 as mg
    from morganapublic_gb300 import meshgen
    m = meshgen.kuhn_cube(a.n, jitter=a.jitter, seed=a.seed, permute=True)
    if a.only == "setup":
        # mesh preprocessing on the GPU (P2 edges, CSR pattern) against the host builds
        res = {}
        for r in range(a.warmup + a.steps):
            t0 = time.perf_counter()
            mh = mg.Mesh(m.xyz, m.conn, order=a.order)
            t1 = time.perf_counter()
            bh = mg.MatrixBuilder(mh)
            t2 = time.perf_counter()
            md = mg.Mesh(m.xyz, m.conn, order=a.order, edges_on_device=True)
            t3 = time.perf_counter()
            bd = mg.MatrixBuilder(md, pattern_on_device=True)
            t4 = time.perf_counter()
            same = all(np.array_equal(u, w) for u, w in zip(bh.pattern(), bd.pattern()))
            if r >= a.warmup:
                for k, v in (("mesh_host_s", t1 - t0), ("plan_host_s", t2 - t1), ("mesh_device_s", t3 - t2),
                             ("plan_device_pattern_s", t4 - t3)):
                    res.setdefault(k, []).append(v)
            bh.close(), bd.close(), mh.close(), md.close()
        print(json.dumps({"only": "setup", "n": a.n, "order": a.order, "identical": same,
                          **{k: statistics.median(v) for k, v in res.items()}}))
        return 0
    kappa = torch.from_numpy(meshgen.lognormal(len(m.conn), a.sigma, a.seed)).cuda()
    mesh = mg.Mesh(m.xyz, m.conn, order=a.order)
    b = mg.MatrixBuilder(mesh)
    quad = 4 if a.order == 1 else 11
    stream = torch.cuda.Stream()
    x = torch.from_numpy(np.random.default_rng(a.seed).uniform(-1, 1, b.ndof)).cuda()
    v64 = b.assemble("stiff_kappa", coeff=kappa, quad=quad, prec="f64")
    v32 = b.assemble("stiff_kappa", coeff=kappa, quad=quad, prec="f32")
    x32, y, y32 = x.float(), torch.empty_like(x), torch.empty_like(x, dtype=torch.float32)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    if a.only == "suite":
        # every kernel of the path once per round (for a per-kernel ncu launch list):
        # assembly FP64 + FP32, load vector, Dirichlet elimination, SpMV FP64 + FP32,
        # a few PCG iterations FP64 and FP32-refined, adjoint gradient
        mask = torch.from_numpy(m.boundary if a.order == 1 else meshgen.p2_boundary(m.boundary, mesh.edges()[0]))
        lam = torch.from_numpy(np.random.default_rng(a.seed + 1).uniform(-1, 1, b.ndof)).cuda()
        g = torch.empty(len(m.conn), dtype=torch.float64, device="cuda")
        with torch.cuda.stream(stream):
            for r in range(a.warmup + a.steps):
                b.assemble("stiff_kappa", coeff=kappa, quad=quad, prec="f64", out=v64, stream=stream)
                b.assemble("stiff_kappa", coeff=kappa, quad=quad, prec="f32", out=v32, stream=stream)
                rhs = b.build_vector(quad=quad, stream=stream)
                b.apply_dirichlet(v64, mask, rhs, stream=stream)
                b.apply_dirichlet(v32, mask, stream=stream)
                b.apply(v64, x, out=y, stream=stream)
                b.apply(v32, x32, out=y32, stream=stream)
                b.cg(v64, rhs, rtol=1e-30, maxit=16, stream=stream, raise_on_fail=False)
                b.cg_refined(v64, v32, rhs, rtol=1e-30, max_outer=2, max_inner=16, stream=stream,
                             raise_on_fail=False)
                b.adjoint_grad(x, lam, quad=quad, out=g, stream=stream)
        torch.cuda.synchronize()
        print(json.dumps({"only": a.only, "n": a.n, "order": a.order, "rounds": a.warmup + a.steps}))
        return 0
    if a.only == "lagrange":
        # boundary multipliers: host build, B = opLA3dA (face matrices + gather), saddle fill,
        # saddle SpMV; median CUDA-event time per call, L2 flushed before each
        t0 = time.perf_counter()
        lg = mg.LagrangeBuilder(b)
        build_s = time.perf_counter() - t0
        bv = lg.assemble(quad=1)
        sv = lg.saddle(v64, bv)
        xs = torch.from_numpy(np.random.default_rng(a.seed).uniform(-1, 1, b.ndof + lg.n_multipliers)).cuda()
        ys = torch.empty_like(xs)
        calls = {"b_assemble": lambda: lg.assemble(quad=1, out=bv, stream=stream),
                 "saddle_fill": lambda: lg.saddle(v64, bv, out=sv, stream=stream),
                 "saddle_spmv": lambda: lg.saddle_apply(sv, xs, out=ys, stream=stream)}
        res = {}
        torch.cuda.synchronize()
        with torch.cuda.stream(stream):
            for name, fn in calls.items():
                ts = []
                for r in range(a.warmup + a.steps):
                    flush.fill_(float(r))
                    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                    e0.record(stream)
                    fn()
                    e1.record(stream)
                    torch.cuda.synchronize()
                    if r >= a.warmup:
                        ts.append(e0.elapsed_time(e1))
                res[name + "_ms"] = statistics.median(ts)
        nb = 4 if a.order == 1 else 10
        F, nzb, nzs, rows = lg.n_faces, lg.nnz_b, lg.nnz_saddle, b.ndof + lg.n_multipliers
        # the reference algorithm for B on one host core: face integrals (C restatement) and
        # insertion-order sums into the pattern; the boundary-face search is outside the timing
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle as orc
        faces = orc.boundary_faces(m.conn)
        dofs = mesh.elem_dofs()
        t0 = time.perf_counter()
        orc.lagrange(a.order, 1, m.xyz, m.conn, dofs, b.ndof, faces=faces)
        cpu_s = time.perf_counter() - t0
        cpu = {"value": F / cpu_s, "unit": "faces/s", "cores": 1, "kind": "port",
               "sample": f"B of all {F} boundary faces once (face integrals in C, -O2; sums in numpy), {cpu_s:.2f} s"}
        byts = {"b_assemble": F * (8 + 16 + 3 * 32 + 2 * 3 * nb * 8) + nzb * 12 + 4 * F * 3 * nb,
                "saddle_fill": nzs * 20, "saddle_spmv": spmv_bytes(rows, nzs, 8)}
        print(json.dumps({"only": "lagrange", "n": a.n, "order": a.order, "faces": F, "multipliers": lg.n_multipliers,
                          "nnz_b": nzb, "nnz_saddle": nzs, "build_s": build_s, **res,
                          **{k + "_gbs": byts[k] / res[k + "_ms"] / 1e6 for k in byts},
                          "b_faces_per_s": F / (res["b_assemble_ms"] * 1e-3), "cpu_baseline": cpu,
                          "algorithmic_bytes": byts}))
        lg.close()
        return 0
    if a.only in ("cg64", "cg32"):
        # a fixed number of PCG iterations on the Dirichlet system (f = 1)
        rhs = b.build_vector(quad=quad)
        mask = torch.from_numpy(m.boundary if a.order == 1 else meshgen.p2_boundary(m.boundary, mesh.edges()[0]))
        b.apply_dirichlet(v64, mask, rhs)
        b.apply_dirichlet(v32, mask)
        ts = []
        with torch.cuda.stream(stream):
            for r in range(a.warmup + a.steps):
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                if a.only == "cg64":
                    _, info = b.cg(v64, rhs, rtol=1e-30, maxit=64, stream=stream, raise_on_fail=False)
                else:
                    _, info = b.cg_refined(v64, v32, rhs, rtol=1e-30, max_outer=1, max_inner=64, stream=stream,
                                           raise_on_fail=False)
                torch.cuda.synchronize()
                if r >= a.warmup:
                    ts.append((time.perf_counter() - t0) * 1e3 / max(1, info.iterations))
        print(json.dumps({"only": a.only, "n": a.n, "ms_per_iteration": statistics.median(ts)}))
        return 0
    lam = torch.from_numpy(np.random.default_rng(a.seed + 1).uniform(-1, 1, b.ndof)).cuda()
    g = torch.empty(len(m.conn), dtype=torch.float64, device="cuda")
    nb = 4 if a.order == 1 else 10
    fn = {"asm64": lambda: b.assemble("stiff_kappa", coeff=kappa, quad=quad, prec="f64", out=v64, stream=stream),
          "asm32": lambda: b.assemble("stiff_kappa", coeff=kappa, quad=quad, prec="f32", out=v32, stream=stream),
          "spmv64": lambda: b.apply(v64, x, out=y, stream=stream),
          "spmv32": lambda: b.apply(v32, x32, out=y32, stream=stream),
          "adj": lambda: b.adjoint_grad(x, lam, quad=quad, out=g, stream=stream),
          "rhs": lambda: b.build_vector(field=x, elem_scale=kappa, quad=quad, out=y, stream=stream)}[a.only]
    E, nv = len(m.conn), len(m.xyz)
    byts = {"asm64": asm_bytes(E, nv, b.nnz, 8, nb), "asm32": asm_bytes(E, nv, b.nnz, 4, nb),
            "spmv64": spmv_bytes(b.ndof, b.nnz, 8), "spmv32": spmv_bytes(b.ndof, b.nnz, 4),
            "adj": adj_bytes(E, nv, b.ndof, nb), "rhs": rhs_bytes(E, nv, b.ndof, nb)}[a.only]
    ts = []
    torch.cuda.synchronize()
    with torch.cuda.stream(stream):
        for r in range(a.warmup + a.steps):
            flush.fill_(float(r))
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            fn()
            e1.record(stream)
            torch.cuda.synchronize()
            if r >= a.warmup:
                ts.append(e0.elapsed_time(e1))
    ms = statistics.median(ts)
    print(json.dumps({"only": a.only, "n": a.n, "order": a.order, "ms": ms, "gbs": byts / ms / 1e6,
                      "algorithmic_bytes": byts}))
    return 0


def replica_throughput(ms_local, units_local, world, device):
    """Replicas: every rank runs the whole step on its own GPU.  Returns the step
    time as the maximum over ranks and the job throughput world * units / time."""
    ms = ms_local
    if world > 1:
        import torch
        import torch.distributed as dist
        t = torch.tensor([ms_local], device=device, dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    return ms, world * units_local / (ms * 1e-3)


def _timed_cuda(torch, stream, fn, reps, flush=None):
    """median CUDA-event time (ms) of fn on `stream`; L2 flushed before each rep when `flush` is given"""
    ts = []
    with torch.cuda.stream(stream):
        for r in range(reps + 2):
            if flush is not None:
                flush.fill_(float(r))
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            fn()
            e1.record(stream)
            torch.cuda.synchronize()
            if r >= 2:
                ts.append(e0.elapsed_time(e1))
    return statistics.median(ts)


def _rec(peak, bytes_, ms, units=None):
    gbs = bytes_ / (ms * 1e-3) / 1e9
    d = {"ms": ms, "gbs": gbs, "frac_of_hbm": gbs / peak, "algorithmic_bytes": bytes_}
    if units:
        d["tets_per_s"] = units / (ms * 1e-3)
    return d


def _sin_field(X):
    import numpy as np
    return np.sin(np.pi * X[:, 0]) * np.sin(np.pi * X[:, 1]) * np.sin(np.pi * X[:, 2])


def p2_record(seed=1):
    """P2 (10-node) kappa-stiffness on 48^3 cells x 6 tets, Keast 11-point rule, kappa lognormal sigma 0.5.
    The right-hand side is A u_I for the P2 interpolant u_I of sin(pi x) sin(pi y) sin(pi z) (zero on the
    boundary, Dirichlet rows eliminated), so u_I is the exact discrete solution and each solver's error
    against it is its solve error.  FP64 Jacobi-PCG vs FP32-inner/FP64-refined CG, both to a 1e-10 relative
    residual; each solve run twice, the second timed."""
    import numpy as np
    import torch
    import morganapublic_gb300 as mg
    from morganapublic_gb300 import meshgen
    n, q = 48, 11
    stream = torch.cuda.Stream()
    peak, peak_kind = peaks()
    m = meshgen.kuhn_cube(n)
    kappa_h = meshgen.lognormal(len(m.conn), 0.5, seed)
    setup = {}
    t0 = time.perf_counter()
    mesh = mg.Mesh(m.xyz, m.conn, order=2)
    setup["mesh_edges_host_s"] = time.perf_counter() - t0
    t0 = time.perf_counter()
    b = mg.MatrixBuilder(mesh)
    setup["plan_host_s"] = time.perf_counter() - t0
    t0 = time.perf_counter()
    mesh_d = mg.Mesh(m.xyz, m.conn, order=2, edges_on_device=True)
    setup["mesh_edges_device_s"] = time.perf_counter() - t0
    t0 = time.perf_counter()
    b_d = mg.MatrixBuilder(mesh_d, pattern_on_device=True)
    setup["plan_pattern_on_device_s"] = time.perf_counter() - t0
    setup["identical"] = bool(np.array_equal(mesh.elem_dofs(), mesh_d.elem_dofs()) and
                              all(np.array_equal(u, w) for u, w in zip(b.pattern(), b_d.pattern())))
    b_d.close()
    mesh_d.close()
    E, ndof, nnz = len(m.conn), b.ndof, b.nnz
    en, _ = mesh.edges()
    X = np.concatenate([m.xyz, 0.5 * (m.xyz[en[:, 0]] + m.xyz[en[:, 1]])])
    bmask = meshgen.p2_boundary(m.boundary, en)
    uI = _sin_field(X)
    uI[bmask] = 0.0
    kappa = torch.from_numpy(kappa_h).cuda()
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    with torch.cuda.stream(stream):
        A64 = b.assemble("stiff_kappa", coeff=kappa, quad=q, prec="f64", stream=stream)
        A32 = b.assemble("stiff_kappa", coeff=kappa, quad=q, prec="f32", stream=stream)
        mask = torch.from_numpy(bmask)
        b.apply_dirichlet(A64, mask, stream=stream)
        b.apply_dirichlet(A32, mask, stream=stream)
        uI_d = torch.from_numpy(uI).cuda()
        rhs = b.apply(A64, uI_d, stream=stream)
    torch.cuda.synchronize()
    t64 = _timed_cuda(torch, stream, lambda: b.assemble("stiff_kappa", coeff=kappa, quad=q, prec="f64", out=A64,
                                                        stream=stream), 20, flush)
    t32 = _timed_cuda(torch, stream, lambda: b.assemble("stiff_kappa", coeff=kappa, quad=q, prec="f32", out=A32,
                                                        stream=stream), 20, flush)
    t64n = _timed_cuda(torch, stream, lambda: b.assemble("stiff_kappa", coeff=kappa, quad=q, prec="f64_native",
                                                         out=A64, stream=stream), 20, flush)
    with torch.cuda.stream(stream):
        b.assemble("stiff_kappa", coeff=kappa, quad=q, prec="f64", out=A64, stream=stream)
        b.apply_dirichlet(A64, mask, stream=stream)
        b.apply_dirichlet(A32, mask, stream=stream)
    y = torch.empty_like(rhs)
    ts64 = _timed_cuda(torch, stream, lambda: b.apply(A64, uI_d, out=y, stream=stream), 20, flush)
    A32c = A32.clone()
    x32 = uI_d.float()
    y32 = torch.empty_like(x32)
    ts32 = _timed_cuda(torch, stream, lambda: b.apply(A32c, x32, out=y32, stream=stream), 20, flush)
    for rep in range(2):
        with torch.cuda.stream(stream):
            xs, i64 = b.cg(A64, rhs, rtol=1e-10, maxit=50000, stream=stream)
            xr, imx = b.cg_refined(A64, A32, rhs, rtol=1e-10, inner_rtol=1e-2, stream=stream)
        torch.cuda.synchronize()
    err64 = float(torch.linalg.norm(xs - uI_d) / torch.linalg.norm(uI_d))
    errmx = float(torch.linalg.norm(xr - uI_d) / torch.linalg.norm(uI_d))
    diff = float(torch.linalg.norm(xr - xs) / torch.linalg.norm(xs))
    g = torch.empty(E, dtype=torch.float64, device="cuda")
    yb = torch.empty_like(rhs)
    tadj = _timed_cuda(torch, stream, lambda: b.adjoint_grad(xs, xr, quad=q, out=g, stream=stream), 20, flush)
    trhs = _timed_cuda(torch, stream, lambda: b.build_vector(field=uI_d, elem_scale=kappa, quad=q, out=yb,
                                                             stream=stream), 20, flush)
    nv = len(m.xyz)
    rec = {"config": {"workload": f"P2 kappa-stiffness, {n}^3 cells x 6 tets ({E} tets, {ndof} dofs, {nnz} CSR "
                                  "entries), Keast 11-point rule, lognormal kappa sigma 0.5, rhs = A u_I (u_I = P2 "
                                  "interpolant of sin(pi x) sin(pi y) sin(pi z)), Dirichlet u = 0; L2 flushed "
                                  "before each kernel timing",
                      "tets": E, "dofs": ndof, "nnz": nnz, "setup": setup},
           "assembly_f64": _rec(peak, asm_bytes(E, nv, nnz, 8, nb=10), t64, E),
           "assembly_f32": _rec(peak, asm_bytes(E, nv, nnz, 4, nb=10), t32, E),
           "assembly_f64_native": {**_rec(peak, asm_bytes(E, nv, nnz, 8, nb=10), t64n, E),
                                   "note": "native FP64 element arithmetic (MG_F64_NATIVE), for comparison"},
           "spmv_f64": _rec(peak, spmv_bytes(ndof, nnz, 8), ts64),
           "spmv_f32": _rec(peak, spmv_bytes(ndof, nnz, 4), ts32),
           "adjoint_grad": _rec(peak, adj_bytes(E, nv, ndof, 10), tadj, E),
           "load_vector": _rec(peak, rhs_bytes(E, nv, ndof, 10), trhs, E),
           "cg": {"fp64_pcg": i64.as_dict(), "fp32_refined": imx.as_dict(),
                  "speedup_refined_vs_fp64": i64.seconds / imx.seconds if imx.seconds > 0 else None,
                  "fp64_error_vs_exact_discrete": err64, "refined_error_vs_exact_discrete": errmx,
                  "refined_vs_fp64_rel_diff": diff, "precond": "jacobi", "rtol": 1e-10, "inner_rtol": 1e-2},
           "peak_gbs": peak, "peak_kind": peak_kind}
    b.close()
    mesh.close()
    return rec


def run_config3(a):
    print(json.dumps(p2_record(a.seed)))
    return 0


def main():
    a = parse()
    if a.impl == "reference":
        return run_reference(a)
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if a.only:
        return run_only(a)
    if a.config == 3:
        return run_config3(a)
    cpu_base = None
    if rank == 0 and not a.no_cpu_baseline:
        cpu_base = cpu_baseline_port(a)  # before any CUDA work
    import numpy as np
    import torch
    import torch.distributed as dist
    import morganapublic_gb300 as mg
    from morganapublic_gb300 import meshgen

    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    stream = torch.cuda.Stream()
    peak, peak_kind = peaks()

    m = meshgen.kuhn_cube(a.n, jitter=a.jitter, seed=a.seed, permute=True)
    kappa_h = meshgen.lognormal(len(m.conn), a.sigma, a.seed)
    E, N = len(m.conn), len(m.xyz)
    setup = {}
    t0 = time.perf_counter()
    mesh = mg.Mesh(m.xyz, m.conn, order=1)
    setup["mesh_tables_s"] = time.perf_counter() - t0
    t0 = time.perf_counter()
    b = mg.MatrixBuilder(mesh)
    setup["plan_host_s"] = time.perf_counter() - t0
    nnz, ndof = b.nnz, b.ndof
    bmi = b.block_map_info()
    kappa = torch.from_numpy(kappa_h).cuda()
    x = torch.from_numpy(np.random.default_rng(a.seed).uniform(-1, 1, ndof)).cuda()
    x32 = x.float()
    v64 = torch.empty(nnz, dtype=torch.float64, device="cuda")
    v32 = torch.empty(nnz, dtype=torch.float32, device="cuda")
    y = torch.empty(ndof, dtype=torch.float64, device="cuda")
    y32 = torch.empty(ndof, dtype=torch.float32, device="cuda")
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    b.assemble("stiff_kappa", coeff=kappa, quad=4, prec="f64", out=v64)  # first use: upload of the plan
    torch.cuda.synchronize()
    setup["first_use_s"] = time.perf_counter() - t0
    b.status()

    def step(ev=None):
        if ev:
            ev[0].record(stream)
        b.assemble("stiff_kappa", coeff=kappa, quad=4, prec="f64", out=v64, stream=stream)
        if ev:
            ev[1].record(stream)
        for _ in range(N_SPMV):
            b.apply(v64, x, out=y, stream=stream)
        if ev:
            ev[2].record(stream)

    # the step as stream launches (each launch is long against its launch cost at
    # this size); events on the launching stream split it into the assembly and
    # the SpMVs.  --graph replays it as one CUDA graph instead.
    graph = None
    with torch.cuda.stream(stream):
        for _ in range(a.warmup):
            flush.fill_(1.0)
            step()
        torch.cuda.synchronize()
        if a.graph:
            graph = torch.cuda.CUDAGraph()
            with torch.cuda.graph(graph, stream=stream):
                step()
            torch.cuda.synchronize()
            for _ in range(a.warmup):
                flush.fill_(1.0)
                graph.replay()
            torch.cuda.synchronize()
        evs = [[torch.cuda.Event(enable_timing=True) for _ in range(3)] for _ in range(a.steps)]
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()
        with ClockSampler(local) as clk:
            t_wall0 = time.perf_counter()
            for s in range(a.steps):
                flush.fill_(float(s))
                if graph is None:
                    step(evs[s])
                else:
                    evs[s][0].record(stream)
                    graph.replay()
                    evs[s][2].record(stream)
            torch.cuda.synchronize()
            t_wall = time.perf_counter() - t_wall0
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()
    b.status()
    t_step = [e[0].elapsed_time(e[2]) for e in evs]
    if graph is None:
        t_asm = [e[0].elapsed_time(e[1]) for e in evs]
        t_spmv = [e[1].elapsed_time(e[2]) / N_SPMV for e in evs]
    else:
        t_asm, t_spmv = [], []
    ms_step, value = replica_throughput(statistics.mean(t_step), E, world, "cuda")

    extras, line = {}, None
    if rank == 0:
        B64, B32 = asm_bytes(E, N, nnz, 8), asm_bytes(E, N, nnz, 4)
        S64, S32 = spmv_bytes(ndof, nnz, 8), spmv_bytes(ndof, nnz, 4)
        fl = dict(flush=flush)
        if not t_asm:
            t_asm = [_timed_cuda(torch, stream, lambda: b.assemble("stiff_kappa", coeff=kappa, quad=4, prec="f64",
                                                                   out=v64, stream=stream), 20, **fl)]
            t_spmv = [(ms_step - t_asm[0]) / N_SPMV]
        ta64 = statistics.median(t_asm)
        ts64 = statistics.median(t_spmv)
        ta32 = _timed_cuda(torch, stream, lambda: b.assemble("stiff_kappa", coeff=kappa, quad=4, prec="f32",
                                                             out=v32, stream=stream), 20, **fl)
        ta64n = _timed_cuda(torch, stream, lambda: b.assemble("stiff_kappa", coeff=kappa, quad=4, prec="f64_native",
                                                              out=v64, stream=stream), 20, **fl)
        ts64c = _timed_cuda(torch, stream, lambda: b.apply(v64, x, out=y, stream=stream), 20, **fl)
        ts32 = _timed_cuda(torch, stream, lambda: b.apply(v32, x32, out=y32, stream=stream), 20, **fl)
        lam = torch.from_numpy(np.random.default_rng(a.seed + 1).uniform(-1, 1, ndof)).cuda()
        g = torch.empty(E, dtype=torch.float64, device="cuda")
        yb = torch.empty_like(x)
        b.adjoint_grad(x, lam, quad=4, out=g)  # first call builds the element-geometry cache
        b.build_vector(field=x, elem_scale=kappa, quad=4, out=yb)  # and the load-vector map
        tg = _timed_cuda(torch, stream, lambda: b.adjoint_grad(x, lam, quad=4, out=g, stream=stream), 20, **fl)
        tb = _timed_cuda(torch, stream, lambda: b.build_vector(field=x, elem_scale=kappa, quad=4, out=yb,
                                                               stream=stream), 20, **fl)
        extras["assembly_f64"] = {**_rec(peak, B64, ta64, E),
                                  "note": "in the timed step; double-word FP32 arithmetic, FP64-accurate values"}
        extras["assembly_f32"] = _rec(peak, B32, ta32, E)
        extras["assembly_f64_native"] = {**_rec(peak, B64, ta64n, E),
                                         "note": "native FP64 element arithmetic (MG_F64_NATIVE), for comparison"}
        extras["spmv_f64_in_step"] = {**_rec(peak, S64, ts64),
                                      "note": f"per-SpMV time inside the timed step ({N_SPMV} back to back)"}
        extras["spmv_f64_cold"] = {**_rec(peak, S64, ts64c), "note": "one launch, L2 flushed before it"}
        extras["spmv_f32"] = {**_rec(peak, S32, ts32), "note": "one launch, L2 flushed before it"}
        extras["adjoint_grad"] = _rec(peak, adj_bytes(E, N, ndof), tg, E)
        extras["load_vector"] = _rec(peak, rhs_bytes(E, N, ndof), tb, E)
        extras["block_map"] = {"upper_entries": bmi.n_upper, "sources": bmi.n_contrib, "blocks": bmi.n_blocks,
                               "elems_per_block": bmi.elems_per_block, "runs": bmi.n_runs,
                               "shared_entries": bmi.n_shared,
                               "shared_fraction": bmi.n_shared / max(1, bmi.n_upper),
                               "partial_slots": bmi.n_partial,
                               "padding_factor": bmi.n_src / max(1, bmi.n_contrib),
                               "map_bytes": 2 * bmi.n_src + 8 * 32 * bmi.n_groups + 4 * (bmi.n_groups + bmi.n_blocks)
                               + 8 * 32 * bmi.n_shared_groups + 4 * bmi.n_shared_groups,
                               "note": "one CTA per block of Morton-consecutive elements: element matrices in shared "
                                       "memory, each diagonal / upper CSR entry summed there and written with its "
                                       "mirror (k_block_asm); entries spanning blocks through per-block partial sums "
                                       "added in block order (k_shared_sum)"}
        extras["setup"] = setup
        if graph is not None:
            extras["step_graph_ms"] = ms_step

        # CG: FP64 PCG vs FP32-refined, Dirichlet u = 0, rhs = A u* (u* = sin sin sin at the
        # nodes, zero on the boundary), so u* is the exact discrete solution of the operator
        # the parity tests check against the oracle; each solve's error against it
        if not a.no_cg:
            us = _sin_field(m.xyz)
            us[m.boundary] = 0.0
            us_d = torch.from_numpy(us).cuda()
            mask = torch.from_numpy(m.boundary)
            with torch.cuda.stream(stream):
                A64 = b.assemble("stiff_kappa", coeff=kappa, quad=4, prec="f64", stream=stream)
                A32 = b.assemble("stiff_kappa", coeff=kappa, quad=4, prec="f32", stream=stream)
                b.apply_dirichlet(A64, mask, stream=stream)
                b.apply_dirichlet(A32, mask, stream=stream)
                rhs = b.apply(A64, us_d, stream=stream)
            torch.cuda.synchronize()
            for _ in range(2):  # the second solve of each is reported
                with torch.cuda.stream(stream):
                    xs, i64 = b.cg(A64, rhs, rtol=1e-10, maxit=50000, stream=stream)
                    xr, imx = b.cg_refined(A64, A32, rhs, rtol=1e-10, inner_rtol=1e-2, stream=stream)
                torch.cuda.synchronize()
            nus = torch.linalg.norm(us_d)
            extras["cg"] = {"fp64_pcg": i64.as_dict(), "fp32_refined": imx.as_dict(),
                            "speedup_refined_vs_fp64": i64.seconds / imx.seconds if imx.seconds > 0 else None,
                            "fp64_error_vs_exact_discrete": float(torch.linalg.norm(xs - us_d) / nus),
                            "refined_error_vs_exact_discrete": float(torch.linalg.norm(xr - us_d) / nus),
                            "refined_vs_fp64_solution_rel_diff": float(torch.linalg.norm(xr - xs) /
                                                                       torch.linalg.norm(xs)),
                            "precond": "jacobi", "rtol": 1e-10, "inner_rtol": 1e-2,
                            "rhs": "A u*, u* = sin(pi x) sin(pi y) sin(pi z) at the nodes (zero on the boundary): "
                                   "u* is the exact discrete solution"}
            del A64, A32

        # e2e through the public API with host buffers: kappa in, CSR values out, x in, y out
        kap_pin = torch.from_numpy(kappa_h).pin_memory()
        x_pin = x.cpu().pin_memory()
        v_pin = torch.empty(nnz, dtype=torch.float64).pin_memory()
        y_pin = torch.empty(ndof, dtype=torch.float64).pin_memory()
        kap_d = torch.empty_like(kappa)
        x_d = torch.empty_like(x)
        # copies on a second stream overlap the kernels that do not need them: x
        # arrives during the assembly, the CSR values leave during the SpMVs
        cstream = torch.cuda.Stream()
        ev_x, ev_asm, ev_v = (torch.cuda.Event() for _ in range(3))

        def e2e_step():
            kap_d.copy_(kap_pin, non_blocking=True)
            cstream.wait_stream(stream)
            with torch.cuda.stream(cstream):
                x_d.copy_(x_pin, non_blocking=True)
                ev_x.record(cstream)
            b.assemble("stiff_kappa", coeff=kap_d, quad=4, prec="f64", out=v64, stream=stream)
            ev_asm.record(stream)
            with torch.cuda.stream(cstream):
                cstream.wait_event(ev_asm)
                v_pin.copy_(v64, non_blocking=True)
                ev_v.record(cstream)
            stream.wait_event(ev_x)
            for _ in range(N_SPMV):
                b.apply(v64, x_d, out=y, stream=stream)
            y_pin.copy_(y, non_blocking=True)
            stream.wait_event(ev_v)

        te2e = _timed_cuda(torch, stream, e2e_step, max(3, min(a.steps, 10)), flush)
        h2d, d2h = 8 * E + 8 * ndof, 8 * nnz + 8 * ndof
        e2e = {"value": world * E / (te2e * 1e-3), "unit": "tets/s", "h2d_bytes_per_step": h2d,
               "d2h_bytes_per_step": d2h, "ms_per_step": te2e,
               "note": "kappa and x copied in from pinned host memory, CSR values and y copied out, per step; the x "
                       "upload overlaps the assembly and the values download overlaps the SpMVs (second stream)"}

        # cold e2e: the work the reference arm's step does, from host arrays -- mesh
        # tables, CSR pattern, element order and block map (on the GPU), first assembly and
        # 100 SpMVs, values and y back in host memory; wall clock
        e2e_cold = None
        if not a.no_cold:
            ts, stages = [], []
            for _ in range(3):
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                mc = mg.Mesh(m.xyz, m.conn, order=1)
                t1 = time.perf_counter()
                bc = mg.MatrixBuilder(mc, pattern_on_device=True)
                torch.cuda.synchronize()
                t2 = time.perf_counter()
                vc = bc.assemble("stiff_kappa", coeff=kap_pin, quad=4, prec="f64")
                torch.cuda.synchronize()
                t3 = time.perf_counter()
                xc = x_pin.cuda()
                yc = torch.empty_like(xc)
                for _ in range(N_SPMV):
                    bc.apply(vc, xc, out=yc)
                vh, yh = vc.cpu(), yc.cpu()
                torch.cuda.synchronize()
                ts.append(time.perf_counter() - t0)
                stages.append((t1 - t0, t2 - t1, t3 - t2, ts[-1] - (t3 - t0)))
                del vc, xc, yc, vh, yh
                bc.close()
                mc.close()
            tc = statistics.median(ts)
            e2e_cold = {"value": world * E / tc, "unit": "tets/s", "ms_per_step": tc * 1e3,
                        "runs_s": ts,
                        "stages_s": {k: statistics.median(s[i] for s in stages) for i, k in enumerate(
                            ("mesh_create", "plan_build_device", "first_assembly_with_coefficient_upload",
                             "spmvs_and_copies"))}, "h2d_bytes_per_step": 24 * N + 16 * E + 8 * E + 8 * ndof,
                        "d2h_bytes_per_step": d2h,
                        "note": "from host arrays: mg_mesh_create + mg_pattern_build_device (CSR pattern, element "
                                "order and block map built on the GPU) + first mg_assemble + "
                                f"{N_SPMV} SpMV, values and y copied back; wall clock, median of 3 -- the work one "
                                "step of the reference arm does"}

        if not a.no_p2:
            extras["config3_p2_48"] = p2_record()

        rl = extras["spmv_f64_in_step"] if N_SPMV * ts64 >= ta64 else extras["assembly_f64"]
        kname = "k_spmv<double,1>" if rl is extras["spmv_f64_in_step"] else "k_block_asm<kDW> + k_shared_sum<kDW>"
        traffic, tnote = profiled_traffic(kname, a.n)
        roofline = {"bound": "hbm", "kernel": kname,
                    "achieved": rl["gbs"], "peak": peak, "unit": "GB/s", "frac": rl["gbs"] / peak,
                    "peak_kind": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured" else peak_kind,
                    "traffic": traffic, "traffic_note": tnote,
                    "note": "achieved = algorithmic bytes per launch (4-byte column indices counted) / CUDA-event "
                            "time per launch inside the timed step"}
        clocks = clk.summary()
        line = {"metric": METRIC, "value": value, "unit": "tets/s", "n_gpus": world, "steps": a.steps,
                "warmup": a.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f64",
                "dtype_note": "FP64 values (IEEE doubles in and out, within 1e-12 row-scaled of the FP64 oracle); the "
                              "assembly computes them in double-word FP32 arithmetic (two floats per number), the "
                              "SpMV in native FP64; assembly_f64_native gives the native-FP64 assembly",
                "data": "synthetic (seeded Kuhn cube, jitter, element permutation, lognormal kappa)",
                "config": workload_config(a, E, N, nnz), "roofline": roofline, "cpu_baseline": cpu_base,
                "e2e": e2e, "e2e_cold": e2e_cold, "gpu_launches": a.steps * (2 + N_SPMV),  # block assembly + shared sums + SpMVs
                "clocks": clocks, "wall_s_timed": t_wall, "kernels": extras}
    if world > 1:
        dist.barrier()
        dist.destroy_process_group()
    if line is not None:
        print(json.dumps(line))
    return 0


if __name__ == "__main__":
    sys.exit(main())
