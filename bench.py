"""Benchmark: DOF/s of assemble + Dirichlet + Jacobi-PCG to a 1e-10 relative
residual on one GB300, FP32-refined (FP32 cell-local assembly, FP32 inner CG,
FP64 reliable updates; error against the FP64 solve reported) beside plain
FP64, on the P2 diffusion+mass tetrahedral workload
(TetrahedronMesh box of 64^3 cubes, 1,572,864 cells, 2,146,689 dofs; interior
nodes jittered +-0.2h; lognormal(0,1) per-cell diffusion; reaction 1; f = 1;
u = 0 on the boundary; quadrature index 4).

One step = symbolic CSR pattern + numeric assembly + right-hand side +
Dirichlet elimination + PCG, with the mesh, dof map and coefficients already in
HBM (``value``); ``e2e`` repeats the step through the public API starting from
pinned host arrays (upload, mesh topology, dof numbering, boundary flags,
the step, and the solution copied back).  Inputs (a 0.7 GB FP64 matrix) are
larger than the 129 MB L2, so no L2 flush is needed between steps.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--n 64]

Under torchrun every rank runs an independent replica (the path does not
shard across GPUs; see the design notes); ``value`` is the total dofs solved per
second over all ranks, with the slowest rank's time.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = "DOF/s assemble+PCG to 1e-10 rel res, FP32-refined vs FP64 on GB300; serve p50/p99"
# the C2 record's value: FP32 iterations with FP64 reliable updates on the
# FP64-assembled operator (the 1e-10 residual is against that operator)
HEADLINE = "mixed64"
RTOL = 1e-10
Q = 4
CPU_SAMPLE_N = 24
MAXIT = 20000
BATCH_MAXIT = 100000


def read_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            d = json.load(fh)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


# ---------------------------------------------------------------------------
# clocks sampled during the timed region
# ---------------------------------------------------------------------------
class ClockSampler:
    FIELDS = ("uuid,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, uuid=None):
        self.uuid = uuid
        self.proc = None
        self.lines = []
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                                          "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        rows = [[p.strip() for p in ln.split(",")] for ln in self.lines]
        rows = [r for r in rows if len(r) >= 8]
        uuids = sorted({r[0] for r in rows})
        want = None
        if self.uuid:
            key = self.uuid.replace("GPU-", "").lower()
            for u in uuids:
                if key and (key in u.lower() or u.lower().replace("gpu-", "") in key):
                    want = u
        if want is None and len(uuids) == 1:
            want = uuids[0]
        if want is None:
            return None
        for parts in rows:
            if parts[0] != want:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for nm, v in zip(names, parts[4:8]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------------------
# our arm
# ---------------------------------------------------------------------------
def replica_max(torch, dist, v, world, dev):
    """The slowest rank's time: every rank solves its own replica (the path
    has no data exchange between GPUs), so the job ends with the slowest."""
    if world == 1:
        return v
    t = torch.tensor([v], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_value(gdof, world, ms_per_step):
    """Whole-job DOF/s: all ranks' dofs over the slowest rank's step time."""
    return world * gdof / (ms_per_step / 1e3)


def build_problem(torch, F, node_np, cell_np, kappa_np, dev):
    node = torch.as_tensor(node_np, device=dev)
    cell = torch.as_tensor(cell_np, device=dev)
    kappa = torch.as_tensor(kappa_np, device=dev)
    mesh = F.TetrahedronMesh(node, cell)
    space = F.LagrangeFESpace(mesh, p=2)
    space.cell_to_dof()
    from fealpy_gb300.fem import DirichletBC
    bc = DirichletBC(space, gd=0.0)
    return mesh, space, kappa, bc


STAGES = ("assembly (pattern + values)", "rhs", "dirichlet", "solver copy (SELL)", "pcg")


def solve_step(torch, F, space, kappa, bc, mode, profile=False, marks=None, asm_marks=None, graph=True):
    """symbolic + numeric assembly + RHS + Dirichlet + PCG; returns (x, info, A, F).
    ``marks``: optional list receiving a CUDA event after each stage;
    ``asm_marks``: optional list receiving labelled events inside the assembly."""
    from fealpy_gb300.fem import BilinearForm, LinearForm, ScalarDiffusionIntegrator, ScalarMassIntegrator
    from fealpy_gb300.fem import ScalarSourceIntegrator
    from fealpy_gb300.solver import _sell_of

    def mark():
        if marks is not None:
            e = torch.cuda.Event(enable_timing=True)
            e.record()
            marks.append(e)

    mark()
    space._cache.clear()
    bf = BilinearForm(space)
    bf.add_integrator(ScalarDiffusionIntegrator(coef=kappa, q=Q), ScalarMassIntegrator(coef=1.0, q=Q))
    # FP32-refined: FP32 cell-local assembly (factors from the FP64 Jacobian,
    # determinant and inverse of every cell), FP32 inner CG, FP64 refinement
    # "mixed": FP32 cell-local assembly (the FP32 values are the operator);
    # "mixed64": FP64 assembly, FP32 iterations on its rounded copy, FP64
    # residuals with the FP64 values; "fp64": FP64 throughout
    A = bf.assembly(marks=asm_marks, dtype=torch.float32 if mode == "mixed" else torch.float64)
    mark()
    lf = LinearForm(space)
    lf.add_integrator(ScalarSourceIntegrator(1.0, q=Q))
    Fv = lf.assembly()
    mark()
    A2, F2 = bc.apply(A, Fv)
    mark()
    if not mode.startswith("amg"):
        _sell_of(A2, want32=(mode != "fp64"))
    mark()
    if mode.startswith("amg"):
        # FP64 PCG preconditioned by the aggregation AMG V-cycle (set-up inside
        # the step): V-cycle in FP32 ("amg") or FP64 ("amg64")
        s0 = torch.cuda.Event(enable_timing=True)
        s1 = torch.cuda.Event(enable_timing=True)
        s0.record()
        M = F.GAMGSolver(vcycle_f32=(mode == "amg")).setup(A2)
        s1.record()
        x, info = F.cg(A2, F2, M=M, atol=0.0, rtol=RTOL, maxit=MAXIT, returninfo=True, stop="residual")
        info["amg_levels_n"] = [L.n for L in M.levels]
        if marks is not None:
            s1.synchronize()
            info["amg_setup_ms"] = s0.elapsed_time(s1)
    elif mode != "fp64":
        x, info = F.cg_mixed(A2, F2, rtol=RTOL, maxit=MAXIT, returninfo=True, profile=profile, graph=graph)
    else:
        M = F.JacobiPreconditioner().apply(A2)
        x, info = F.cg(A2, F2, M=M, atol=0.0, rtol=RTOL, maxit=MAXIT, returninfo=True, stop="residual",
                       profile=profile, graph=graph)
    mark()
    return x, info, A2, F2


def amg_record(results, fp64, mixed, world, gdof):
    """C2 with the aggregation AMG V-cycle in cg's M slot (GAMGSolver: MIS
    aggregation, Galerkin coarse levels, Chebyshev smoothing; set-up inside the
    step; PCG and its operator FP64): the V-cycle in FP32 and in FP64."""
    out = {}
    for key, mode in (("fp32_vcycle", "amg"), ("fp64_vcycle", "amg64")):
        r = results.get(mode)
        if r is None:
            continue
        out[key] = {"ms_per_step": r["ms_per_step"], "dof_per_s": world * gdof / (r["ms_per_step"] / 1e3),
                    "cg_iters": r["niter"], "true_relres": r["relres"],
                    "max_rel_err_vs_fp64_jacobi": float((r["x"] - fp64["x"]).abs().max() / fp64["x"].abs().max()),
                    "levels_rows": r["amg_levels"], "setup_ms": r["amg_setup_ms"], "stages_ms": r["stages_ms"],
                    "speedup_vs_fp64_jacobi": fp64["ms_per_step"] / r["ms_per_step"],
                    "speedup_vs_fp32_refined_jacobi": mixed["ms_per_step"] / r["ms_per_step"]}
    if "fp32_vcycle" in out and "fp64_vcycle" in out:
        out["speedup_fp32_vcycle_vs_fp64_vcycle"] = results["amg64"]["ms_per_step"] / results["amg"]["ms_per_step"]
    return out or None


# nominal FP64 rate of the part (FMA = 2 flops); FP64 work of the assembly is
# bound by it, not by HBM
FP64_PEAK_TFLOPS = 1.25


def assembly_roofline(rec, NN, NC, ldof, gdof, peak, n_channel=7):
    """Fractions of the numeric assembly (factor + values kernels) and of the
    symbolic phase (adjacency + pattern) of a C2 record, from its stage times
    (FP64 assembly: s = 8).  HBM: B_asm = NC ldof 4 (cell2dof) + NN 3 8
    (vertex coordinates) + NC 8 (cell coefficient) + nnz 8 (values);
    B_pattern = nnz 4 + (n + 1) 8.  FP64 pipe: every local-matrix entry is
    formed once, NC ldof^2 entries of n_channel multiply-adds (factor x table),
    2 NC ldof^2 n_channel flops; at the part's FP64 rate that is the binding
    limit of the FP64 values kernel (the HBM time of its bytes is far shorter)."""
    st = rec["stages_ms"]
    nnz = rec["nnz"]
    b_asm = NC * ldof * 4 + NN * 3 * 8 + NC * 8 + nnz * 8
    b_pat = nnz * 4 + (gdof + 1) * 8
    t_val = st.get("assembly/values", 0.0)
    t_asm = st.get("assembly/factors", 0.0) + t_val
    t_pat = st.get("assembly/adjacency", 0.0) + st.get("assembly/pattern", 0.0)
    out = {}
    for key, b, t, what in (("assembly", b_asm, t_asm, "cell_factors_kernel + assemble_scalar_kernel<double, 10, 0>"),
                            ("pattern", b_pat, t_pat, "adjacency build + pattern passes")):
        ach = b / (t / 1e3) / 1e9 if t > 0 else 0.0
        out[key] = {"kernels": what, "bound": "hbm", "algorithmic_bytes": b, "ms": t, "achieved": ach,
                    "unit": "GB/s", "frac": ach / peak if peak else None}
    flops = 2.0 * NC * ldof * ldof * n_channel
    tf = flops / (t_val / 1e3) / 1e12 if t_val > 0 else 0.0
    out["assembly_fp64"] = {"kernels": "assemble_scalar_kernel<double, 10, 0>", "bound": "fp64",
                            "algorithmic_flops": flops, "ms": t_val, "achieved": tf, "unit": "TFLOP/s",
                            "peak": FP64_PEAK_TFLOPS, "frac": tf / FP64_PEAK_TFLOPS,
                            "peak_source": "nominal FP64 rate of the part"}
    return out


def spmv_roofline(mixed, gdof, n, peak, peak_kind):
    """`roofline` of the C2 record for the dominant kernel, the FP32 PCG SpMV
    (Ap = A p and p.Ap), from the profiling solve's mean launch time, plus the
    whole FP32 iteration over the timed solve."""
    nnz = mixed["nnz"]
    # SpMV algorithmic bytes B_spmv = nnz (s + 4) + n (8 + 2 s) with s = 4:
    # value + column per nonzero, a row pointer, x read once and y written once
    # (the formula of the measurement definition, used verbatim; the SELL copy
    # reads a 4-byte slot->row map and an 8-byte slice pointer per 32 rows in
    # place of the row pointer).  With 2-byte column steps: nnz (s + 2) + n (12 + 2 s).
    # 15-bit steps: E (s + 2) + n (8 + 2 s), E = nonzeros + long-step entries
    # (a 2-byte code and a value each; per row a first column and a slot map
    # entry replace the row pointer)
    cols = mixed["sell_cols"]
    d16 = cols == "d16"
    if cols == "d15":
        bytes_per_launch = mixed["stored_entries"] * (4 + 2) + gdof * (8 + 8)
    elif d16:
        bytes_per_launch = nnz * (4 + 2) + gdof * (12 + 8)
    else:
        bytes_per_launch = nnz * (4 + 4) + gdof * (8 + 8)
    achieved = bytes_per_launch / (mixed["kernel_ms_avg"] / 1e3) / 1e9 if mixed["kernel_ms_avg"] > 0 else 0.0
    # whole FP32 iteration: B_it = B_spmv + 11 n s (the vector traffic of the
    # update kernels), over the live time per iteration of the timed solve (the
    # step minus its non-PCG stages as measured in the profiling solve)
    pre_ms = sum(v for k, v in mixed["stages_ms"].items() if k in STAGES and k != "pcg")
    it_ms = max(mixed["ms_per_step"] - pre_ms, 1e-9) / max(mixed["niter"], 1)
    bytes_per_iter = bytes_per_launch + 11 * gdof * 4
    it_achieved = bytes_per_iter / (it_ms / 1e3) / 1e9
    traffic = None
    tp = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(tp) and n == 64:
        try:
            traffic = json.load(open(tp)).get({"d16": "pcg_spmv_f32_d16_bytes_per_launch_at_n64",
                                               "d15": "pcg_spmv_f32_d15_bytes_per_launch_at_n64"}.get(
                                                  cols, "pcg_spmv_f32_bytes_per_launch_at_n64"))
        except Exception:
            traffic = None
    return {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak if peak else None, "traffic": traffic,
            "kernel": ("sell_d15_pipe<PipePcg> (SELL-32, 15-bit column steps, next trip loaded before the "
                       "current one is gathered; Ap = A p and p.Ap)" if cols == "d15" else
                       "sell_pcg_spmv<float> (SELL-32" + {"d16": ", 16-bit column steps"}.get(cols, "") +
                       "; Ap = A p and p.Ap)"),
            "algorithmic_bytes_per_launch": bytes_per_launch, "avg_launch_ms": mixed["kernel_ms_avg"],
            "bytes_with_4_byte_columns": nnz * (4 + 4) + gdof * (8 + 8),
            "peak_source": peak_kind,
            "iteration": {"bytes_per_iteration": bytes_per_iter, "us_per_iteration": it_ms * 1e3,
                          "achieved": it_achieved, "unit": "GB/s", "frac": it_achieved / peak if peak else None}}


def run_ours(args):
    import torch
    import torch.distributed as dist
    import fealpy_gb300 as F
    from fealpy_gb300 import _lib
    from fealpy_gb300.workloads import diffusion_mass_tet_box

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)

    from fealpy_gb300 import solver as SV
    SV.SELL_D16 = {"auto": None, "i32": False, "d16": True, "d15": False}[args.sell_cols]
    SV.SELL_D15 = args.sell_cols == "d15"
    n = args.n
    node_np, cell_np, kappa_np = diffusion_mass_tet_box(n)
    mesh, space, kappa, bc = build_problem(torch, F, node_np, cell_np, kappa_np, dev)
    gdof = space.number_of_global_dofs()
    stream = torch.cuda.current_stream(dev)

    def barrier():
        torch.cuda.synchronize(dev)
        if world > 1:
            dist.barrier()

    def max_over_ranks(v):
        return replica_max(torch, dist, v, world, dev)

    results = {}
    modes = [m for m in args.modes.split(",") if m]
    for mode in modes:
        for _ in range(args.warmup):
            solve_step(torch, F, space, kappa, bc, mode, graph=not args.no_graph)
        barrier()
        sampler = ClockSampler(getattr(torch.cuda.get_device_properties(dev), "uuid", None) and
                               str(torch.cuda.get_device_properties(dev).uuid)) if mode == HEADLINE else None
        if sampler:
            sampler.start()
            time.sleep(0.3)
        launches0 = _lib.launch_count()
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        barrier()
        ev0.record(stream)
        infos = []
        # NVTX range "timed_<mode>" lets a profiler capture exactly the timed steps
        torch.cuda.nvtx.range_push(f"timed_{mode}")
        for _ in range(args.steps):
            x, info, A2, F2 = solve_step(torch, F, space, kappa, bc, mode, profile=False, graph=not args.no_graph)
            infos.append(info)
        ev1.record(stream)
        torch.cuda.nvtx.range_pop()
        barrier()
        ms = ev0.elapsed_time(ev1)
        clocks = sampler.stop() if sampler else None
        launches = _lib.launch_count() - launches0
        ms = max_over_ranks(ms)
        # true relative residual in FP64 arithmetic for the operator solved
        A64 = F.CSRTensor(A2.crow, A2.col, A2.values.to(torch.float64), A2.shape)
        F64 = F2.to(torch.float64)
        r = F64 - A64 @ x
        relres = float(torch.linalg.norm(r) / torch.linalg.norm(F64))
        # SpMV kernel duration: one more solve with CUDA events around every
        # SpMV launch (host-polled loop, same kernels as the graph loop)
        marks, amarks = [], []
        _, pinfo, _, _ = solve_step(torch, F, space, kappa, bc, mode, profile=True, marks=marks, asm_marks=amarks)
        torch.cuda.synchronize(dev)
        stages = {name: marks[k].elapsed_time(marks[k + 1]) for k, name in enumerate(STAGES)}
        for k in range(1, len(amarks)):
            stages["assembly/" + amarks[k][0]] = amarks[k - 1][1].elapsed_time(amarks[k][1])
        kms = pinfo.get("kernel_ms", 0.0)
        kl = pinfo.get("kernel_launches", 0)
        results[mode] = {"ms": ms, "ms_per_step": ms / args.steps, "x": x, "relres": relres,
                         "niter": infos[-1]["niter"], "n_updates": infos[-1].get("n_updates", 0),
                         "kernel_ms_avg": kms / max(kl, 1), "kernel_launches": kl, "launches": launches,
                         "other_ms_avg": pinfo.get("other_ms", 0.0) / max(kl, 1),
                         "extra_ms_avg": pinfo.get("extra_ms", 0.0) / max(kl, 1), "stages_ms": stages,
                         "amg_levels": infos[-1].get("amg_levels_n"), "amg_setup_ms": pinfo.get("amg_setup_ms"),
                         "clocks": clocks, "nnz": A2.nnz, "n": gdof,
                         "sell_launch": list(A2._sell.launch) if getattr(A2, "_sell", None) is not None else None,
                         "sell_cols": A2._sell.cols if getattr(A2, "_sell", None) is not None else None,
                         "stored_entries": A2._sell.stored_entries() if getattr(A2, "_sell", None) is not None
                         else A2.nnz, "A2": A2, "F2": F2}

    if not {"fp64", "mixed", HEADLINE} <= set(modes) or args.no_e2e:
        # profiling run: report the per-mode timings on stderr only
        for m, r in results.items():
            print(f"[profile run] {m}: {r['ms_per_step']:.3f} ms/step, {r['niter']} iterations, "
                  f"relres {r['relres']:.3e}, spmv avg {r['kernel_ms_avg'] * 1e3:.1f} us, update "
                  f"{r['other_ms_avg'] * 1e3:.1f} us, other {r['extra_ms_avg'] * 1e3:.1f} us, cols {r['sell_cols']}, "
                  f"stages {json.dumps(r['stages_ms'])}", file=sys.stderr)
        if world > 1:
            dist.destroy_process_group()
        return
    x64 = results["fp64"]["x"]
    A64op, F64op = results["fp64"]["A2"], results["fp64"]["F2"]
    # each FP32-refined solution against the FP64-assembled operator and the
    # FP64 solution
    for m in ("mixed", "mixed64"):
        if m in results:
            xm = results[m]["x"]
            results[m]["err_vs_fp64"] = float(torch.max(torch.abs(xm - x64)) / torch.max(torch.abs(x64)))
            results[m]["relres_vs_fp64_operator"] = float(torch.linalg.norm(F64op - A64op @ xm) /
                                                         torch.linalg.norm(F64op))
    err = results[HEADLINE]["err_vs_fp64"]

    # e2e: from pinned host arrays through the public API, solution back to host
    node_h = torch.as_tensor(node_np).pin_memory()
    cell_h = torch.as_tensor(cell_np).pin_memory()
    kappa_h = torch.as_tensor(kappa_np).pin_memory()
    x_h = torch.empty(gdof, dtype=torch.float64).pin_memory()

    def e2e_step():
        nd = node_h.to(dev, non_blocking=True)
        cl = cell_h.to(dev, non_blocking=True)
        kp = kappa_h.to(dev, non_blocking=True)
        m = F.TetrahedronMesh(nd, cl)
        sp_ = F.LagrangeFESpace(m, p=2)
        from fealpy_gb300.fem import DirichletBC
        bc_ = DirichletBC(sp_, gd=0.0)
        x, info, _, _ = solve_step(torch, F, sp_, kp, bc_, HEADLINE)
        x_h.copy_(x, non_blocking=True)
        torch.cuda.synchronize(dev)

    e2e_step()
    barrier()
    t0 = time.perf_counter()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    e2e_steps = max(1, min(args.steps, 3))
    for _ in range(e2e_steps):
        e2e_step()
    e1.record(stream)
    barrier()
    e2e_ms = max_over_ranks(max(e0.elapsed_time(e1), (time.perf_counter() - t0) * 1e3))
    h2d = node_np.nbytes + cell_np.nbytes + kappa_np.nbytes
    d2h = gdof * 8

    peak, peak_kind = read_peaks()
    mixed = results[HEADLINE]
    m32 = results["mixed"]
    fp64 = results["fp64"]
    value = replica_value(gdof, world, mixed["ms_per_step"])
    roofline = spmv_roofline(mixed, gdof, n, peak, peak_kind)
    roofline.update(assembly_roofline(mixed, node_np.shape[0], cell_np.shape[0], space.number_of_local_dofs(),
                                      gdof, peak))

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline(CPU_SAMPLE_N, rounds=2)

    # the other configurations, one step each, on rank 0 of a single-GPU run:
    # C5 elasticity 128^3, C3 batched meshes, C4 serving at two arrival rates
    extras = {}
    if rank == 0 and world == 1 and not args.no_extras:
        ex_args = argparse.Namespace(**vars(args))
        ex_args.steps, ex_args.warmup = 1, 1
        jobs = [("elasticity", lambda: elasticity_record(ex_args)), ("batched", lambda: batched_record(ex_args))]
        if not args.no_serving:
            jobs.append(("serving", lambda: serving_record(ex_args, [100.0, 1000.0], args.serve_count)))
        for key, fn in jobs:
            t0 = time.perf_counter()
            try:
                extras[key] = fn()
            except Exception as e:  # recorded, so that one configuration cannot void the record
                extras[key] = {"error": f"{type(e).__name__}: {e}"}
            extras[key]["wall_s"] = time.perf_counter() - t0

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "DOF/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": mixed["ms_per_step"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64",
            "data": "synthetic (seeded jittered tet box, lognormal coefficients)",
            "config": {"workload": f"P2 diffusion+mass TetrahedronMesh box {n}^3 (C2)", "cells": int(cell_np.shape[0]),
                       "gdof": gdof, "nnz": mixed["nnz"], "quadrature": Q, "rtol": RTOL,
                       "l2": "inputs larger than L2 (no flush)", "parallelism": f"replicas x{world}"},
            "headline": "fp32_refined_fp64_operator: FP64 cell-local assembly, FP32 inner CG on its FP32 copy, "
                        "FP64 reliable updates with the FP64 values; the variant whose 1e-10 relative residual is "
                        "against the FP64-assembled operator",
            "fp32_refined_fp64_operator": {
                "ms_per_step": mixed["ms_per_step"], "dof_per_s": value, "cg_iters": mixed["niter"],
                "reliable_updates": mixed["n_updates"], "true_relres_vs_fp64_operator": mixed["relres"],
                "max_rel_err_vs_fp64": mixed["err_vs_fp64"], "stages_ms": mixed["stages_ms"],
                "spmv_us": mixed["kernel_ms_avg"] * 1e3, "update_us": mixed["other_ms_avg"] * 1e3,
                "other_kernels_us": mixed["extra_ms_avg"] * 1e3, "sell_launch_threads_blocks": mixed["sell_launch"],
                "sell_columns": mixed["sell_cols"], "sell_stored_entries": mixed["stored_entries"]},
            "fp32_refined": {"operator": "FP32-assembled (FP32 cell-local assembly from the FP64 geometry)",
                             "ms_per_step": m32["ms_per_step"], "dof_per_s": world * gdof / (m32["ms_per_step"] / 1e3),
                             "cg_iters": m32["niter"], "reliable_updates": m32["n_updates"],
                             "true_relres": m32["relres"], "true_relres_vs_fp64_operator": m32["relres_vs_fp64_operator"],
                             "max_rel_err_vs_fp64": m32["err_vs_fp64"], "stages_ms": m32["stages_ms"],
                             "spmv_us": m32["kernel_ms_avg"] * 1e3, "update_us": m32["other_ms_avg"] * 1e3,
                             "other_kernels_us": m32["extra_ms_avg"] * 1e3,
                             "sell_launch_threads_blocks": m32["sell_launch"], "sell_columns": m32["sell_cols"],
                             "sell_stored_entries": m32["stored_entries"],
                             "speedup_vs_fp64": fp64["ms_per_step"] / m32["ms_per_step"]},
            "fp64": {"ms_per_step": fp64["ms_per_step"], "dof_per_s": world * gdof / (fp64["ms_per_step"] / 1e3),
                     "cg_iters": fp64["niter"], "true_relres": fp64["relres"], "stages_ms": fp64["stages_ms"],
                     "spmv_us": fp64["kernel_ms_avg"] * 1e3, "update_us": fp64["other_ms_avg"] * 1e3,
                     "other_kernels_us": fp64["extra_ms_avg"] * 1e3,
                     "sell_launch_threads_blocks": fp64["sell_launch"], "sell_columns": fp64["sell_cols"]},
            "speedup_fp32_refined_vs_fp64": fp64["ms_per_step"] / mixed["ms_per_step"],
            "amg": amg_record(results, fp64, mixed, world, gdof),
            "e2e": {"value": world * gdof * e2e_steps / (e2e_ms / 1e3), "unit": "DOF/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h, "steps": e2e_steps},
            "gpu_launches": mixed["launches"],
            "roofline": roofline,
            "clocks": mixed["clocks"],
            "cpu_baseline": cpu,
        }
        line.update(extras)
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.barrier()
        dist.destroy_process_group()


# ---------------------------------------------------------------------------
# CPU reference (the oracle: numpy/scipy restatement of the reference path)
# ---------------------------------------------------------------------------
def oracle_step(n):
    from oracle import fem_oracle as O
    from fealpy_gb300.workloads import diffusion_mass_tet_box
    node, cell, kappa = diffusion_mass_tet_box(n)
    t0 = time.perf_counter()
    out = O.poisson_pipeline(node, cell, 2, kappa=kappa, rho=1.0, q=Q, rtol=RTOL)
    dt = time.perf_counter() - t0
    return out["n"], dt, out["info"]["niter"]


# at most this many concurrent replicas of the host sample
REF_MAX_PROCS = 64


def _oracle_worker(n):
    return oracle_step(n)


def host_replica_rounds(n, rounds, warmup=1):
    """Whole-host throughput of the reference path: as many concurrent
    single-threaded replicas of the n^3 sample as the host has cores (spawned
    processes, one BLAS thread each), `rounds` timed rounds after `warmup`
    untimed ones.  Returns (processes, dofs per replica, seconds per round,
    PCG iterations)."""
    import multiprocessing
    procs = max(1, min(os.cpu_count() or 1, REF_MAX_PROCS))
    try:
        return _replica_rounds(n, rounds, warmup, procs, multiprocessing)
    except Exception as e:  # no process pool here: one replica in this process
        print(f"[cpu baseline] process pool unavailable ({e}); one replica in-process", file=sys.stderr)
        for _ in range(max(warmup, 1)):
            oracle_step(n)
        times, gdof, niter = [], 0, 0
        for _ in range(rounds):
            gdof, dt, niter = oracle_step(n)
            times.append(dt)
        return 1, gdof, times, niter


def _replica_rounds(n, rounds, warmup, procs, multiprocessing):
    saved = {k: os.environ.get(k) for k in ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS", "MKL_NUM_THREADS")}
    for k in saved:
        os.environ[k] = "1"  # inherited by the spawned replicas
    try:
        ctx = multiprocessing.get_context("spawn")
        with ctx.Pool(procs) as pool:
            for _ in range(max(warmup, 1)):
                pool.map(_oracle_worker, [n] * procs)
            times = []
            gdof = niter = 0
            for _ in range(rounds):
                t0 = time.perf_counter()
                res = pool.map(_oracle_worker, [n] * procs)
                times.append(time.perf_counter() - t0)
                gdof, niter = res[0][0], res[0][2]
    finally:
        for k, v in saved.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v
    return procs, gdof, times, niter


def cpu_baseline(n, rounds=2):
    """The oracle port's whole-host throughput on the n^3 sample (see
    host_replica_rounds); also the single-replica time of a round."""
    procs, gdof, times, niter = host_replica_rounds(n, rounds, warmup=1)
    t = statistics.median(times)
    return {"value": procs * gdof / t, "unit": "DOF/s", "cores": procs, "kind": "port",
            "sample": f"{procs} concurrent single-threaded replicas (spawned processes, one BLAS thread each) of the "
                      f"P2 diffusion+mass tet box {n}^3 ({gdof} dofs, {niter} PCG iterations), median of {rounds} "
                      f"rounds; numpy/scipy oracle restating the reference numpy path (einsum, lexsort+add.at "
                      f"coalesce, scipy csr_matvec CG)",
            "seconds_per_round": t}


# the reference arm: at most this much host time on timed steps (a full
# assemble + Dirichlet + PCG solve of the 64^3 system per step)
REF_TIME_BUDGET_S = 150.0


def _mem_available_gb():
    try:
        with open("/proc/meminfo") as fh:
            for ln in fh:
                if ln.startswith("MemAvailable:"):
                    return int(ln.split()[1]) / 1e6
    except Exception:
        pass
    return None


def run_reference(args):
    """The reference algorithm (the oracle port of FEALPy's numpy path) on the
    same configuration as our arm: P2 diffusion + mass on the n^3 tet box,
    full assembly + right-hand side + Dirichlet + Jacobi-PCG to 1e-10 per
    step, split over the host's cores (processes over row ranges, threads
    over row blocks in the CG products; results bit-identical to the
    sequential oracle).  One untimed warm-up step (worker set-up: mesh,
    topology, dof numbering, as excluded from our arm's value), then as many
    timed steps as fit in REF_TIME_BUDGET_S, at least one."""
    import multiprocessing
    import resource
    from oracle import parallel_port as PP
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    n = args.n
    cores = PP.host_cores()
    avail = _mem_available_gb()
    # about 3 GB per worker at 64^3 (set-up + one row range), scaled by size
    per_worker = 3.0 * (n / 64.0) ** 3
    procs = cores if avail is None else max(1, min(cores, int((avail - 20.0 * (n / 64.0) ** 3) / per_worker)))
    saved = {k: os.environ.get(k) for k in ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS", "MKL_NUM_THREADS")}
    for k in saved:
        os.environ[k] = "1"
    ctx = multiprocessing.get_context("spawn")
    gdof = (2 * n + 1) ** 3
    times, stages, niter = [], [], 0
    try:
        with ctx.Pool(procs) as pool:
            t_w = time.perf_counter()
            PP.assemble(pool, "c2", n, gdof, 4 * procs)  # warm-up: builds the set-up in every worker
            warm_s = time.perf_counter() - t_w
            want = max(1, args.steps)
            while len(times) < want:
                t0 = time.perf_counter()
                out = PP.assemble(pool, "c2", n, gdof, 4 * procs)
                t1 = time.perf_counter()
                A = PP.BlockOperator(out["blocks"], out["bounds"], cores)
                try:
                    x, info = PP.jacobi_cg(A, out["b"], atol=1e-30, rtol=RTOL)
                finally:
                    A.close()
                t2 = time.perf_counter()
                times.append(t2 - t0)
                niter = info["niter"]
                stages.append({"assembly_rhs_dirichlet_s": t1 - t0, "pcg_s": t2 - t1,
                               "worker_setup_in_step_s": out["setup_s"]})
                if sum(times) + times[-1] > REF_TIME_BUDGET_S:
                    break
    finally:
        for k, v in saved.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v
    rss = max(resource.getrusage(resource.RUSAGE_SELF).ru_maxrss, resource.getrusage(resource.RUSAGE_CHILDREN).ru_maxrss)
    tot = sum(times)
    value = gdof * len(times) / tot
    sample = (f"full C2 step at {n}^3 ({gdof} dofs): assembly + right-hand side + Dirichlet + Jacobi-PCG to "
              f"{RTOL:g} ({niter} iterations) per step; {procs} processes over row ranges, {cores} threads in "
              f"the CG products; {len(times)} timed step(s) after 1 untimed warm-up ({warm_s:.1f} s, includes "
              f"the workers' mesh/topology/dof set-up)")
    line = {"metric": METRIC, "value": value, "unit": "DOF/s", "n_gpus": world, "steps": len(times),
            "warmup": 1, "requested_steps": args.steps, "requested_warmup": args.warmup,
            "ms_per_step": tot / len(times) * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic (seeded jittered tet box, lognormal coefficients)", "impl": "reference",
            "config": {"workload": f"P2 diffusion+mass TetrahedronMesh box {n}^3 (C2)", "gdof": gdof, "quadrature": Q,
                       "rtol": RTOL, "same_config": True},
            "stages": stages, "peak_rss_gb": rss / 1e6, "host_cores": cores, "mem_available_gb": avail,
            "cpu_baseline": {"value": value, "unit": "DOF/s", "cores": cores, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": "DOF/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# batched workload: 256 uneven triangle meshes, P1-P3, one graph loop
# ---------------------------------------------------------------------------
def batched_setup(torch, F, meshes, dev):
    """Mesh upload, topology and dof numbering (outside the timed region, as
    for the single-mesh workload)."""
    from fealpy_gb300.fem import DirichletBC
    probs = []
    for m in meshes:
        mesh = F.TriangleMesh(torch.as_tensor(m["node"], device=dev), torch.as_tensor(m["cell"], device=dev))
        space = F.LagrangeFESpace(mesh, p=m["p"])
        space.cell_to_dof()
        probs.append((space, torch.as_tensor(m["kappa"], device=dev), DirichletBC(space, gd=0.0), m["p"]))
    return probs


# precision "auto" of the batched workload: P3 systems above this many dofs
# iterate in FP64 from the start (their condition numbers are beyond what FP32
# iterations resolve: with "mixed" exactly these systems stagnate in FP32 and
# are continued in FP64), all others FP32-refined
AUTO_FP64_P3_DOFS = 100_000
# batched workload, multigrid-lane variant: systems of at least this many dofs
# are solved by multigrid PCG beside the batch
BATCH_LANE_MIN_DOFS = 100_000


def batched_assembler(probs):
    """The batched assembly of the problems (forms built once: diffusion with
    the checkerboard coefficient, quadrature p + 3, f = 1, u = 0)."""
    from fealpy_gb300.fem import BilinearForm, LinearForm, ScalarDiffusionIntegrator, ScalarSourceIntegrator
    from fealpy_gb300.fem.batch_assembly import BatchAssembler
    systems = []
    for space, kappa, bc, p in probs:
        bf = BilinearForm(space)
        bf.add_integrator(ScalarDiffusionIntegrator(coef=kappa, q=p + 3))
        lf = LinearForm(space)
        lf.add_integrator(ScalarSourceIntegrator(1.0, q=p + 3))
        systems.append((bf, lf, bc))
    return BatchAssembler(systems)


def batched_step(torch, F, probs, dtype, bs_kw, marks=None, fp64=False, graph=True, lane_min_dofs=None,
                 assembler=None, stats=None):
    """Assemble every problem (diffusion with the checkerboard coefficient,
    quadrature p + 3, f = 1, u = 0) and solve all of them in one batch.
    ``fp64``: False, True or "auto" (see AUTO_FP64_P3_DOFS).  With
    ``lane_min_dofs``, systems of at least that many dofs are solved by
    multigrid PCG on worker streams beside the batch instead."""
    from fealpy_gb300.fem import BilinearForm, LinearForm, ScalarDiffusionIntegrator, ScalarSourceIntegrator
    from fealpy_gb300.batch import BatchSolver, solve_with_multigrid_lane
    bs = BatchSolver(len(probs), **bs_kw)
    systems = []
    lane = []
    if assembler is not None:
        # every mesh of a degree assembled together: a few launches per degree
        from fealpy_gb300 import _lib as L
        l0 = L.launch_count()
        ea, eb = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ea.record()
        built = assembler.assemble(dtype)
        eb.record()
        if stats is not None:
            eb.synchronize()
            stats["assembly_launches"] = L.launch_count() - l0
            stats["assembly_ms"] = ea.elapsed_time(eb)
    else:
        built = []
        for k, (space, kappa, bc, p) in enumerate(probs):
            space._cache.clear()
            bf = BilinearForm(space)
            bf.add_integrator(ScalarDiffusionIntegrator(coef=kappa, q=p + 3))
            lf = LinearForm(space)
            lf.add_integrator(ScalarSourceIntegrator(1.0, q=p + 3))
            built.append(bc.apply(bf.assembly(dtype=dtype), lf.assembly()))
    for k, (space, kappa, bc, p) in enumerate(probs):
        A2, F2 = built[k]
        systems.append((A2, F2))
        if lane_min_dofs is not None and A2.shape[0] >= lane_min_dofs:
            lane.append((k, A2, F2, RTOL, BATCH_MAXIT))
            continue
        sys64 = (p == 3 and A2.shape[0] > AUTO_FP64_P3_DOFS) if fp64 == "auto" else bool(fp64)
        bs.add(A2, F2, rtol=RTOL, maxit=BATCH_MAXIT, key=k, fp64=sys64)
    if marks is not None:
        e = torch.cuda.Event(enable_timing=True)
        e.record()
        marks.append(e)
    if lane:
        res = solve_with_multigrid_lane(bs, lane, graph=graph)
    else:
        res = bs.solve_all(graph=graph)
    return res, systems, bs


def cpu_sample_batched(meshes, budget_s=15.0, max_dofs=80000):
    """The oracle port of the reference numpy path, one mesh after another
    (the reference has no batched solve), on the smallest meshes of the
    batch until about ``budget_s`` of host time: DOF/s of that sample."""
    from oracle import fem_oracle as O
    order = sorted(range(len(meshes)), key=lambda k: (meshes[k]["p"] * meshes[k]["nx"]) ** 2)
    dofs, t, used = 0, 0.0, 0
    for k in order:
        m = meshes[k]
        if (m["p"] * m["nx"] + 1) ** 2 > max_dofs or t > budget_s:
            break
        t0 = time.perf_counter()
        out = O.poisson_pipeline(m["node"], m["cell"], m["p"], kappa=m["kappa"], q=m["p"] + 3, rtol=RTOL)
        t += time.perf_counter() - t0
        dofs += out["n"]
        used += 1
    return {"value": dofs / t if t > 0 else None, "unit": "DOF/s", "cores": os.cpu_count(), "kind": "port",
            "sample": f"{used} smallest meshes of the batch solved one after another ({dofs} dofs, {t:.1f} s)"}


def run_batched(args):
    print(json.dumps(batched_record(args)), flush=True)


def batched_record(args):
    import torch
    import fealpy_gb300 as F
    from fealpy_gb300.workloads import batched_tri_meshes
    from fealpy_gb300.batch import autotune
    from fealpy_gb300 import _lib
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    # FP64 cell-local assembly for the batched meshes: the P3 systems reach
    # condition numbers where an FP32-assembled operator is 1e-3 away from the
    # FP64 one; the iterations still run in FP32 (FP64 continuation where they
    # stall), the refinement in FP64
    asm_dtype = torch.float64
    meshes = batched_tri_meshes(args.batch_count)
    probs = batched_setup(torch, F, meshes, dev)
    asm = batched_assembler(probs)
    gdof = sum(pr[0].number_of_global_dofs() for pr in probs)
    # tile capacity for the finest candidate split (4 slices of 32 rows per
    # tile) plus one partial tile per system
    kw = dict(max_slice_tiles=gdof // 128 + 2 * len(probs) + 1024, max_row_tiles=1 << 18)
    # autotune the slice tiling on the first step's systems
    res, systems, _ = batched_step(torch, F, probs, asm_dtype, kw, assembler=asm)
    times = autotune(systems[:64], device=dev, **kw)
    spt, thr = min(times, key=times.get)
    kw.update(slices_per_tile=spt, slice_threads=thr)
    for _ in range(max(args.warmup - 1, 0)):
        batched_step(torch, F, probs, asm_dtype, kw, assembler=asm)
    torch.cuda.synchronize()
    l0 = _lib.launch_count()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    marks = []
    asm_stats = {}
    e0.record()
    torch.cuda.nvtx.range_push("timed_batched")
    for _ in range(args.steps):
        prec = {"mixed": False, "fp64": True, "auto": "auto"}[args.batch_precision]
        res, systems, bs = batched_step(torch, F, probs, asm_dtype, kw, marks, fp64=prec,
                                        graph=not args.no_graph, assembler=asm, stats=asm_stats)
    e1.record()
    torch.cuda.nvtx.range_pop()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / args.steps
    solve_ms = marks[-1].elapsed_time(e1)
    rel, err, iters = [], [], []
    for k, (A2, F2) in enumerate(systems):
        r = res[k]
        Ad = F.CSRTensor(A2.crow, A2.col, A2.values.to(torch.float64), A2.shape)
        bd = F2.to(torch.float64)
        rel.append(float(torch.linalg.norm(bd - Ad @ r.x) / torch.linalg.norm(bd)))
        iters.append(r.niter)
    # error of the FP32-assembled solve against the FP64 pipeline, on a sample
    for k in range(0, len(probs), max(len(probs) // 8, 1)):
        space, kappa, bc, p = probs[k]
        from fealpy_gb300.fem import BilinearForm, LinearForm, ScalarDiffusionIntegrator, ScalarSourceIntegrator
        bf = BilinearForm(space)
        bf.add_integrator(ScalarDiffusionIntegrator(coef=kappa, q=p + 3))
        lf = LinearForm(space)
        lf.add_integrator(ScalarSourceIntegrator(1.0, q=p + 3))
        A64, F64 = bc.apply(bf.assembly(), lf.assembly())
        x64 = F.cg(A64, F64, M=F.JacobiPreconditioner().apply(A64), atol=0.0, rtol=1e-12, maxit=MAXIT,
                   stop="residual")
        err.append(float((res[k].x - x64).abs().max() / x64.abs().max()))
    line = {"metric": "DOF/s batched assemble+PCG to 1e-10 rel res (256 uneven tri meshes, P1-P3)",
            "value": gdof / (ms / 1e3), "unit": "DOF/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64",
            "data": "synthetic (seeded meshes, checkerboard coefficients)",
            "config": {"workload": f"{len(probs)} TriangleMesh boxes nx log-uniform [16,512], p in {{1,2,3}} (C3)",
                       "iterations": args.batch_precision,
                       "gdof": gdof, "rtol": RTOL, "autotune_us": {f"{a}x{b}": t for (a, b), t in times.items()},
                       "slices_per_tile": spt, "slice_threads": thr},
            "solve_ms": solve_ms, "assembly_ms": ms - solve_ms, "graph": bs.used_graph,
            "batched_assembly": {"ms": asm_stats.get("assembly_ms"), "launches": asm_stats.get("assembly_launches"),
                                 "what": "pattern, factors, values, right-hand side, Dirichlet and split of all "
                                         "256 systems, grouped by degree (fem.batch_assembly.BatchAssembler)"},
            "fp64_continuations": bs.fallbacks,
            "fp64_iterations": sum(getattr(res[k], "fp64_iterations", 0) for k in res),
            "max_true_relres": max(rel), "iters_max": max(iters), "iters_mean": sum(iters) / len(iters),
            "max_rel_err_vs_fp64_sample": max(err), "gpu_launches": (_lib.launch_count() - l0) // args.steps,
            "cpu_baseline": None if args.no_cpu_baseline else cpu_sample_batched(meshes)}
    # variant: the large systems by multigrid PCG beside the batch (the
    # configuration asks for one launch for all 256; this shows what the
    # Jacobi iterations of the largest P3 systems cost)
    prec = {"mixed": False, "fp64": True, "auto": "auto"}[args.batch_precision]
    batched_step(torch, F, probs, asm_dtype, kw, fp64=prec, lane_min_dofs=BATCH_LANE_MIN_DOFS, assembler=asm)
    torch.cuda.synchronize()
    e0.record()
    for _ in range(args.steps):
        res_l, systems_l, _ = batched_step(torch, F, probs, asm_dtype, kw, fp64=prec,
                                           lane_min_dofs=BATCH_LANE_MIN_DOFS, graph=not args.no_graph,
                                           assembler=asm)
    e1.record()
    torch.cuda.synchronize()
    ms_l = e0.elapsed_time(e1) / args.steps
    rel_l = []
    for k, (A2, F2) in enumerate(systems_l):
        Ad = F.CSRTensor(A2.crow, A2.col, A2.values.to(torch.float64), A2.shape)
        bd = F2.to(torch.float64)
        rel_l.append(float(torch.linalg.norm(bd - Ad @ res_l[k].x) / torch.linalg.norm(bd)))
    n_lane = sum(1 for (A2, _) in systems_l if A2.shape[0] >= BATCH_LANE_MIN_DOFS)
    line["multigrid_lane"] = {"lane_min_dofs": BATCH_LANE_MIN_DOFS, "lane_systems": n_lane,
                              "ms_per_step": ms_l, "dof_per_s": gdof / (ms_l / 1e3),
                              "max_true_relres": max(rel_l), "speedup_vs_one_batch": ms / ms_l}
    return line


# ---------------------------------------------------------------------------
# serving workload: Poisson arrivals, continuous batching under a memory budget
# ---------------------------------------------------------------------------
def run_amg(args):
    """The multigrid on the C2 system at ``--n``: one set-up in the NVTX range
    "setup" (after a warm-up one), three V-cycles in the range "vcycles" (for a
    profiler's launch list: the PCG loop runs inside a conditional graph whose
    kernel nodes a profiler does not list), then set-up, V-cycle and PCG times
    by CUDA events.  Prints one JSON line."""
    import torch
    import fealpy_gb300 as F
    from fealpy_gb300.workloads import diffusion_mass_tet_box
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    node_np, cell_np, kappa_np = diffusion_mass_tet_box(args.n)
    mesh, space, kappa, bc = build_problem(torch, F, node_np, cell_np, kappa_np, dev)
    _, _, A2, F2 = solve_step(torch, F, space, kappa, bc, "fp64")
    F.GAMGSolver().setup(A2)
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_push("setup")
    M = F.GAMGSolver().setup(A2)
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_pop()
    M.vcycle(F2)
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_push("vcycles")
    for _ in range(3):
        M.vcycle(F2)
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_pop()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(6)]
    ev[0].record()
    M = F.GAMGSolver().setup(A2)
    ev[1].record()
    ev[2].record()
    for _ in range(10):
        M.vcycle(F2)
    ev[3].record()
    ev[4].record()
    x, info = F.cg(A2, F2, M=M, atol=0.0, rtol=RTOL, maxit=MAXIT, returninfo=True, stop="residual")
    ev[5].record()
    torch.cuda.synchronize()
    print(json.dumps({"workload": f"multigrid on the P2 diffusion+mass tet box {args.n}^3", "rows": A2.shape[0],
                      "levels_rows": [L.n for L in M.levels], "setup_ms": ev[0].elapsed_time(ev[1]),
                      "vcycle_ms": ev[2].elapsed_time(ev[3]) / 10, "pcg_ms": ev[4].elapsed_time(ev[5]),
                      "pcg_iters": info["niter"]}), flush=True)


def run_elasticity(args):
    print(json.dumps(elasticity_record(args)), flush=True)


def elasticity_record(args):
    """P1 vector linear elasticity on an n^3 tetrahedral box (default 128^3:
    12,582,912 cells, 6,440,067 dofs): lambda = 1, mu = 0.5 scaled per cell by
    exp(N(0, 0.5)), clamped at x = 0, body force (0, 0, -1), q = 4, rtol 1e-8;
    FP32-refined iterations (FP64 operator) beside plain FP64."""
    import torch
    import fealpy_gb300 as F
    from fealpy_gb300.fem import BilinearForm, LinearForm, LinearElasticityIntegrator, VectorSourceIntegrator
    from fealpy_gb300.fem import DirichletBC
    from fealpy_gb300.workloads import elasticity_tet_box
    from fealpy_gb300 import solver as SV
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    SV.SELL_TRIPLES = not args.no_triples
    n = args.elast_n
    node_np, cell_np, scale_np = elasticity_tet_box(n)
    mesh = F.TetrahedronMesh(torch.as_tensor(node_np, device=dev), torch.as_tensor(cell_np, device=dev))
    ts = F.TensorFunctionSpace(F.LagrangeFESpace(mesh, 1), (-1, 3))
    mat = F.LinearElasticMaterial("m", lame_lambda=1.0, shear_modulus=0.5,
                                  cell_scale=torch.as_tensor(scale_np, device=dev))
    bc = DirichletBC(ts, gd=0.0, threshold=lambda x: torch.abs(x[..., 0]) < 1e-12)
    gdof = ts.number_of_global_dofs()
    rtol = 1e-8

    def step(mode):
        bf = BilinearForm(ts)
        bf.add_integrator(LinearElasticityIntegrator(mat, q=4))
        A = bf.assembly()
        lf = LinearForm(ts)
        lf.add_integrator(VectorSourceIntegrator(source=[0.0, 0.0, -1.0], q=4))
        A2, F2 = bc.apply(A, lf.assembly())
        if mode == "mixed":
            x, info = F.cg_mixed(A2, F2, rtol=rtol, maxit=200000, returninfo=True, graph=not args.no_graph)
        elif mode == "amg":
            from fealpy_gb300.amg import multigrid_solve
            x, niter, reason, relres = multigrid_solve(A2, F2, rtol, 200000)
            info = {"niter": niter, "reason": reason, "fp64_iterations": 0}
        else:
            x, info = F.cg(A2, F2, M=F.JacobiPreconditioner().apply(A2), atol=0.0, rtol=rtol, maxit=200000,
                           returninfo=True, stop="residual", graph=not args.no_graph)
        return x, info, A2, F2

    res = {}
    for mode in ("mixed", "fp64", "amg"):
        for _ in range(args.warmup):
            step(mode)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(args.steps):
            x, info, A2, F2 = step(mode)
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / args.steps
        r = F2 - A2 @ x
        res[mode] = {"ms_per_step": ms, "dof_per_s": gdof / (ms / 1e3), "cg_iters": info["niter"],
                     "true_relres": float(torch.linalg.norm(r) / torch.linalg.norm(F2)),
                     "fp64_iterations": info.get("fp64_iterations", info["niter"] if mode == "fp64" else 0),
                     "x": x, "nnz": A2.nnz, "A2": A2, "F2": F2,
                     "sell": A2._sell.cols if getattr(A2, "_sell", None) is not None else None}
    err = float((res["mixed"]["x"] - res["fp64"]["x"]).abs().max() / res["fp64"]["x"].abs().max())
    # roofline of the dominant kernel, the FP32 SpMV of the FP32-refined
    # iterations, from one more (host-polled) solve with CUDA events around
    # every SpMV.  Algorithmic bytes: node-triple copy T (4 + 3 s) + n (8 + 2 s)
    # (a column and three values per triple slot, T = stored triples; a slot
    # map entry and a slice pointer share per row, x read once, y written
    # once); 4-byte columns: nnz (4 + s) + n (8 + 2 s)
    A2 = res["mixed"].pop("A2")
    F2 = res["mixed"].pop("F2")
    for m in ("fp64", "amg"):
        res[m].pop("A2", None)
        res[m].pop("F2", None)
    err_amg = float((res["amg"]["x"] - res["fp64"]["x"]).abs().max() / res["fp64"]["x"].abs().max())
    _, pinfo = F.cg_mixed(A2, F2, rtol=rtol, maxit=200000, returninfo=True, profile=True)
    S = A2._sell
    peak, peak_kind = read_peaks()
    if S.node_triples:
        b = S.stored_entries() * (4 + 3 * 4) + gdof * (8 + 8)
    else:
        b = S.stored_entries() * (4 + 2 if S.d15 else 4 + 4) + gdof * (8 + 8)
    avg = pinfo["kernel_ms"] / max(pinfo["kernel_launches"], 1)
    ach = b / (avg / 1e3) / 1e9 if avg > 0 else 0.0
    roof = {"bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s", "frac": ach / peak, "traffic": None,
            "kernel": f"sell_pcg_spmv<float> ({S.cols}; Ap = A p and p.Ap)", "algorithmic_bytes_per_launch": b,
            "avg_launch_ms": avg, "peak_source": peak_kind}
    for m in res:
        res[m].pop("x")
    line = {"metric": "DOF/s assemble+PCG to 1e-8 rel res, P1 vector elasticity (C5)",
            "value": res["mixed"]["dof_per_s"], "unit": "DOF/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": res["mixed"]["ms_per_step"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64",
            "data": "synthetic (seeded per-cell material scale)",
            "config": {"workload": f"LinearElasticityIntegrator P1 TetrahedronMesh box {n}^3 (C5)",
                       "cells": int(cell_np.shape[0]), "gdof": gdof, "rtol": rtol, "quadrature": 4},
            "fp32_refined": res["mixed"], "fp64": res["fp64"], "max_rel_err_vs_fp64": err,
            "multigrid": dict(res["amg"], preconditioner="aggregation AMG V-cycle (FP32), FP64 PCG",
                              max_rel_err_vs_fp64=err_amg,
                              speedup_vs_fp32_refined=res["mixed"]["ms_per_step"] / res["amg"]["ms_per_step"]),
            "speedup_fp32_refined_vs_fp64": res["fp64"]["ms_per_step"] / res["mixed"]["ms_per_step"],
            "roofline": roof}
    return line


def cpu_sample_serving(reqs, budget_s=15.0, max_dofs=60000):
    """Sequential FIFO replay of the stream's smallest requests with the oracle
    port of the reference numpy path (one solve after another, no overlap):
    DOF/s and seconds per request of that sample."""
    from oracle import fem_oracle as O
    from fealpy_gb300.workloads import tri_box_arrays, tet_box_arrays, jitter_interior
    small = sorted((r for r in reqs if r["dofs"] <= max_dofs), key=lambda r: r["t"])
    dofs, t, used = 0, 0.0, 0
    for r in small:
        if t > budget_s:
            break
        n = r["n"]
        if r["kind"] == "tri":
            node, cell = tri_box_arrays(n, n)
            node = jitter_interior(node, 1.0 / n, 0.15, seed=r["seed"])
        else:
            node, cell = tet_box_arrays(n, n, n)
            node = jitter_interior(node, 1.0 / n, 0.2, seed=r["seed"])
        kappa = np.exp(np.random.default_rng(r["seed"]).normal(0.0, 1.0, cell.shape[0]))
        t0 = time.perf_counter()
        out = O.poisson_pipeline(node, cell, r["p"], kappa=kappa, q=r["p"] + 2, rtol=RTOL)
        t += time.perf_counter() - t0
        dofs += out["n"]
        used += 1
    return {"value": dofs / t if t > 0 else None, "unit": "DOF/s", "cores": os.cpu_count(), "kind": "port",
            "seconds_per_request": t / max(used, 1),
            "sample": f"{used} requests of <= {max_dofs} dofs replayed one after another ({dofs} dofs, {t:.1f} s)"}


def run_serving(args):
    print(json.dumps(serving_record(args, [float(r) for r in args.serve_rates.split(",")], args.serve_count)),
          flush=True)


# serving: requests of at least this many dofs take the multigrid lane in the
# lane variant of the sweep (PCG with the AMG V-cycle beside the batch)
SERVE_AMG_MIN_DOFS = 20_000


def serving_record(args, rates, count):
    import torch
    from fealpy_gb300.serving import SolveServer, poisson_request_problem
    from fealpy_gb300.workloads import serving_requests
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    # warm-up: library load, graph capture, allocator
    warm = serving_requests(8, rate=1e6, seed=99, dof_range=(1e3, 2e4))
    SolveServer(max_slots=8, device=dev).run(warm)
    # and the multigrid lane (its worker and builder threads, streams, sizes)
    warm = serving_requests(24, rate=1e6, seed=98, dof_range=(1e4, 3e5))
    SolveServer(max_slots=8, device=dev, amg_min_dofs=SERVE_AMG_MIN_DOFS).run(warm)
    rows = []
    for rate in rates:
        reqs = serving_requests(count, rate=rate, seed=3)
        for prec, lane in (("mixed", None), ("fp64", None), ("mixed", SERVE_AMG_MIN_DOFS),
                           ("fp64", SERVE_AMG_MIN_DOFS)):
            torch.cuda.synchronize()
            srv = SolveServer(hbm_budget=150e9, max_slots=256, chunk=args.serve_chunk, fp64=(prec == "fp64"),
                              device=dev, amg_min_dofs=lane)
            out = srv.run(reqs, poisson_request_problem)
            rows.append({"rate_rps": rate, "precision": prec,
                         "multigrid_lane_min_dofs": lane, "multigrid_lane_requests": out["amg_lane_requests"],
                         "p50_ms": out["p50_s"] * 1e3,
                         "p99_ms": out["p99_s"] * 1e3, "throughput_rps": out["throughput_rps"],
                         "dofs_per_s": out["dofs_per_s"], "makespan_s": out["makespan_s"],
                         "peak_resident_gb": out["peak_resident_bytes"] / 1e9,
                         "fp64_continuations": out["fp64_continuations"], "max_relres": out["max_relres"]})
            print(json.dumps(rows[-1]), file=sys.stderr, flush=True)
    best = max(r["throughput_rps"] for r in rows if r["precision"] == "mixed" and r["multigrid_lane_min_dofs"] is None)
    best_lane = max((r["throughput_rps"] for r in rows if r["multigrid_lane_min_dofs"] is not None), default=None)
    line = {"metric": "serving: p50/p99 latency and throughput of Poisson solves to 1e-10 (continuous batching)",
            "value": best, "unit": "requests/s", "n_gpus": 1, "steps": len(rows), "warmup": 1,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64 / f64",
            "data": "synthetic request stream (seeded Poisson arrivals, jittered meshes, lognormal coefficients)",
            "config": {"workload": "70% tri P1/P2, 30% tet P1, 1e3-2e6 dofs log-uniform (C4)",
                       "requests_per_rate": count, "hbm_budget_gb": 150, "slots": 256,
                       "chunk_iterations": args.serve_chunk},
            "sweep": rows, "best_throughput_with_multigrid_lane_rps": best_lane,
            "cpu_baseline": None if args.no_cpu_baseline else cpu_sample_serving(
                serving_requests(count, rate=50.0, seed=3))}
    return line


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--n", type=int, default=64)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--modes", default="fp64,mixed,mixed64,amg,amg64",
                    help="solver modes to time (a single-mode run is for profiling and prints no JSON line)")
    ap.add_argument("--no-e2e", action="store_true", help="skip the end-to-end leg (profiling runs)")
    ap.add_argument("--no-graph", action="store_true",
                    help="host-polled solver loop instead of the CUDA-graph loop (profiling runs: a profiler "
                         "cannot capture kernels inside a graph that has conditional nodes)")
    ap.add_argument("--workload", choices=["c2", "batched", "serving", "elasticity", "amg"], default="c2",
                    help="c2: the P2 tet box (default, the headline line); batched: 256 uneven triangle meshes; "
                         "serving: the request stream; elasticity: P1 vector elasticity on a tet box")
    ap.add_argument("--elast-n", type=int, default=128)
    ap.add_argument("--no-triples", action="store_true",
                    help="elasticity: SELL copy with a column per entry instead of one per node triple")
    ap.add_argument("--batch-count", type=int, default=256)
    ap.add_argument("--batch-precision", choices=["mixed", "fp64", "auto"], default="mixed",
                    help="iterations of the batched solve: FP32 with FP64 refinement (default), plain FP64, or auto (FP64 for P3 systems above 1e5 dofs)")
    ap.add_argument("--serve-count", type=int, default=200, help="requests per arrival rate")
    ap.add_argument("--serve-rates", default="50,200,1000")
    ap.add_argument("--serve-chunk", type=int, default=64)
    ap.add_argument("--no-serving", action="store_true", help="skip the serving sweep of the default run")
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the C5, C3 and C4 records of the default run (only the C2 line)")
    ap.add_argument("--sell-cols", choices=["auto", "i32", "d16", "d15"], default="d15",
                    help="column format of the FP32-refined solver's SELL copy: d15 = 15-bit steps in FEALPy's "
                         "numbering (default), i32 = 4-byte columns, d16 = 16-bit steps of a renumbered matrix, "
                         "auto = d16 where its bridges fit; the FP64 solver's copy has 4-byte columns")
    args = ap.parse_args()
    if args.workload == "batched" and args.impl == "ours":
        run_batched(args)
        return
    if args.workload == "serving" and args.impl == "ours":
        run_serving(args)
        return
    if args.workload == "elasticity" and args.impl == "ours":
        run_elasticity(args)
        return
    if args.workload == "amg" and args.impl == "ours":
        run_amg(args)
        return
    if args.warmup < 3 and args.impl == "ours":
        print("warning: fewer than 3 warm-up steps", file=sys.stderr)
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
