"""Serving loop: continuous batching of Poisson solve requests on one GPU (no
FEALPy counterpart; each request is what FEALPy would do with one
``BilinearForm.assembly`` + ``DirichletBC.apply`` + ``fealpy/solver/cg.py``
call).

Requests arrive over time.  The loop admits queued requests into free slots
of a :class:`~fealpy_gb300.batch.BatchSolver` while the device-memory budget
allows (every admitted request keeps its CSR, SELL copy and Krylov vectors
resident until it finishes), runs the batch for a chunk of iterations,
returns the finished solutions to the host, and repeats.  Requests that
arrive while others are iterating join at the next chunk boundary, so their
work overlaps on the device with the work already in flight; their systems
are built ahead by a builder thread on a second CUDA stream while the batch
iterates, and results go back to the host by asynchronous copies.

Latency of a request = the moment its solution is on the host minus its
arrival time; p50/p99 over all requests and the throughput (requests/s over
the whole stream) are reported by :meth:`SolveServer.run`.
"""
import time
from concurrent.futures import Future, ThreadPoolExecutor
from typing import Callable, Dict, List, Optional

import numpy as np
import torch

from .amg import multigrid_solve
from .batch import BatchSolver

__all__ = ["SolveServer", "poisson_request_problem", "resident_estimate", "multigrid_solve"]


def resident_estimate(n: int, nnz: int, fp64: bool) -> int:
    """Device bytes a request keeps resident while admitted: CSR (int64 row
    pointer, int32 columns, values), the SELL copy (about 4% padding), FP64
    b, x and inverse diagonal, and six Krylov vectors."""
    vb = 8 if fp64 else 4
    csr = (n + 1) * 8 + nnz * (4 + vb)
    sell = int(nnz * 1.05) * (4 + (8 if fp64 else 4)) + n * 4 + (n // 32 + 2) * 8
    vec = n * 8 * 3 + n * 6 * (8 if fp64 else 4)
    return csr + sell + vec


def poisson_request_problem(req: dict, device, dtype=torch.float64, inputs: Optional[dict] = None):
    """Build the system of one serving request on the device: a jittered
    TriangleMesh box (P1/P2) or TetrahedronMesh box (P1), lognormal(0, 1)
    per-cell coefficient, f = 1, u = 0 on the boundary; or, for kind
    'elast', P1 vector elasticity on a tetrahedral box (lambda = 1, mu = 0.5
    scaled per cell by a lognormal(0, 0.5) factor, clamped at x = 0, body
    force (0, 0, -1)).  Returns (A, b).  ``inputs`` (a dict), when given,
    receives host copies of the mesh and coefficients (for checking a result
    against another implementation)."""
    from . import TriangleMesh, TetrahedronMesh, LagrangeFESpace
    from .fem import BilinearForm, LinearForm, ScalarDiffusionIntegrator, ScalarSourceIntegrator, DirichletBC
    g = torch.Generator(device="cpu").manual_seed(int(req["seed"]))
    if req["kind"] == "elast":
        from . import TensorFunctionSpace, LinearElasticMaterial
        from .fem import LinearElasticityIntegrator, VectorSourceIntegrator
        n = int(req["n"])
        mesh = TetrahedronMesh.from_box([0, 1, 0, 1, 0, 1], n, n, n, device=device)
        scale = torch.exp(0.5 * torch.randn(mesh.number_of_cells(), generator=g, dtype=torch.float64)).to(device)
        ts = TensorFunctionSpace(LagrangeFESpace(mesh, 1), (-1, 3))
        mat = LinearElasticMaterial("m", lame_lambda=1.0, shear_modulus=0.5, cell_scale=scale)
        if inputs is not None:
            inputs.update(kind="elast", node=mesh.node.cpu().numpy(), cell=mesh.cell.cpu().numpy(), p=1,
                          scale=scale.cpu().numpy())
        bf = BilinearForm(ts)
        bf.add_integrator(LinearElasticityIntegrator(mat, q=4))
        lf = LinearForm(ts)
        lf.add_integrator(VectorSourceIntegrator(source=[0.0, 0.0, -1.0], q=4))
        bc = DirichletBC(ts, gd=0.0, threshold=lambda x: torch.abs(x[..., 0]) < 1e-12)
        return bc.apply(bf.assembly(dtype=dtype), lf.assembly())
    n, p = int(req["n"]), int(req["p"])
    if req["kind"] == "tri":
        mesh = TriangleMesh.from_box([0, 1, 0, 1], n, n, device=device)
        amp = 0.15
    else:
        mesh = TetrahedronMesh.from_box([0, 1, 0, 1, 0, 1], n, n, n, device=device)
        amp = 0.2
    node = mesh.node
    d = (torch.rand(node.shape, generator=g, dtype=torch.float64) * 2.0 - 1.0).to(device) * (amp / n)
    inside = torch.all((node > 1e-12) & (node < 1.0 - 1e-12), dim=1)
    node.add_(d * inside.unsqueeze(1))
    kappa = torch.exp(torch.randn(mesh.number_of_cells(), generator=g, dtype=torch.float64)).to(device)
    if inputs is not None:
        inputs.update(kind=req["kind"], node=node.cpu().numpy(), cell=mesh.cell.cpu().numpy(), p=p,
                      kappa=kappa.cpu().numpy())
    space = LagrangeFESpace(mesh, p=p)
    bf = BilinearForm(space)
    bf.add_integrator(ScalarDiffusionIntegrator(coef=kappa, q=p + 2))
    lf = LinearForm(space)
    lf.add_integrator(ScalarSourceIntegrator(1.0, q=p + 2))
    return DirichletBC(space, gd=0.0).apply(bf.assembly(dtype=dtype), lf.assembly())


class SolveServer:
    """Continuous-batching solve server.

    ``fp64``: plain FP64 PCG for every request (else FP32 iterations with FP64
    refinement, FP64 continuation where FP32 stalls).  ``hbm_budget`` bounds
    the resident bytes of admitted requests; ``max_slots`` the batch size;
    ``chunk`` the iterations run between admissions; ``build_workers``
    threads build queued requests ahead, each on its own high-priority
    stream (measured on the C4 stream with the multigrid lane: 1 builder
    20-26 req/s, 2: 37, 4: 40-47, 6: 49).

    ``amg_min_dofs``: requests of at least this many dofs go to a multigrid
    lane: PCG with the aggregation AMG V-cycle (``GAMGSolver``; FP32 V-cycle,
    or FP64 with ``fp64``), on worker threads with their own CUDA streams,
    beside the batch.  Jacobi needs iterations that grow with the
    mesh size (thousands for the largest requests), the multigrid about sixty;
    the batch keeps the many small requests.  ``amg_workers`` lane requests
    run at once, each on its worker's stream.  A lane result is the same alone
    and in any mix (its hierarchy and iterations depend only on its system)."""

    def __init__(self, *, hbm_budget: float = 150e9, max_slots: int = 256, chunk: int = 64, fp64: bool = False,
                 rtol: float = 1e-10, maxit: int = 100000, device=None, amg_min_dofs: Optional[int] = None,
                 amg_workers: int = 4, build_workers: int = 6, **batch_kw):
        self.device = torch.device(device) if device is not None else torch.device("cuda",
                                                                                   torch.cuda.current_device())
        self.hbm_budget, self.max_slots, self.chunk = float(hbm_budget), int(max_slots), int(chunk)
        self.fp64, self.rtol, self.maxit = bool(fp64), float(rtol), int(maxit)
        # requests of at least this many dofs (the request's "dofs") are solved
        # by the multigrid lane instead of the batch; None: every request in
        # the batch
        self.amg_min_dofs = None if amg_min_dofs is None else int(amg_min_dofs)
        self.amg_workers = max(int(amg_workers), 1)
        self.build_workers = max(int(build_workers), 1)
        kw = dict(max_slice_tiles=1 << 18, max_row_tiles=1 << 18)
        kw.update(batch_kw)
        self.batch = BatchSolver(self.max_slots, device=self.device, **kw)
        self.resident = 0
        self.peak_resident = 0
        self._bytes: Dict[object, int] = {}

    def admit(self, key, A, b) -> bool:
        """Admit one assembled request if a slot and the budget allow."""
        need = resident_estimate(A.shape[0], A.nnz, self.fp64)
        if not self.batch.fits(A.shape[0]) or self.resident + need > self.hbm_budget:
            return False
        self.batch.add(A, b, rtol=self.rtol, maxit=self.maxit, key=key, fp64=self.fp64)
        self._bytes[key] = need
        self.resident += need
        self.peak_resident = max(self.peak_resident, self.resident)
        return True

    def run(self, requests: List[dict], build: Callable = poisson_request_problem, *, time_scale: float = 1.0,
            keep_solutions: bool = False, prefetch: int = 16) -> dict:
        """Serve ``requests`` (dicts with arrival time ``t`` in seconds) in
        real time.  ``build(req, device)`` makes the system of a request.

        Requests are built ahead of admission (up to ``prefetch`` queued ones)
        by a builder thread on its own CUDA stream while the batch iterates on
        the main stream, so that mesh set-up, assembly and boundary conditions
        overlap with the running solves; a built system is admitted after the
        main stream waits on its build event.  Finished solutions are copied
        to pinned host memory asynchronously, and a completion thread records
        the moment each copy lands (latency = that moment minus the arrival).
        Returns latencies (s), p50/p99, throughput and, with
        ``keep_solutions``, every solution on the host."""
        order = sorted(range(len(requests)), key=lambda i: requests[i]["t"])
        queue: List[int] = []
        nxt = 0
        lat: Dict[int, float] = {}
        info: Dict[int, dict] = {}
        sols: Dict[int, np.ndarray] = {}
        futures: Dict[int, Future] = {}
        # high priority: the batch's tile kernels fill every SM, so the build
        # kernels are scheduled first whenever blocks retire between them;
        # one stream per builder thread
        import threading
        build_local = threading.local()
        main_stream = torch.cuda.current_stream(self.device)

        def build_async(req):
            build_stream = getattr(build_local, "stream", None)
            if build_stream is None:
                build_stream = build_local.stream = torch.cuda.Stream(self.device, priority=-1)
            with torch.cuda.stream(build_stream):
                A, b = build(req, self.device)
                ev = torch.cuda.Event()
                ev.record(build_stream)
            return A, b, ev

        def complete(key, x_dev, x_host, ev, arrival):
            ev.synchronize()  # the copy has landed: the request ends here
            lat[key] = time.perf_counter() - t0 - arrival
            if keep_solutions:
                sols[key] = x_host.numpy()
            del x_dev

        lane_local = threading.local()
        lane_done = [0]
        lane_lock = threading.Lock()

        def amg_job(key, A, b, ev, arrival):
            """One request through the multigrid lane: hierarchy, PCG, true
            residual, asynchronous copy; the request ends when the copy lands.
            Each lane worker thread has its own CUDA stream."""
            amg_stream = getattr(lane_local, "stream", None)
            if amg_stream is None:
                amg_stream = lane_local.stream = torch.cuda.Stream(self.device)
            with torch.cuda.stream(amg_stream):
                amg_stream.wait_event(ev)
                x, niter, reason, relres = multigrid_solve(A, b, self.rtol, self.maxit, self.fp64)
                x_host = torch.empty(x.shape, dtype=x.dtype, pin_memory=True)
                x_host.copy_(x, non_blocking=True)
                done = torch.cuda.Event()
                done.record(amg_stream)
            done.synchronize()
            lat[key] = time.perf_counter() - t0 - arrival
            info[key] = {"relres": relres, "niter": niter, "lane": "amg", "reason": reason}
            if keep_solutions:
                sols[key] = x_host.numpy()
            with lane_lock:
                lane_done[0] += 1

        def to_lane(i):
            return self.amg_min_dofs is not None and requests[i].get("dofs", 0) >= self.amg_min_dofs

        builder = ThreadPoolExecutor(self.build_workers)
        finisher = ThreadPoolExecutor(1)
        lane = ThreadPoolExecutor(self.amg_workers)
        done_jobs = []
        lane_jobs = []
        t0 = time.perf_counter()
        try:
            finished = 0
            pending_lane: List[Future] = []
            while finished + lane_done[0] < len(requests):
                for j in [j for j in pending_lane if j.done()]:
                    j.result()  # a failure in the lane surfaces here
                    pending_lane.remove(j)
                now = time.perf_counter() - t0
                while nxt < len(order) and requests[order[nxt]]["t"] * time_scale <= now:
                    queue.append(order[nxt])
                    nxt += 1
                for i in queue[:max(prefetch, 1)]:
                    if i not in futures:
                        futures[i] = builder.submit(build_async, requests[i])
                # admission: FIFO while a slot and the memory budget allow; a
                # request still being built is waited for while the batch runs
                # below half its slots, otherwise it blocks the ones behind it
                # until the next chunk boundary.  Requests of the multigrid
                # lane leave the queue as soon as they are built.
                while queue:
                    i = queue[0]
                    fut = futures[i]
                    if to_lane(i):
                        if not fut.done():
                            break
                        A, b, ev = fut.result()
                        lane_jobs.append(lane.submit(amg_job, i, A, b, ev, requests[i]["t"] * time_scale))
                        pending_lane.append(lane_jobs[-1])
                        queue.pop(0)
                        del futures[i]
                        for j in queue[:max(prefetch, 1)]:
                            if j not in futures:
                                futures[j] = builder.submit(build_async, requests[j])
                        continue
                    if self.batch.free_slots() <= 0:
                        break
                    if not fut.done() and 2 * self.batch.active() >= self.max_slots:
                        break
                    A, b, ev = fut.result()
                    main_stream.wait_event(ev)
                    if not self.admit(i, A, b):
                        if self.batch.active() == 0:
                            raise RuntimeError(f"request {i} does not fit in the memory budget")
                        break
                    queue.pop(0)
                    del futures[i]
                    for j in queue[:max(prefetch, 1)]:
                        if j not in futures:
                            futures[j] = builder.submit(build_async, requests[j])
                if self.batch.active() == 0:
                    if nxt < len(order) and not queue:
                        wait = requests[order[nxt]]["t"] * time_scale - (time.perf_counter() - t0)
                        if wait > 0:
                            time.sleep(min(wait, 0.002) if pending_lane else wait)
                    else:
                        time.sleep(0.0005)  # builds or lane jobs in flight
                    continue
                for r in self.batch.step(max_iterations=self.chunk):
                    x_host = torch.empty(r.x.shape, dtype=r.x.dtype, pin_memory=True)
                    x_host.copy_(r.x, non_blocking=True)
                    ev = torch.cuda.Event()
                    ev.record(main_stream)
                    info[r.key] = r.info()
                    self.resident -= self._bytes.pop(r.key)
                    done_jobs.append(finisher.submit(complete, r.key, r.x, x_host, ev,
                                                     requests[r.key]["t"] * time_scale))
                    finished += 1
            for j in done_jobs:
                j.result()
            for j in lane_jobs:
                j.result()
        finally:
            builder.shutdown(wait=True)
            finisher.shutdown(wait=True)
            lane.shutdown(wait=True)
        makespan = time.perf_counter() - t0
        v = np.array([lat[i] for i in range(len(requests))])
        out = {"n": len(requests), "p50_s": float(np.percentile(v, 50)), "p99_s": float(np.percentile(v, 99)),
               "mean_s": float(v.mean()), "throughput_rps": len(requests) / makespan, "makespan_s": makespan,
               "dofs_per_s": float(sum(req.get("dofs", 0) for req in requests) / makespan),
               "peak_resident_bytes": int(self.peak_resident), "fp64_continuations": self.batch.fallbacks,
               "amg_lane_requests": len(lane_jobs),
               "max_relres": max(d["relres"] for d in info.values()), "latencies_s": v.tolist(), "info": info}
        if keep_solutions:
            out["solutions"] = sols
        return out
