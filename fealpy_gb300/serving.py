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
work overlaps on the device with the work already in flight.

Latency of a request = the moment its solution is on the host minus its
arrival time; p50/p99 over all requests and the throughput (requests/s over
the whole stream) are reported by :meth:`SolveServer.run`.
"""
import time
from typing import Callable, Dict, List, Optional

import numpy as np
import torch

from .batch import BatchSolver

__all__ = ["SolveServer", "poisson_request_problem", "resident_estimate"]


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
    ``chunk`` the iterations run between admissions."""

    def __init__(self, *, hbm_budget: float = 150e9, max_slots: int = 256, chunk: int = 64, fp64: bool = False,
                 rtol: float = 1e-10, maxit: int = 100000, device=None, **batch_kw):
        self.device = torch.device(device) if device is not None else torch.device("cuda",
                                                                                   torch.cuda.current_device())
        self.hbm_budget, self.max_slots, self.chunk = float(hbm_budget), int(max_slots), int(chunk)
        self.fp64, self.rtol, self.maxit = bool(fp64), float(rtol), int(maxit)
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
            keep_solutions: bool = False) -> dict:
        """Serve ``requests`` (dicts with arrival time ``t`` in seconds) in
        real time.  ``build(req, device)`` makes the system of a request when
        it is admitted.  Returns latencies (s), p50/p99, throughput and, with
        ``keep_solutions``, every solution on the host."""
        order = sorted(range(len(requests)), key=lambda i: requests[i]["t"])
        queue: List[int] = []
        nxt = 0
        lat: Dict[int, float] = {}
        info: Dict[int, dict] = {}
        sols: Dict[int, np.ndarray] = {}
        pending_sys: Dict[int, tuple] = {}
        t0 = time.perf_counter()
        while len(lat) < len(requests):
            now = time.perf_counter() - t0
            while nxt < len(order) and requests[order[nxt]]["t"] * time_scale <= now:
                queue.append(order[nxt])
                nxt += 1
            # admission: FIFO while a slot and the memory budget allow
            while queue and self.batch.free_slots() > 0:
                i = queue[0]
                if i not in pending_sys:
                    pending_sys[i] = build(requests[i], self.device)
                A, b = pending_sys[i]
                if not self.admit(i, A, b):
                    if self.batch.active() == 0:
                        raise RuntimeError(f"request {i} does not fit in the memory budget")
                    break
                queue.pop(0)
                del pending_sys[i]
            if self.batch.active() == 0:
                if nxt < len(order):
                    wait = requests[order[nxt]]["t"] * time_scale - (time.perf_counter() - t0)
                    if wait > 0:
                        time.sleep(wait)
                continue
            for r in self.batch.step(max_iterations=self.chunk):
                x = r.x.cpu()  # the result on the host ends the request
                done = time.perf_counter() - t0
                lat[r.key] = done - requests[r.key]["t"] * time_scale
                info[r.key] = r.info()
                if keep_solutions:
                    sols[r.key] = x.numpy()
                self.resident -= self._bytes.pop(r.key)
        makespan = time.perf_counter() - t0
        v = np.array([lat[i] for i in range(len(requests))])
        out = {"n": len(requests), "p50_s": float(np.percentile(v, 50)), "p99_s": float(np.percentile(v, 99)),
               "mean_s": float(v.mean()), "throughput_rps": len(requests) / makespan, "makespan_s": makespan,
               "dofs_per_s": float(sum(req.get("dofs", 0) for req in requests) / makespan),
               "peak_resident_bytes": int(self.peak_resident), "fp64_continuations": self.batch.fallbacks,
               "max_relres": max(d["relres"] for d in info.values()), "latencies_s": v.tolist(), "info": info}
        if keep_solutions:
            out["solutions"] = sols
        return out
