"""Aggregation algebraic multigrid for the ``M`` slot of ``cg``, with the
interface of FEALPy's ``GAMGSolver`` (``fealpy/solver/gamg_solver.py:14-256``:
``GAMGSolver(theta, csize, ..., isolver, maxit, rtol, atol).setup(A)`` then
``solve(b)``; the hierarchy also applies as a preconditioner, ``M @ r``).

FEALPy builds a Ruge-Stuben hierarchy and smooths with Gauss-Seidel sweeps,
both sequential algorithms.  The GB300 hierarchy is built and applied by the
library's kernels (``csrc/amg.cu``): maximal-independent-set aggregation
(a root and its neighbours), Galerkin coarse matrices of the aggregate indicator (summed in a
fixed order: the hierarchy and every V-cycle are deterministic), Chebyshev
smoothing with the diagonal, coarse corrections scaled by ``omega``, and a
Chebyshev solve on the coarsest level.  Each V-cycle is a fixed symmetric
linear map, so it is a valid CG preconditioner; ``cg(A, b, M=amg)`` runs the
whole PCG loop in the library (``fgb_pcg_amg``).
"""
import ctypes
from typing import List, Optional

import torch

from . import _lib
from . import kernels as K
from .sparse import CSRTensor
from ._lib import call, ptr, stream_ptr, workspace, status_word, check_status_word

__all__ = ["GAMGSolver", "AMGPreconditioner", "multigrid_solve"]


class _Level:
    def __init__(self, indptr, indices, values):
        self.indptr, self.indices, self.values = indptr, indices, values
        self.n = indptr.numel() - 1
        self.nnz = indices.numel()
        self.dinv = None
        self.lmax = 0.0
        self.agg = self.member_ptr = self.members = self.values32 = self.dinv32 = self.sell = None
        self.n_coarse = 0


def _level_sell(L: "_Level", with32: bool = True, with64: bool = False):
    """SELL-32 copy of a level with FP32 values for an FP32 V-cycle's sweeps
    and FP64 values for an FP64 V-cycle or PCG's operator: 15-bit column
    steps where every row's columns ascend, else 4-byte columns; the solver's
    autotuned launch shape."""
    from . import solver as _solver
    v64 = L.values if with64 else None
    v32 = L.values32 if with32 else None
    try:
        S = K.sell_build(L.indptr, L.indices, v64, v32, want64=with64, want32=with32, d15=True)
    except _lib.FgbError:
        S = K.sell_build(L.indptr, L.indices, v64, v32, want64=with64, want32=with32, d16=False)
    dt = torch.float32 if with32 else torch.float64
    # the solver's autotuned launch shape when this size was tuned before (the
    # same matrix solved by cg), else the kernels' default shape: a hierarchy
    # is built per system, and timing candidate shapes for every new size
    # would cost more than it saves
    shape = _solver._LAUNCH_CACHE.get((S.n, S.padded_nnz, dt, S.cols))
    if shape is not None:
        S.set_launch(*shape)
    return S


class GAMGSolver:
    """Algebraic multigrid (see the module docstring).

    Parameters as FEALPy's GAMGSolver where they apply: ``theta`` (strength
    threshold of the aggregation graph; 0 takes every nonzero coupling, which
    suits Lagrange matrices of degree 2 and 3 whose couplings change sign),
    ``csize`` (coarsest size), ``ptype`` ('V'), ``sstep`` (Chebyshev degree of
    each smoothing), ``isolver`` ('CG': PCG with the V-cycle, 'MG': V-cycle
    iterations), ``maxit``, ``rtol``, ``atol``.  GB300 additions: ``omega``
    (coarse-correction scale, plain aggregation needs > 1), ``cdeg`` (degree
    of the coarsest Chebyshev solve), ``max_levels``, ``vcycle_f32`` (the
    V-cycle runs in FP32 on FP32 copies of the level matrices; the PCG
    operator and its vectors stay FP64), ``sell_min_rows`` (levels of at
    least this many rows smooth on a SELL-32 copy, 15-bit column steps where
    the columns ascend, instead of the CSR arrays; in either precision),
    ``block_size`` (aggregate whole nodes of a vector space with that many
    interleaved components, as elasticity matrices need)."""

    def __init__(self, theta: float = 0.0, csize: int = 300, ctype: str = "A", itype: str = "T", ptype: str = "V",
                 sstep: int = 3, isolver: str = "CG", maxit: int = 200, csolver: str = "chebyshev",
                 rtol: float = 1e-8, atol: float = 1e-8, omega: float = 1.7, cdeg: int = 16, max_levels: int = 10,
                 vcycle_f32: bool = True, sell_min_rows: int = 1 << 16, block_size: int = 1):
        if ptype != "V":
            raise NotImplementedError("the GB300 multigrid provides V-cycles")
        if isolver not in ("CG", "MG"):
            raise ValueError("isolver must be 'CG' or 'MG'")
        self.theta, self.csize, self.ptype, self.sstep = float(theta), int(csize), ptype, int(sstep)
        self.isolver, self.maxit, self.rtol, self.atol = isolver, int(maxit), float(rtol), float(atol)
        self.omega, self.cdeg, self.max_levels = float(omega), int(cdeg), int(max_levels)
        self.vcycle_f32 = bool(vcycle_f32)
        self.sell_min_rows = int(sell_min_rows)
        self.block_size = max(int(block_size), 1)
        self.levels: List[_Level] = []
        self._desc = None
        self.A = None

    # ------------------------------------------------------------ set-up
    def _aggregate(self, lev: "_Level", dev, st, s):
        """(agg, number of aggregates, 1/a_ii, Chebyshev bound) of a level."""
        lib = _lib.lib()
        n = lev.n
        ws = workspace(lib.fgb_amg_setup_workspace_bytes(n), dev)
        agg = torch.empty(n, dtype=torch.int32, device=dev)
        dinv = torch.empty(n, dtype=torch.float64, device=dev)
        nagg = ctypes.c_int64(0)
        lmax = ctypes.c_double(0.0)
        call("fgb_amg_aggregate", n, ptr(lev.indptr), ptr(lev.indices), ptr(lev.values), self.theta, ptr(agg),
             ctypes.byref(nagg), ptr(dinv), ctypes.byref(lmax), ptr(st), ptr(ws), ws.numel(), s)
        check_status_word("multigrid set-up (the matrix needs a positive diagonal)", st)
        return agg, int(nagg.value), dinv, float(lmax.value)

    def _coarse(self, indptr, indices, values, agg, nc, dev, st, s):
        """P^T A P for the aggregate indicator of ``agg``: (member_ptr, members,
        coarse indptr, indices, values)."""
        lib = _lib.lib()
        n = indptr.numel() - 1
        member_ptr = torch.empty(nc + 1, dtype=torch.int64, device=dev)
        members = torch.empty(max(n, 1), dtype=torch.int32, device=dev)
        cptr = torch.empty(nc + 1, dtype=torch.int64, device=dev)
        cws = workspace(lib.fgb_amg_coarse_workspace_bytes(n, nc), dev)
        nnz = ctypes.c_int64(0)
        call("fgb_amg_coarse_count", n, ptr(indptr), ptr(indices), ptr(values), ptr(agg), nc, ptr(member_ptr),
             ptr(members), ptr(cptr), ctypes.byref(nnz), ptr(st), ptr(cws), cws.numel(), s)
        ccol = torch.empty(max(int(nnz.value), 1), dtype=torch.int32, device=dev)
        cval = torch.empty(max(int(nnz.value), 1), dtype=torch.float64, device=dev)
        call("fgb_amg_coarse_fill", n, ptr(indptr), ptr(indices), ptr(values), ptr(agg), nc, ptr(member_ptr),
             ptr(members), ptr(cptr), ptr(ccol), ptr(cval), ptr(st), ptr(cws), cws.numel(), s)
        check_status_word("multigrid coarse matrix (aggregate rows above the candidate capacity)", st)
        return member_ptr, members, cptr, ccol[: int(nnz.value)], cval[: int(nnz.value)]

    def _block_aggregate(self, lev: "_Level", dev, st, s):
        """Aggregates of whole nodes for a matrix of ``block_size`` interleaved
        components (dof = block_size * node + component): the node graph is
        P_b^T |A| P_b (P_b groups each node's dofs), its aggregates expand to
        one coarse dof per (aggregate, component), so every level keeps the
        interleaved layout."""
        b = self.block_size
        n = lev.n
        _, _, dinv, lmax = self._aggregate(lev, dev, st, s)  # 1/a_ii and the bound of the dof matrix
        dof = torch.arange(n, device=dev, dtype=torch.int32)
        node = dof // b
        absval = lev.values.abs()
        _, _, nptr, ncol, nval = self._coarse(lev.indptr, lev.indices, absval, node, n // b, dev, st, s)
        agg_n, nagg, _, _ = self._aggregate(_Level(nptr, ncol, nval), dev, st, s)
        an = agg_n[node.long()]
        agg = torch.where(an >= 0, an * b + dof % b, an).to(torch.int32).contiguous()
        return agg, nagg * b, dinv, lmax

    def setup(self, A: CSRTensor, P=None, R=None, mesh=None, space=None, cdegree=None):
        """Build the hierarchy of ``A`` (FP64 CSR on the device)."""
        if P is not None or R is not None or mesh is not None or space is not None:
            raise NotImplementedError("the GB300 multigrid builds its own (algebraic) hierarchy")
        if not isinstance(A, CSRTensor):
            raise TypeError("A must be a CSRTensor")
        dev = A.values.device
        if dev.type != "cuda":
            raise ValueError("GAMGSolver runs on the GPU only")
        self.A = A
        s = stream_ptr(dev)
        st = status_word(dev)
        lev = _Level(A.crow.contiguous(), A.col.to(torch.int32).contiguous(),
                     A.values.to(torch.float64).contiguous())
        self.levels = []
        while True:
            n = lev.n
            if self.block_size > 1 and n % self.block_size == 0:
                lev.agg, nc, lev.dinv, lev.lmax = self._block_aggregate(lev, dev, st, s)
            else:
                lev.agg, nc, lev.dinv, lev.lmax = self._aggregate(lev, dev, st, s)
            self.levels.append(lev)
            # a level that shrinks by less than half adds sweeps and no
            # convergence: the current one is then the coarsest
            last = (n <= self.csize or len(self.levels) >= self.max_levels or nc == 0 or nc > 0.5 * n)
            if last:
                lev.agg = None
                break
            lev.n_coarse = nc
            lev.member_ptr, lev.members, cptr, ccol, cval = self._coarse(lev.indptr, lev.indices, lev.values,
                                                                         lev.agg, nc, dev, st, s)
            lev = _Level(cptr, ccol, cval)
        for k, L in enumerate(self.levels):
            L.values32 = L.values.to(torch.float32) if self.vcycle_f32 else None
            L.dinv32 = L.dinv.to(torch.float32) if self.vcycle_f32 else None
            if L.n >= self.sell_min_rows:
                # values of the V-cycle's type; the finest copy also carries
                # the FP64 values for PCG's operator
                L.sell = _level_sell(L, with32=self.vcycle_f32, with64=(k == 0 or not self.vcycle_f32))
        self._desc = (_lib.AmgLevel * len(self.levels))()
        for k, L in enumerate(self.levels):
            d = self._desc[k]
            d.n, d.nnz = L.n, L.nnz
            d.indptr, d.indices, d.values, d.dinv = (L.indptr.data_ptr(), L.indices.data_ptr(), L.values.data_ptr(),
                                                    L.dinv.data_ptr())
            d.lmax = L.lmax
            d.values32 = L.values32.data_ptr() if L.values32 is not None else None
            d.dinv32 = L.dinv32.data_ptr() if L.dinv32 is not None else None
            d.sell = ctypes.addressof(L.sell.desc) if L.sell is not None else None
            if L.agg is not None:
                d.agg, d.n_coarse = L.agg.data_ptr(), L.n_coarse
                d.member_ptr, d.members = L.member_ptr.data_ptr(), L.members.data_ptr()
        return self

    def _ws(self):
        dev = self.levels[0].values.device
        nb = _lib.lib().fgb_amg_workspace_bytes(self._desc, len(self.levels))
        if nb == 0:
            raise RuntimeError("multigrid hierarchy is inconsistent")
        return workspace(nb, dev)

    def info(self):
        """Rows, nonzeros and Chebyshev bound of every level."""
        return [{"n": L.n, "nnz": L.nnz, "lmax": L.lmax} for L in self.levels]

    # ------------------------------------------------------------ apply
    def vcycle(self, r: torch.Tensor) -> torch.Tensor:
        """One V-cycle applied to r (x = 0 start)."""
        if self._desc is None:
            raise RuntimeError("call setup(A) first")
        dev = self.levels[0].values.device
        r = r.to(device=dev, dtype=torch.float64).contiguous()
        x = torch.empty_like(r)
        ws = self._ws()
        call("fgb_amg_vcycle", self._desc, len(self.levels), self.sstep, self.cdeg, self.omega, ptr(r), ptr(x),
             ptr(ws), ws.numel(), stream_ptr(dev))
        _lib.add_launches(6 * len(self.levels) * self.sstep)
        return x

    __matmul__ = vcycle

    def pcg(self, b: torch.Tensor, x0: Optional[torch.Tensor] = None, atol: float = 1e-12, rtol: float = 1e-8,
            maxit: int = 10000, norm: int = 0):
        """CG preconditioned by the V-cycle (FEALPy's recurrence; norm 0 stops
        on sqrt(r.z), 1 on ||r||); returns (x, info)."""
        dev = self.levels[0].values.device
        b = b.to(device=dev, dtype=torch.float64).contiguous()
        x = torch.zeros_like(b) if x0 is None else x0.to(device=dev, dtype=torch.float64).clone()
        ws = self._ws()
        info = _lib.PcgInfo()
        call("fgb_pcg_amg", self._desc, len(self.levels), self.sstep, self.cdeg, self.omega, ptr(b), ptr(x),
             float(atol), float(rtol), int(maxit), int(norm), ctypes.byref(info), ptr(ws), ws.numel(), stream_ptr(dev))
        _lib.add_launches(info.launches)
        return x, info

    def solve(self, b: torch.Tensor):
        """Solve A x = b: PCG with the V-cycle ('CG') or V-cycle iterations
        x += V(b - A x) ('MG'); returns (x, info) with FEALPy's keys."""
        if self.isolver == "CG":
            x, info = self.pcg(b, atol=self.atol, rtol=self.rtol, maxit=self.maxit, norm=1)
            return x, {"residual": info.residual, "niter": int(info.niter)}
        A = self.A
        dev = self.levels[0].values.device
        b = b.to(device=dev, dtype=torch.float64)
        x = torch.zeros_like(b)
        vals = A.values.to(torch.float64)
        res, bn = K.residual_norm(A.crow, A.col, vals, b, x)
        it = 0
        while it < self.maxit:
            if res < self.atol or res < self.rtol * bn:
                break
            r = b - K.csr_spmv(A.crow, A.col, A.values, x)
            x += self.vcycle(r)
            it += 1
            res, _ = K.residual_norm(A.crow, A.col, vals, b, x)
        return x, {"residual": res, "niter": it}


class AMGPreconditioner:
    """``AMGPreconditioner(**kw).apply(A)`` builds the hierarchy and returns
    it for ``cg(A, b, M=...)`` (the shape of ``JacobiPreconditioner``)."""

    def __init__(self, **kw):
        self.kw = kw

    def apply(self, A: CSRTensor) -> GAMGSolver:
        return GAMGSolver(**self.kw).setup(A)


def multigrid_solve(A, b, rtol: float = 1e-10, maxit: int = 100000, fp64: bool = False, block_size: int = 0):
    """One system by multigrid PCG on the current stream (the multigrid lane
    of the serving loop and of the batched solve): the AMG hierarchy (FP32
    V-cycle, FP64 with ``fp64``), PCG on the iterated residual, restarted
    from the iterate on the true residual b - A x while that is above
    ``rtol`` and still halves (the iterated residual drifts below the true
    one on ill-conditioned systems).  ``block_size`` 0: node blocks of 3
    when the matrix is marked as three interleaved components, else none.
    Returns (x with the smallest true residual, iterations, stop reason, its
    true relative residual)."""
    from .solver import cg
    if block_size == 0:
        block_size = 3 if getattr(A, "node_block", 1) == 3 else 1
    M = GAMGSolver(vcycle_f32=not fp64, block_size=block_size).setup(A)
    vals = A.values.to(torch.float64)
    x, niter, reason = None, 0, 0
    best_x, best_r = None, float("inf")
    for _ in range(4):
        x, inf = cg(A, b, x0=x, M=M, atol=0.0, rtol=rtol, maxit=maxit, returninfo=True, stop="residual")
        niter += int(inf["niter"])
        reason = int(inf["reason"])
        res, bnorm = K.residual_norm(A.crow, A.col, vals, b, x)
        r_new = res / bnorm if bnorm > 0 else 0.0
        improved = r_new < 0.5 * best_r
        if r_new < best_r:
            best_x, best_r = x, r_new
        if r_new <= rtol or not improved:
            break
    return best_x, niter, reason, best_r
