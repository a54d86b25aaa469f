"""Jacobi-preconditioned CG with FEALPy's interface (``fealpy/solver/cg.py:14-123``)
and its FP32-refined variant.

``cg`` keeps the reference iteration exactly (same recurrences, same stopping
rule on ``sqrt(r.z)``, ``info = {'residual', 'niter'}``) but runs it as two
fused GPU kernels per iteration with all scalars on the device.
``cg_mixed`` runs the iterations in FP32 and restores FP64 accuracy with
reliable updates (FP64 residual recomputation) until the true relative
residual ``||b - A x|| / ||b||`` reaches ``rtol``.
"""
import logging
from typing import Optional

import torch

from .sparse import CSRTensor, COOTensor
from . import kernels as K

__all__ = ["cg", "cg_mixed", "JacobiPreconditioner"]

logger = logging.getLogger("fealpy_gb300")


class JacobiPreconditioner:
    """``M = diag(A)^-1`` as a diagonal CSRTensor
    (``fealpy/solver/iterative_solver_manger.py:273-280``)."""

    def apply(self, A: CSRTensor) -> CSRTensor:
        d = A.diags()
        M = CSRTensor(d.crow, d.col, 1.0 / d.values, A.shape)
        return M


def _diag_inv_of(M):
    if M is None:
        return None
    if isinstance(M, CSRTensor) and M.is_diagonal():
        return M.values.contiguous()
    raise NotImplementedError("cg on the GB300 path takes M=None, a diagonal CSRTensor (Jacobi) or a GAMGSolver "
                              "hierarchy")


def _info_dict(info, extra=None):
    out = {"residual": info.residual, "niter": int(info.niter), "reason": int(info.reason),
           "launches": int(info.launches), "kernel_ms": float(info.kernel_ms),
           "kernel_launches": int(info.kernel_launches), "other_ms": float(info.other_ms),
           "extra_ms": float(info.extra_ms), "graph": bool(info.graph), "persistent": int(info.graph) == 2}
    if extra:
        out.update(extra)
    return out


# Launch shape of the SELL slice kernels per (rows, padded entries, value
# type), found once by timing the candidates (kernels.sell_autotune) and
# reused for every later matrix of the same size.
_LAUNCH_CACHE = {}
# column format of the solvers' SELL copies: False = 4-byte columns (default:
# measured faster on the P2 64^3 system, where the renumbering the 2-byte
# steps need costs more gather locality than the 25% fewer matrix bytes
# save), None = delta-coded columns of the renumbered matrix where the bridges
# add at most 25% entries, True = delta-coded always
SELL_D16: Optional[bool] = False
# FP32 copies (cg_mixed) with 15-bit column steps in the matrix's own
# numbering: 6 bytes per FP32 nonzero instead of 8, the gather locality of
# FEALPy's numbering unchanged.  The FP64 solver's copy keeps 4-byte columns
# (its SpMV is limited by the FP64 multiply-add rate, not by the bytes).
SELL_D15 = True
# cg_mixed with graph=True runs systems of at most this many rows and at most
# this many nonzeros per row on average as one persistent cooperative kernel
# (no launches per iteration); the others as the CUDA-graph loop of separate
# kernels, whose gathers keep their L1 hits.  Measured per solve (graph loop /
# persistent): P1 triangles 4.2 K rows 4.6 / 4.0 ms, 66 K rows 18.2 / 15.7 ms,
# 263 K rows 50.4 / 37.3 ms; P2 tetrahedra 118 K rows 6.1 / 6.5 ms, 531 K rows
# 16.0 / 16.4 ms.
PERSISTENT_MAX_ROWS = 1 << 19
# node-triple copies (one column per three values) for matrices of vector
# spaces with three interleaved components
SELL_TRIPLES = True
PERSISTENT_MAX_ROW_NNZ = 10


def _triples(A: CSRTensor) -> bool:
    return SELL_TRIPLES and getattr(A, "node_block", 1) == 3 and A.shape[0] % 3 == 0


def _sell_of(A: CSRTensor, want32: bool, tune: bool = True):
    """SELL-32 copy of A for the solvers (cached on the matrix), with its
    launch shape from the autotuner cache."""
    S = getattr(A, "_sell", None)
    if S is None or (want32 and S.val32 is None) or (not want32 and S.val64 is None):
        d15 = SELL_D15 and want32
        if A.values.dtype == torch.float32 and want32:
            # FP32-assembled operator: the FP32 values are the matrix (no FP64 copy)
            S = K.sell_build(A.crow, A.col, None, A.values.contiguous(), want64=False, want32=True, d16=SELL_D16,
                             blocks=getattr(A, "dof_blocks", None), triples=_triples(A), d15=d15)
        else:
            v32 = A._f32 if (want32 and A._f32 is not None) else None
            S = K.sell_build(A.crow, A.col, A.values.to(torch.float64).contiguous(), v32, want64=True, want32=want32,
                             d16=SELL_D16, blocks=getattr(A, "dof_blocks", None), triples=_triples(A), d15=d15)
        A._sell = S
        if tune:
            dt = torch.float32 if want32 else torch.float64
            key = (S.n, S.padded_nnz, dt, S.cols)
            shape = _LAUNCH_CACHE.get(key)
            if shape is None:
                times = K.sell_autotune(S, dt)
                shape = min(times, key=times.get)
                _LAUNCH_CACHE[key] = shape
                logger.info(f"SELL launch shape for n={S.n}: {shape} ({times[shape]:.1f} us per SpMV)")
            S.set_launch(*shape)
    return S


def _cg_operator(A, b, x0, M, atol, rtol, maxit, batch_first):
    """FEALPy's recurrence and stopping rule (``fealpy/solver/cg.py:76-123``)
    for an operator that is not a stored matrix: anything with ``@`` (``cg``
    takes ``SupportsMatmul``, ``fealpy/solver/cg.py:10-17``), such as a
    BilinearForm before assembly, whose product is the matrix-free kernel
    pair.  The products are the operator's own; the vector updates and dot
    products run on the device, and the stopping test reads one scalar per
    iteration.  ``M`` is None, a diagonal CSRTensor (Jacobi: an element-wise
    product) or any operator with ``@``."""
    if b.ndim != 1:
        raise NotImplementedError("an operator without a stored matrix takes one right-hand side")
    info = {"residual": 0.0, "niter": 0}
    b = b.to(torch.float64)
    b_norm = float(torch.linalg.norm(b))
    if b_norm < 1e-15:
        return torch.zeros_like(b), info
    if M is None:
        prec = lambda v: v
    elif isinstance(M, CSRTensor) and M.is_diagonal():
        dinv = M.values.to(torch.float64)
        prec = lambda v: dinv * v
    elif hasattr(M, "__matmul__"):
        prec = lambda v: M @ v
    else:
        raise TypeError(f"M must support matrix products, got {type(M).__name__}")
    x = torch.zeros_like(b) if x0 is None else x0.to(torch.float64).clone()
    r = b - A @ x
    z = prec(r)
    p = z
    rz = torch.dot(r, z)
    n_iter = 0
    while True:
        Ap = A @ p
        alpha = rz / torch.dot(p, Ap)
        x = x + alpha * p
        r = r - alpha * Ap
        z = prec(r)
        rz_new = torch.dot(r, z)
        res = float(torch.sqrt(rz_new))
        n_iter += 1
        info["residual"] = res
        info["niter"] = n_iter
        if res < atol or res < rtol * b_norm:
            break
        if maxit is not None and n_iter >= maxit:
            logger.info(f"CG: failed, stopped by maxit ({maxit}).")
            break
        p = z + (rz_new / rz) * p
        rz = rz_new
    return x, info


def cg(A, b: torch.Tensor, x0: Optional[torch.Tensor] = None, M=None, *, batch_first: bool = False,
       atol: float = 1e-12, rtol: float = 1e-8, maxit: Optional[int] = 10000, returninfo: bool = False,
       check_every: int = 16, lanes_per_row: int = 0, stop: str = "preconditioned", profile: bool = False,
       solver_format: str = "sell", graph: bool = True):
    """Solve ``A x = b`` by (preconditioned) CG; see module docstring.

    ``stop='preconditioned'`` (default) is FEALPy's test on ``sqrt(r.z)``;
    ``stop='residual'`` tests the 2-norm of the iterated residual instead.
    ``solver_format='sell'`` (default) iterates on a SELL-32 copy of ``A``
    ('csr' iterates on the CSR arrays); ``graph`` runs the iterations as a
    device-side CUDA-graph loop.  ``profile`` records CUDA-event times of the
    SpMV kernel into the info (host-polled loop)."""
    if not isinstance(b, torch.Tensor):
        raise AssertionError("b must be a Tensor")
    if b.ndim not in (1, 2):
        raise ValueError("b must be a 1D or 2D dense tensor")
    if x0 is not None and x0.shape != b.shape:
        raise ValueError("x0 and b must have the same shape")
    if isinstance(A, COOTensor):
        A = A.tocsr()
    if not isinstance(A, CSRTensor):
        if not hasattr(A, "__matmul__"):
            raise TypeError(f"A must support matrix products, got {type(A).__name__}")
        x, info = _cg_operator(A, b, x0, M, atol, rtol, maxit, batch_first)
        return (x, info) if returninfo else x
    A._single("cg")
    if stop not in ("preconditioned", "residual"):
        raise ValueError("stop must be 'preconditioned' or 'residual'")
    from .amg import GAMGSolver
    if b.ndim == 2:
        # (n, batch) right-hand sides (or (batch, n) with batch_first):
        # FEALPy's joint recurrence, fealpy/solver/cg.py:60-123
        if isinstance(M, GAMGSolver):
            raise NotImplementedError("several right-hand sides take M=None or a Jacobi preconditioner")
        if stop != "preconditioned":
            raise ValueError("several right-hand sides stop on sqrt(sum r.z) as FEALPy does")
        dinv = _diag_inv_of(M)
        B = (b.transpose(0, 1) if batch_first else b).to(torch.float64).contiguous()
        X = torch.zeros_like(B) if x0 is None else (x0.transpose(0, 1) if batch_first else x0).to(
            torch.float64).contiguous().clone()
        info = K.pcg_multi(A.crow, A.col, A.values, dinv, B, X, atol, rtol,
                           maxit if maxit is not None else 2 ** 62)
        x = X.transpose(0, 1) if batch_first else X
        out = _info_dict(info)
        return (x, out) if returninfo else x
    if isinstance(M, GAMGSolver):
        # multigrid preconditioner: the whole PCG loop in the library
        x, info = M.pcg(b, x0=x0, atol=atol, rtol=rtol, maxit=maxit if maxit is not None else 2 ** 62,
                        norm=0 if stop == "preconditioned" else 1)
        out = {"residual": info.residual, "niter": int(info.niter), "reason": int(info.reason),
               "launches": int(info.launches), "graph": False, "persistent": False, "amg_levels": len(M.levels)}
        return (x, out) if returninfo else x
    dinv = _diag_inv_of(M)
    b = b.to(dtype=torch.float64).contiguous()
    x = torch.zeros_like(b) if x0 is None else x0.to(torch.float64).clone()
    maxit = maxit if maxit is not None else 2 ** 62
    norm = 0 if stop == "preconditioned" else 1
    if solver_format == "sell":
        S = _sell_of(A, want32=False)
        info = K.pcg_sell_f64(S, dinv, b, x, atol, rtol, maxit, check_every, norm, graph and not profile, profile)
    elif solver_format == "csr":
        info = K.pcg_f64(A.crow, A.col, A.values.to(torch.float64), dinv, b, x, atol, rtol, maxit, check_every,
                         lanes_per_row, norm, profile)
    else:
        raise ValueError("solver_format must be 'sell' or 'csr'")
    out = _info_dict(info)
    if info.reason == 3:
        logger.info(f"CG: failed, stopped by maxit ({maxit}).")
    if returninfo:
        return x, out
    return x


def cg_mixed(A: CSRTensor, b: torch.Tensor, x0: Optional[torch.Tensor] = None, M=None, *, rtol: float = 1e-10,
             delta: float = 0.2, maxit: int = 100000, returninfo: bool = False, check_every: int = 32,
             lanes_per_row: int = 0, profile: bool = False, solver_format: str = "sell", graph: bool = True):
    """FP32 Jacobi-PCG iterations with FP64 reliable updates; stops on the true
    relative residual computed in FP64 arithmetic.  ``M`` must be None (Jacobi
    from ``A`` is used) or the diagonal CSR of ``JacobiPreconditioner``.

    An FP64 ``A`` keeps its FP64 values for the residual recomputation (the
    FP32 copy only drives the iterations).  An FP32 ``A`` (assembled with
    ``dtype=torch.float32``) is the operator itself: the residual is formed
    from its FP32 values in FP64 arithmetic, so the solve reaches ``rtol`` for
    that operator, and the difference to the FP64-assembled solution is the
    assembly's FP32 rounding."""
    if not isinstance(A, CSRTensor):
        raise NotImplementedError("cg_mixed takes a CSRTensor matrix")
    A._single("cg_mixed")
    dinv = _diag_inv_of(M)
    if dinv is None:
        dinv = A.diagonal_inverse()
    dinv = dinv.to(torch.float64).contiguous()
    b = b.to(dtype=torch.float64).contiguous()
    x = torch.zeros_like(b) if x0 is None else x0.to(torch.float64).clone()
    if solver_format == "sell":
        S = _sell_of(A, want32=True)
        small = A.shape[0] <= PERSISTENT_MAX_ROWS and A.nnz <= PERSISTENT_MAX_ROW_NNZ * A.shape[0]
        mode = 0 if (profile or not graph) else (2 if small else 1)
        info = K.pcg_sell_mixed(S, dinv, b, x, rtol, delta, maxit, check_every, mode, profile)
    elif solver_format == "csr":
        if A.values.dtype != torch.float64:
            raise NotImplementedError("solver_format='csr' cg_mixed needs an FP64 matrix")
        info = K.pcg_mixed(A.crow, A.col, A.values, A.values_f32(), dinv, b, x, rtol, delta, maxit, check_every,
                           lanes_per_row, profile)
    else:
        raise ValueError("solver_format must be 'sell' or 'csr'")
    out = _info_dict(info, {"relres": info.true_relres, "n_updates": int(info.n_updates), "fp64_iterations": 0})
    if info.reason == 7:
        # the FP32 iterations stopped improving the true residual (a condition
        # number beyond FP32): continue with FP64 PCG from the current iterate
        logger.info(f"cg_mixed: FP32 iterations stagnated at relres {info.true_relres:.2e}; continuing in FP64")
        dinv64 = dinv if dinv is not None else A.diagonal_inverse().to(torch.float64)
        M64 = CSRTensor(torch.arange(A.shape[0] + 1, device=x.device), torch.arange(A.shape[0], device=x.device,
                        dtype=torch.int32), dinv64, A.shape)
        vals64 = A.values.to(torch.float64)
        left, its, rel, reason = max(maxit - int(info.niter), 1), 0, float(info.true_relres), 3
        # FP64 PCG restarted from the current iterate until the true residual
        # (formed in FP64) meets rtol; each restart re-forms r = b - A x, so the
        # drift of the iterated residual cannot end the solve early
        for _ in range(8):
            x, i64 = cg(A, b, x0=x, M=M64, atol=0.0, rtol=rtol, maxit=left, returninfo=True, stop="residual",
                        graph=graph)
            its += i64["niter"]
            left -= i64["niter"]
            res, bn = K.residual_norm(A.crow, A.col, vals64, b, x)
            new = res / bn if bn > 0 else 0.0
            if new <= rtol:
                rel, reason = new, 2
                break
            if left <= 0 or new > 0.9 * rel:
                rel, reason = new, (3 if left <= 0 else 7)
                break
            rel = new
        out.update({"niter": out["niter"] + its, "reason": reason, "relres": rel, "fp64_iterations": its,
                    "graph": out["graph"] and i64["graph"]})
    if returninfo:
        return x, out
    return x
