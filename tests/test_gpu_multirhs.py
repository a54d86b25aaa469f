"""Several right-hand sides in one cg call (the (n, batch) path of
``fealpy/solver/cg.py:60-123``): per-column recurrences, one joint stopping
test on sqrt(sum_c r_c . z_c).  Against the reference's own solutions and
iteration counts (``cg_multi_rhs.npz``, made by ``make_golden.py --coef``) on
a P2 tetrahedral diffusion + mass matrix with three random columns, with the
Jacobi preconditioner and without one.  Tolerances: iterations within 1,
solutions within 1e-9 relative."""
import os

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def cuda():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch.device("cuda:0")


def rel(a, b):
    a = a.detach().cpu().numpy() if isinstance(a, torch.Tensor) else np.asarray(a)
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


def test_multi_rhs_against_reference(golden_dir):
    dev = cuda()
    import fealpy_gb300 as F
    z = np.load(os.path.join(golden_dir, "cg_multi_rhs.npz"))
    n = len(z["crow"]) - 1
    A = F.CSRTensor(torch.as_tensor(z["crow"], device=dev), torch.as_tensor(z["col"], device=dev),
                    torch.as_tensor(z["val"], device=dev), (n, n))
    B = torch.as_tensor(z["B"], device=dev)
    M = F.JacobiPreconditioner().apply(A)
    x, info = F.cg(A, B, M=M, atol=1e-30, rtol=1e-10, returninfo=True)
    assert x.shape == B.shape
    assert abs(info["niter"] - int(z["niter_jacobi"])) <= 1, (info["niter"], int(z["niter_jacobi"]))
    assert rel(x, z["x_jacobi"]) < 1e-9
    assert info["residual"] < 1e-10 * float(np.linalg.norm(z["B"]))
    xp, ip = F.cg(A, B, atol=1e-30, rtol=1e-10, returninfo=True)
    assert abs(ip["niter"] - int(z["niter_plain"])) <= 1, (ip["niter"], int(z["niter_plain"]))
    assert rel(xp, z["x_plain"]) < 1e-9
    # batch_first: the same solve on the transposed layout
    xb = F.cg(A, B.transpose(0, 1).contiguous(), M=M, atol=1e-30, rtol=1e-10, batch_first=True)
    assert torch.equal(xb.transpose(0, 1), x)
    # every column of the joint solve is a solution of its own system
    for c in range(B.shape[1]):
        r = B[:, c] - A @ x[:, c]
        assert float(torch.linalg.norm(r)) < 1e-8 * float(torch.linalg.norm(B))


def test_multi_rhs_zero_and_initial_guess(golden_dir):
    dev = cuda()
    import fealpy_gb300 as F
    z = np.load(os.path.join(golden_dir, "cg_multi_rhs.npz"))
    n = len(z["crow"]) - 1
    A = F.CSRTensor(torch.as_tensor(z["crow"], device=dev), torch.as_tensor(z["col"], device=dev),
                    torch.as_tensor(z["val"], device=dev), (n, n))
    zero = torch.zeros((n, 2), dtype=torch.float64, device=dev)
    x0, i0 = F.cg(A, zero, returninfo=True)
    assert torch.count_nonzero(x0) == 0 and i0["niter"] == 0
    # starting from the reference solution: converged at the first test
    B = torch.as_tensor(z["B"], device=dev)
    xs = torch.as_tensor(z["x_jacobi"], device=dev)
    x1, i1 = F.cg(A, B, x0=xs, M=F.JacobiPreconditioner().apply(A), atol=1e-30, rtol=1e-8, returninfo=True)
    assert i1["niter"] <= 2 and rel(x1, z["x_jacobi"]) < 1e-9
