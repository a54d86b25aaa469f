"""The persistent FP32-refined solver's grid-barrier time limit, made to run
out on purpose: with a wait limit of one poll the blocks that arrive early at
a barrier give up, raise the shared error flag and return, every other block
sees the flag and returns too, and the call reports a CUDA-error status
(RuntimeError) instead of hanging.  The context stays usable: the next solve
in the same process, with the default limit, converges and matches the
host-polled loop."""
import os

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def test_grid_barrier_limit_runs_out_and_the_next_solve_succeeds(golden_dir):
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA device")
    dev = torch.device("cuda", 0)
    import fealpy_gb300 as F
    from fealpy_gb300 import kernels as K
    from fealpy_gb300.solver import _sell_of
    z = np.load(os.path.join(golden_dir, "c1_poisson_tri_p1_64.npz"))
    A = F.CSRTensor(torch.as_tensor(z["bc_crow"], device=dev), torch.as_tensor(z["bc_col"], device=dev),
                    torch.as_tensor(z["bc_val"], device=dev), (len(z["bc_crow"]) - 1,) * 2)
    b = torch.as_tensor(z["bc_F"], device=dev)
    S = _sell_of(A, want32=True)
    dinv = A.diagonal_inverse().to(torch.float64).contiguous()

    x = torch.zeros_like(b)
    with pytest.raises(RuntimeError, match="CUDA error"):
        K.pcg_sell_mixed(S, dinv, b, x, 1e-10, graph=2, barrier_polls=1)
    torch.cuda.synchronize()

    # same process, default limit: the persistent kernel runs to convergence
    x = torch.zeros_like(b)
    info = K.pcg_sell_mixed(S, dinv, b, x, 1e-10, graph=2)
    assert info.graph == 2 and info.reason == 2 and info.true_relres <= 1e-10, (info.graph, info.reason)
    xp = torch.zeros_like(b)
    infop = K.pcg_sell_mixed(S, dinv, b, xp, 1e-10, graph=0)
    assert infop.reason == 2 and abs(int(info.niter) - int(infop.niter)) <= 2
    err = float((x - xp).abs().max() / xp.abs().max())
    assert err < 1e-9, err
    uh = torch.as_tensor(z["uh"], device=dev)
    assert float((x - uh).abs().max() / uh.abs().max()) < 1e-8
