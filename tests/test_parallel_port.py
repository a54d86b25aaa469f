"""The parallel form of the oracle pipeline (oracle/parallel_port.py, timed by
the bench's reference arm) against the sequential oracle: the row ranges
concatenate to the same pre- and post-Dirichlet CSR bit for bit, the same
right-hand sides, and the block-threaded Jacobi-PCG gives the same iterates."""
import multiprocessing

import numpy as np

from oracle import fem_oracle as O
from oracle import parallel_port as PP


def test_parallel_port_equals_sequential_oracle():
    from fealpy_gb300.workloads import diffusion_mass_tet_box
    n = 6
    node, cell, kappa = diffusion_mass_tet_box(n)
    ref = O.poisson_pipeline(node, cell, 2, kappa=kappa, rho=1.0, q=4, rtol=1e-10)
    N = ref["n"]
    ctx = multiprocessing.get_context("spawn")
    with ctx.Pool(2) as pool:
        out = PP.assemble(pool, "c2", n, N, 5, keep_pre=True)
    pre = out["pre"]
    # concatenate the per-range row pointers
    offs = np.cumsum([0] + [o["crow"][-1] for o in pre])
    crow = np.concatenate([[0]] + [o["crow"][1:] + offs[k] for k, o in enumerate(pre)])
    assert np.array_equal(crow, ref["crow"])
    assert np.array_equal(np.concatenate([o["col"] for o in pre]), ref["col"])
    assert np.array_equal(np.concatenate([o["val"] for o in pre]), ref["val"])
    assert np.array_equal(np.concatenate([o["F"] for o in pre]), ref["F"])
    boffs = np.cumsum([0] + [o["bc_crow"][-1] for o in pre])
    bcrow = np.concatenate([[0]] + [o["bc_crow"][1:] + boffs[k] for k, o in enumerate(pre)])
    assert np.array_equal(bcrow, ref["bc_crow"])
    assert np.array_equal(np.concatenate([o["bc_col"] for o in pre]), ref["bc_col"])
    assert np.array_equal(np.concatenate([o["bc_val"] for o in pre]), ref["bc_val"])
    assert np.array_equal(out["b"], ref["bc_F"])
    A = PP.BlockOperator(out["blocks"], out["bounds"], 3)
    try:
        x, info = PP.jacobi_cg(A, out["b"], atol=1e-30, rtol=1e-10)
    finally:
        A.close()
    assert info["niter"] == ref["info"]["niter"]
    assert np.array_equal(x, ref["x"])
