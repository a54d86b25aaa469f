"""fgb_pcg_f64_noalloc (FP64 Jacobi-PCG with the scratch in a static device
array of the library) against fgb_pcg_f64 with a caller workspace, called
through the C ABI on the C1 system (P1 Poisson on a 64x64 triangle box after
Dirichlet elimination, 4,225 rows).  Two no-allocation calls in a row must
both match the workspace solve, and the second must leave the device's free
memory unchanged; a size above the fixed limit is refused before any device
work.  This file is named to be collected last so that it
also runs after every other GPU test in the same process."""
import ctypes
import os

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

MAX_ROWS = 65536  # FGB_PCG_NOALLOC_MAX_ROWS in include/fealpy_gb300.h
TOL = 1e-12       # relative difference allowed between the two entry points


def _system(golden_dir):
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA device")
    z = np.load(os.path.join(golden_dir, "c1_poisson_tri_p1_64.npz"))
    dev = torch.device("cuda", 0)
    crow = torch.as_tensor(z["bc_crow"], dtype=torch.int64, device=dev)
    col = torch.as_tensor(z["bc_col"], dtype=torch.int32, device=dev)
    val = torch.as_tensor(z["bc_val"], dtype=torch.float64, device=dev)
    b = torch.as_tensor(z["bc_F"], dtype=torch.float64, device=dev)
    n = crow.numel() - 1
    d = torch.zeros(n, dtype=torch.float64, device=dev)
    rows = torch.repeat_interleave(torch.arange(n, device=dev), crow[1:] - crow[:-1])
    diag = rows == col.to(torch.int64)
    d.index_put_((rows[diag],), val[diag], accumulate=True)
    return n, crow, col, val, (1.0 / d).contiguous(), b, z


def _p(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


def test_noalloc_matches_workspace_entry_point(golden_dir):
    from fealpy_gb300 import _lib
    lib = _lib.lib()
    n, crow, col, val, dinv, b, z = _system(golden_dir)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    args = (float(0.0), float(1e-10), 10000, 16, 0, 0)  # atol, rtol, maxit, check_every, lanes, norm

    x_ws = torch.zeros(n, dtype=torch.float64, device=b.device)
    ws = torch.empty(int(lib.fgb_pcg_workspace_bytes(n)), dtype=torch.uint8, device=b.device)
    info_ws = _lib.PcgInfo()
    rc = lib.fgb_pcg_f64(n, _p(crow), _p(col), _p(val), _p(dinv), _p(b), _p(x_ws), *args[:2], args[2], args[3],
                         args[4], args[5], 0, _p(ws), ws.numel(), ctypes.byref(info_ws), stream)
    assert rc == 0 and info_ws.reason == 2

    for call in range(2):
        x = torch.zeros(n, dtype=torch.float64, device=b.device)
        info = _lib.PcgInfo()
        torch.cuda.synchronize()
        free_before = torch.cuda.mem_get_info(b.device)[0]
        rc = lib.fgb_pcg_f64_noalloc(n, _p(crow), _p(col), _p(val), _p(dinv), _p(b), _p(x), *args[:2], args[2],
                                     args[3], args[4], args[5], ctypes.byref(info), stream)
        torch.cuda.synchronize()
        free_after = torch.cuda.mem_get_info(b.device)[0]
        assert rc == 0, (call, lib.fgb_status_string(rc))
        if call == 1:
            # the defining property: a call allocates no device memory (the
            # first call is exempt: it may load the library's device code)
            assert free_after == free_before, (free_before, free_after)
        assert info.reason == info_ws.reason and abs(info.niter - info_ws.niter) <= 1, (call, info.niter)
        err = float((x - x_ws).abs().max() / x_ws.abs().max())
        assert err <= TOL, (call, err)
        # and the solve is the reference's: same solution as the oracle fixture
        uh = torch.as_tensor(z["uh"], device=b.device)
        assert float((x - uh).abs().max() / uh.abs().max()) < 1e-9


def test_noalloc_refuses_sizes_above_the_limit(golden_dir):
    from fealpy_gb300 import _lib
    lib = _lib.lib()
    n, crow, col, val, dinv, b, _ = _system(golden_dir)
    x = torch.zeros(n, dtype=torch.float64, device=b.device)
    info = _lib.PcgInfo()
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    rc = lib.fgb_pcg_f64_noalloc(MAX_ROWS + 1, _p(crow), _p(col), _p(val), _p(dinv), _p(b), _p(x), 0.0, 1e-10,
                                 100, 16, 0, 0, ctypes.byref(info), stream)
    assert rc == 8 and b"limit" in lib.fgb_status_string(rc)
    assert torch.count_nonzero(x) == 0
