"""SELL storage formats.  Delta-coded copy (sell_build(d16=True)): the
locality renumbering is a permutation and deterministic, the renumbered copy
multiplies like the CSR matrix (FP64 within 1e-14 of scipy; FP32 within
1e-5), steps above 65535 are bridged, rows above the shared-memory stage and
key groups above 64 rows take their fallbacks, and the solvers on the
renumbered copy give the solution in the caller's numbering.  Node-triple
copy (sell_build(triples=True), vector spaces with three interleaved
components): SpMV against scipy, and the solvers against the copy with a
column per entry.  15-bit copy (sell_build(d15=True), the matrix's own
numbering): SpMV against scipy on FEALPy matrices and on gaps that need long
steps, empty rows, an FP32-only copy, refusal of unsorted rows, and the
FP32-refined solver against the 4-byte copy."""
import os

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def cuda():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch.device("cuda:0")


def rel_err(a, b):
    a = a.detach().cpu().numpy() if isinstance(a, torch.Tensor) else np.asarray(a)
    b = np.asarray(b)
    return np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)


def _spd(n, extra_cols, seed=0):
    """Symmetric diagonally dominant CSR: a 1-D Laplacian plus symmetric
    couplings (i, j) for the given extra column offsets (wrapped)."""
    import scipy.sparse as sp
    rng = np.random.default_rng(seed)
    rows, cols = [np.arange(n - 1)], [np.arange(1, n)]
    for off in extra_cols:
        i = np.arange(n)
        j = (i + off) % n
        keep = i < j
        rows.append(i[keep])
        cols.append(j[keep])
    r = np.concatenate(rows)
    c = np.concatenate(cols)
    v = -rng.uniform(0.1, 1.0, size=r.size)
    A = sp.coo_matrix((np.concatenate([v, v]), (np.concatenate([r, c]), np.concatenate([c, r]))), shape=(n, n)).tocsr()
    A.sum_duplicates()
    d = np.asarray(-A.sum(axis=1)).ravel() + 1.0
    A = (A + sp.diags(d)).tocsr()
    A.sort_indices()
    return A


def _build(A, dev, d16, want32=True, blocks=None):
    from fealpy_gb300 import kernels as K
    t = lambda a: torch.as_tensor(a, device=dev)
    return K.sell_build(t(A.indptr.astype(np.int64)), t(A.indices.astype(np.int32)), t(A.data), None, want64=True,
                        want32=want32, d16=d16, blocks=blocks)


def _merge_order(sizes):
    """Stable merge of dof blocks by key floor(j * n0 / nb): sort of all rows
    by (key, block, j), the order the block renumbering computes in closed
    form."""
    keys = []
    start = 0
    for b, nb in enumerate(sizes):
        for j in range(nb):
            keys.append(((j * sizes[0]) // nb, b, j, start + j))
        start += nb
    return np.array([k[3] for k in sorted(keys)])


def _check_spmv(S, A, dev):
    from fealpy_gb300 import kernels as K
    x = np.random.default_rng(5).normal(size=A.shape[0])
    ref = A @ x
    assert rel_err(K.sell_spmv(S, torch.as_tensor(x, device=dev), torch.float64), ref) < 1e-14
    assert rel_err(K.sell_spmv(S, torch.as_tensor(x, device=dev, dtype=torch.float32), torch.float32), ref) < 1e-5


def test_d16_golden_matrices_match_csr(golden_dir):
    dev = cuda()
    import scipy.sparse as sp
    for name in ("small_tet_p2.npz", "small_tri_p3.npz", "c1_poisson_tri_p1_64.npz"):
        z = np.load(os.path.join(golden_dir, name))
        n = len(z["crow"]) - 1
        A = sp.csr_matrix((z["val"], z["col"], z["crow"]), shape=(n, n))
        S = _build(A, dev, True)
        assert S.d16 and S.order is not None and S.padded_nnz >= A.nnz
        order = S.order.cpu().numpy()
        assert np.array_equal(np.sort(order), np.arange(n))
        S2 = _build(A, dev, True)
        assert torch.equal(S.order, S2.order) and torch.equal(S.col16, S2.col16) and torch.equal(S.val64, S2.val64)
        _check_spmv(S, A, dev)


def test_d16_bridges_long_rows_and_identity_fallback():
    dev = cuda()
    import scipy.sparse as sp
    from fealpy_gb300 import kernels as K
    # couplings 150000 apart in a 400000-row matrix: the renumbering puts the
    # coupled rows next to each other; kept in its own numbering, every
    # coupled row needs two bridges
    A = _spd(400000, [150000])
    S = _build(A, dev, True)
    assert S.order is not None and S.padded_nnz >= A.nnz
    _check_spmv(S, A, dev)
    t = lambda a: torch.as_tensor(a, device=dev)
    S = K._sell_build_d16(t(A.indptr.astype(np.int64)), t(A.indices.astype(np.int32)), t(A.data), None, True, True,
                          force=True, renumber=False)
    assert S.order is None and S.padded_nnz >= A.nnz + 2 * 250000
    _check_spmv(S, A, dev)
    # one row with 3000 entries (above the 1024-entry stage) and its column
    B = _spd(20000, [7]).tolil()
    cols = np.arange(0, 20000, 7)[:3000]
    B[5, cols] = -1e-3
    B[cols, 5] = -1e-3
    B = B.tocsr()
    B = (B + sp.diags(np.abs(B).sum(axis=1).A.ravel())).tocsr()
    B.sort_indices()
    _check_spmv(_build(B, dev, True), B, dev)
    # an arrow matrix: every row's smallest column is 0 (one key group of all
    # rows), so the renumbering falls back to the identity
    n = 5000
    C = sp.lil_matrix((n, n))
    C.setdiag(float(n))
    C[0, :] = 1.0
    C[:, 0] = 1.0
    C[0, 0] = float(n) * 2
    C = C.tocsr()
    C.sort_indices()
    S = _build(C, dev, True)
    assert np.array_equal(S.order.cpu().numpy(), np.arange(n))
    _check_spmv(S, C, dev)


def test_d16_solvers_match_int32_columns(golden_dir):
    """cg (FP64) and cg_mixed on the renumbered copy: same stopping test,
    solution in the caller's numbering, within 1e-9 of the 4-byte-column
    solve."""
    dev = cuda()
    import fealpy_gb300 as F
    from fealpy_gb300 import solver as SV
    from fealpy_gb300.sparse import CSRTensor
    z = np.load(os.path.join(golden_dir, "c1_poisson_tri_p1_64.npz"))
    out = {}
    old = SV.SELL_D16
    try:
        for mode in (False, True):
            SV.SELL_D16 = mode
            A = CSRTensor(torch.as_tensor(z["bc_crow"], device=dev), torch.as_tensor(z["bc_col"], device=dev),
                          torch.as_tensor(z["bc_val"], device=dev), (len(z["bc_crow"]) - 1,) * 2)
            b = torch.as_tensor(z["bc_F"], device=dev)
            x64, i64 = F.cg(A, b, M=F.JacobiPreconditioner().apply(A), atol=1e-30, rtol=1e-10, returninfo=True)
            assert A._sell.d16 == mode
            xm, im = F.cg_mixed(A, b, rtol=1e-10, returninfo=True)
            assert im["relres"] <= 1e-10
            out[mode] = (x64, i64["niter"], xm)
    finally:
        SV.SELL_D16 = old
    assert abs(out[True][1] - out[False][1]) <= 1
    assert rel_err(out[True][0], out[False][0].cpu().numpy()) < 1e-9
    assert rel_err(out[True][2], out[False][2].cpu().numpy()) < 1e-8
    assert rel_err(out[True][0], z["uh"]) < 1e-9


def test_d16_block_merge_renumbering(golden_dir):
    """The renumbering from the space's dof blocks: vertex dofs, then edge
    (and for P3 triangles cell) dofs merged by relative position."""
    dev = cuda()
    import scipy.sparse as sp
    for name, blocks in (("small_tet_p2.npz", lambda z: [len(z["node"]), len(z["edge"])]),
                         ("small_tri_p3.npz", lambda z: [len(z["node"]), 2 * len(z["edge"]), len(z["cell"])])):
        z = np.load(os.path.join(golden_dir, name))
        n = len(z["crow"]) - 1
        bl = blocks(z)
        assert sum(bl) == n
        A = sp.csr_matrix((z["val"], z["col"], z["crow"]), shape=(n, n))
        S = _build(A, dev, True, blocks=bl)
        assert np.array_equal(S.order.cpu().numpy(), _merge_order(bl))
        _check_spmv(S, A, dev)


def test_node_triple_copy_matches_csr(golden_dir):
    """Node-triple copy of the P1 elasticity matrices (before and after the
    Dirichlet rows, which leave partial triples): SpMV against scipy."""
    dev = cuda()
    import scipy.sparse as sp
    from fealpy_gb300 import kernels as K
    z = np.load(os.path.join(golden_dir, "small_elasticity_tet_p1.npz"))
    for pre in ("", "bc_"):
        n = len(z[pre + "crow"]) - 1
        A = sp.csr_matrix((z[pre + "val"], z[pre + "col"], z[pre + "crow"]), shape=(n, n))
        A.sort_indices()
        t = lambda a: torch.as_tensor(a, device=dev)
        S = K.sell_build(t(A.indptr.astype(np.int64)), t(A.indices.astype(np.int32)), t(A.data), None,
                         want64=True, want32=True, triples=True)
        assert S.node_triples and S.padded_nnz >= A.nnz and S.order is None
        _check_spmv(S, A, dev)


def test_node_triple_solvers_match_entry_copy(golden_dir):
    """cg and cg_mixed on the elasticity system with node triples against the
    copy with a column per entry: iteration counts within 1, solutions within
    1e-9 (FP64) / 1e-7 (FP32-refined, relres 1e-10)."""
    dev = cuda()
    import fealpy_gb300 as F
    from fealpy_gb300 import solver as SV
    from fealpy_gb300.sparse import CSRTensor
    z = np.load(os.path.join(golden_dir, "small_elasticity_tet_p1.npz"))
    out = {}
    old = SV.SELL_TRIPLES
    try:
        for mode in (False, True):
            SV.SELL_TRIPLES = mode
            A = CSRTensor(torch.as_tensor(z["bc_crow"], device=dev), torch.as_tensor(z["bc_col"], device=dev),
                          torch.as_tensor(z["bc_val"], device=dev), (len(z["bc_crow"]) - 1,) * 2)
            A.node_block = 3
            b = torch.as_tensor(z["bc_F"], device=dev)
            x64, i64 = F.cg(A, b, M=F.JacobiPreconditioner().apply(A), atol=1e-30, rtol=1e-10, returninfo=True)
            assert A._sell.node_triples == mode
            xm, im = F.cg_mixed(A, b, rtol=1e-10, returninfo=True)
            assert im["relres"] <= 1e-10
            out[mode] = (x64, i64["niter"], xm)
    finally:
        SV.SELL_TRIPLES = old
    assert abs(out[True][1] - out[False][1]) <= 1
    assert rel_err(out[True][0], out[False][0].cpu().numpy()) < 1e-9
    assert rel_err(out[True][2], out[False][2].cpu().numpy()) < 1e-7


# ------------------------------------------------------------- 15-bit steps
def _build_d15(A, dev, want64=True, want32=True):
    from fealpy_gb300 import kernels as K
    t = lambda a: torch.as_tensor(a, device=dev)
    return K.sell_build(t(A.indptr.astype(np.int64)), t(A.indices.astype(np.int32)),
                        t(A.data) if want64 else None, None if want64 else t(A.data.astype(np.float32)),
                        want64=want64, want32=want32, d15=True)


def _long_entries(A):
    """Long-step entries the 15-bit copy needs: one per step above 32767 (the
    steps here are below 2^30, which one long step covers)."""
    row = np.repeat(np.arange(A.shape[0]), np.diff(A.indptr))
    same = row[1:] == row[:-1]
    st = np.diff(A.indices.astype(np.int64))[same]
    assert st.max(initial=0) < (1 << 30)
    return int(np.count_nonzero(st > 32767))


def test_d15_golden_and_config_matrices_match_csr(golden_dir):
    """15-bit copies (own numbering) of FEALPy matrices: P2/P3 triangles, P1
    Poisson, and the P2 tetrahedral C2-law matrix whose vertex rows step from
    the vertex block into the edge block (one long step per such row)."""
    dev = cuda()
    import scipy.sparse as sp
    for name in ("small_tet_p2.npz", "small_tri_p3.npz", "c1_poisson_tri_p1_64.npz", "cfg_c2_tet_p2_8.npz"):
        z = np.load(os.path.join(golden_dir, name))
        n = len(z["crow"]) - 1
        for pre in ("", "bc_"):
            A = sp.csr_matrix((z[pre + "val"], z[pre + "col"], z[pre + "crow"]), shape=(n, n))
            S = _build_d15(A, dev)
            assert S.d15 and not S.d16 and S.order is None and S.cols == "d15"
            assert S.stored_entries() == A.nnz + _long_entries(A)
            S2 = _build_d15(A, dev)
            assert torch.equal(S.col16, S2.col16) and torch.equal(S.val32, S2.val32)
            _check_spmv(S, A, dev)


def test_d15_long_steps_empty_rows_and_fp32_operator():
    """Gaps of exactly 32767 and 32768, multiples of 32768, gaps of millions
    (one long-step entry each), empty rows, and an FP32-only copy."""
    dev = cuda()
    import scipy.sparse as sp
    n = 1_500_000
    A = _spd(n, [32767, 32768, 3 * 32768, 1_234_567]).tocoo()
    empty = np.array([5, 77, n - 3])  # empty rows (and columns), as the solvers may meet
    keep = ~(np.isin(A.row, empty) | np.isin(A.col, empty))
    A = sp.csr_matrix((A.data[keep], (A.row[keep], A.col[keep])), shape=(n, n))
    A.sort_indices()
    assert np.all(np.diff(A.indptr)[empty] == 0)
    S = _build_d15(A, dev)
    assert S.stored_entries() == A.nnz + _long_entries(A) and _long_entries(A) > 0
    _check_spmv(S, A, dev)
    from fealpy_gb300 import kernels as K
    S32 = _build_d15(A, dev, want64=False)
    assert S32.val64 is None and S32.val32 is not None
    x = np.random.default_rng(6).normal(size=n)
    y = K.sell_spmv(S32, torch.as_tensor(x, device=dev, dtype=torch.float32), torch.float32)
    assert rel_err(y, A.astype(np.float32).astype(np.float64) @ x) < 1e-5
    # a row whose columns do not ascend is refused
    t = lambda a: torch.as_tensor(a, device=dev)
    bad_ptr = t(np.array([0, 2, 3], dtype=np.int64))
    bad_col = t(np.array([1, 0, 1], dtype=np.int32))
    with pytest.raises(RuntimeError):
        K.sell_build(bad_ptr, bad_col, t(np.ones(3)), None, want64=True, want32=True, d15=True)


def test_d15_solvers_match_the_four_byte_copy(golden_dir):
    """cg_mixed on the 15-bit copy (the default for FP32 copies) against the
    same solve on the 4-byte copy: every row's product is the same sum in the
    same order (a long-step entry adds an exact zero), but the rows sit in
    other slots (their lengths differ) and the kernels' launch shapes group
    the p.Ap partials differently, so the FP32 dot products round
    differently: FP32 iteration counts of these small systems move by a few
    percent with such rounding, so the counts agree within 10% (and 2),
    solutions within 1e-9, and both meet the reference's solution."""
    dev = cuda()
    import fealpy_gb300 as F
    from fealpy_gb300 import solver as SV
    for name in ("c1_poisson_tri_p1_64.npz", "cfg_c2_tet_p2_8.npz"):
        z = np.load(os.path.join(golden_dir, name))
        out = {}
        for d15 in (True, False):
            A = F.CSRTensor(torch.as_tensor(z["bc_crow"], device=dev), torch.as_tensor(z["bc_col"], device=dev),
                            torch.as_tensor(z["bc_val"], device=dev), (len(z["bc_crow"]) - 1,) * 2)
            b = torch.as_tensor(z["bc_F" if "bc_F" in z else "F"], device=dev)
            saved = SV.SELL_D15
            SV.SELL_D15 = d15
            try:
                x, info = F.cg_mixed(A, b, rtol=1e-10, returninfo=True, graph=False)
                assert A._sell.d15 == d15
            finally:
                SV.SELL_D15 = saved
            assert info["relres"] <= 1e-10 and rel_err(x, z["uh"]) < 1e-8, (name, d15, info)
            out[d15] = (x, info["niter"])
        assert abs(out[True][1] - out[False][1]) <= max(2, out[False][1] // 10), (name, out[True][1], out[False][1])
        assert rel_err(out[True][0], out[False][0].cpu().numpy()) < 1e-9, name


def test_d15_pipelined_kernels_match_one_trip_kernels(golden_dir):
    """FP32 products of 15-bit copies run in the pipelined kernel (a warp
    loads its next trip of packs before it gathers the current one) unless
    switched off: its products equal the one-trip kernel's bit for bit (every
    row is the same sum in the same order), on the C2-law matrix and on a
    matrix with long steps, rows wider than a trip and empty rows; the
    FP32-refined solves agree (the p.Ap partials are grouped by the blocks of
    another launch shape: iterations within 10%, solutions within 1e-9)."""
    dev = cuda()
    import scipy.sparse as sp
    import fealpy_gb300 as F
    from fealpy_gb300 import _lib, kernels as K
    from fealpy_gb300 import solver as SV
    z = np.load(os.path.join(golden_dir, "cfg_c2_tet_p2_8.npz"))
    n0 = len(z["bc_crow"]) - 1
    c2 = sp.csr_matrix((z["bc_val"], z["bc_col"], z["bc_crow"]), shape=(n0, n0))
    wide = _spd(200_000, list(range(2, 30)) + [40_000, 1_000_000 % 200_000 + 7], seed=4).tocoo()
    empty = np.array([3, 64, 199_990])
    keep = ~(np.isin(wide.row, empty) | np.isin(wide.col, empty))
    wide = sp.csr_matrix((wide.data[keep], (wide.row[keep], wide.col[keep])), shape=wide.shape)
    wide.sort_indices()
    lib = _lib.lib()
    try:
        for name, A_np in (("c2", c2), ("wide", wide)):
            S = _build_d15(A_np, dev)
            xs = torch.as_tensor(np.random.default_rng(2).normal(size=A_np.shape[0]), device=dev,
                                 dtype=torch.float32)
            lib.fgb_sell_set_pipeline(1)
            y1 = K.sell_spmv(S, xs, torch.float32)
            lib.fgb_sell_set_pipeline(0)
            y0 = K.sell_spmv(S, xs, torch.float32)
            assert torch.equal(y1, y0), name
            if name == "wide":
                continue
            b = torch.as_tensor(z["bc_F"] if "bc_F" in z else z["F"], device=dev)
            out = {}
            for pipe in (1, 0):
                lib.fgb_sell_set_pipeline(pipe)
                A = F.CSRTensor(torch.as_tensor(z["bc_crow"], device=dev), torch.as_tensor(z["bc_col"], device=dev),
                                torch.as_tensor(z["bc_val"], device=dev), (n0, n0))
                saved = SV.SELL_D15
                SV.SELL_D15 = True
                try:
                    x, info = F.cg_mixed(A, b, rtol=1e-10, returninfo=True, graph=False)
                finally:
                    SV.SELL_D15 = saved
                assert info["relres"] <= 1e-10 and rel_err(x, z["uh"]) < 1e-8, (pipe, info)
                out[pipe] = (x, info["niter"])
            assert abs(out[1][1] - out[0][1]) <= max(2, out[0][1] // 10)
            assert rel_err(out[1][0], out[0][0].cpu().numpy()) < 1e-9
    finally:
        lib.fgb_sell_set_pipeline(1)

