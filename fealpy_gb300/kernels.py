"""Host wrappers of the assembly, boundary-condition and solver entry points.

Each function takes and returns torch CUDA tensors, allocates outputs and
workspaces through torch's caching allocator, launches on the current stream
and maps a non-zero status to an exception.  Nothing here computes on the CPU.
"""
import ctypes
from typing import Optional, Sequence, Tuple

import torch

from . import _lib
from ._lib import call, ptr, stream_ptr, workspace, status_word, check_status_word, dtype_code

__all__ = ["cell_factors", "build_adjacency", "build_pattern", "assemble_scalar", "assemble_elasticity_p1",
           "expand_blocks", "dirichlet_apply", "csr_spmv", "csr_diagonal", "pcg_f64", "pcg_mixed", "gather_sum"]


def _values_1d(values, what: str):
    """The C ABI takes one matrix: values (nnz,)."""
    if values is not None and values.ndim != 1:
        raise ValueError(f"{what} takes the values of one matrix, shaped (nnz,), got {tuple(values.shape)}")


def _dev(mesh_or_tensor):
    d = mesh_or_tensor.device
    if d.type != "cuda":
        raise ValueError("the assembly path needs the mesh on a CUDA device")
    return d


def cell_factors(mesh, channels: Sequence[Tuple[int, int, float]], coef: Optional[torch.Tensor],
                 out_dtype=torch.float64, status: Optional[torch.Tensor] = None,
                 cells: Optional[torch.Tensor] = None) -> torch.Tensor:
    """(NC, nch) factor channels, see ``fgb_cell_factors``.  ``channels`` is a
    list of ``(kind, coef_row or -1, scale)``; ``coef`` is (n_coef, NC) float64.
    ``cells``: the factors of these cells only (a sub-region; NC = its size)."""
    dev = _dev(mesh.node)
    cell_arr = mesh.cell if cells is None else mesh.cell[cells].contiguous()
    NC = cell_arr.shape[0]
    nch = len(channels)
    if nch == 0 or nch > _lib.FGB_MAX_CHANNELS:
        raise ValueError(f"between 1 and {_lib.FGB_MAX_CHANNELS} factor channels are supported, got {nch}")
    out = torch.empty((NC, nch), dtype=out_dtype, device=dev)
    if NC == 0:
        return out
    kinds = (ctypes.c_int32 * nch)(*[int(c[0]) for c in channels])
    coefs = (ctypes.c_int32 * nch)(*[int(c[1]) for c in channels])
    scales = (ctypes.c_double * nch)(*[float(c[2]) for c in channels])
    if coef is not None:
        coef = coef.to(device=dev, dtype=torch.float64).contiguous()
    own = status is None
    st = status_word(dev) if own else status
    call("fgb_cell_factors", mesh.TD, NC, ptr(mesh.node), ptr(cell_arr), nch, kinds, coefs, scales, ptr(coef),
         dtype_code(out_dtype), ptr(out), ptr(st), stream_ptr(dev))
    if own:
        check_status_word("fgb_cell_factors", st)
    return out


def build_adjacency(c2d: torch.Tensor, n_dof: int, status: torch.Tensor):
    """dof -> sorted (cell*ldof + local) adjacency."""
    dev = _dev(c2d)
    c2d = c2d.contiguous()
    NC, ldof = c2d.shape
    adj_ptr = torch.empty(n_dof + 1, dtype=torch.int64, device=dev)
    adj = torch.empty(max(NC * ldof, 1), dtype=torch.int32, device=dev)
    max_deg = torch.zeros(1, dtype=torch.int32, device=dev)
    lib = _lib.lib()
    ws = workspace(lib.fgb_adjacency_workspace_bytes(n_dof), dev)
    call("fgb_adjacency_build", NC, ldof, ptr(c2d), n_dof, ptr(adj_ptr), ptr(adj), ptr(max_deg), ptr(status),
         ptr(ws), ws.numel(), stream_ptr(dev))
    return adj_ptr, adj, max_deg


def build_pattern(adj_ptr, adj, c2d, n_dof: int, status: torch.Tensor, positions: bool = False):
    """Canonical CSR pattern (indptr int64, indices int32).  One host sync (nnz).
    With ``positions`` also the within-row slot of every (adjacency entry,
    local dof) pair (uint8, n_adj * ldof), which lets ``assemble_scalar`` skip
    the column search: returns (indptr, indices, positions)."""
    dev = _dev(c2d)
    ldof = c2d.shape[1]
    lib = _lib.lib()
    ws = workspace(lib.fgb_pattern_workspace_bytes(n_dof), dev)
    indptr = torch.empty(n_dof + 1, dtype=torch.int64, device=dev)
    n_adj = int(adj.numel())
    # one hashed pass that stages every sorted row (n_adj * ldof int32 of
    # scratch), then a copy into the exact-size indices
    stage = torch.empty(max(n_adj * ldof, 1), dtype=torch.int32, device=dev)
    pos = torch.empty(max(n_adj * ldof, 1), dtype=torch.uint8, device=dev) if positions else None
    call("fgb_pattern_build", n_dof, ptr(adj_ptr), ptr(adj), ptr(c2d), ldof, n_adj, ptr(indptr), ptr(stage),
         stage.numel() * 4, ptr(pos), ptr(status), ptr(ws), ws.numel(), stream_ptr(dev))
    nnz = int(indptr[n_dof].item())
    check_status_word("fgb_pattern_build", status)
    indices = torch.empty(max(nnz, 1), dtype=torch.int32, device=dev)
    call("fgb_pattern_compact", n_dof, ptr(adj_ptr), ptr(adj), ptr(c2d), ldof, ptr(indptr), ptr(stage),
         ptr(indices), ptr(status), ptr(ws), ws.numel(), stream_ptr(dev))
    if positions:
        return indptr, indices[:nnz], pos
    return indptr, indices[:nnz]


def expand_blocks(n_node: int, bs: int, dof_priority: bool, indptr, indices):
    dev = _dev(indptr)
    nnz_s = indices.numel()
    out_ptr = torch.empty(n_node * bs + 1, dtype=torch.int64, device=dev)
    out_idx = torch.empty(max(nnz_s * bs * bs, 1), dtype=torch.int32, device=dev)
    call("fgb_pattern_expand_blocks", n_node, bs, int(bool(dof_priority)), ptr(indptr), ptr(indices), ptr(out_ptr),
         ptr(out_idx), stream_ptr(dev))
    return out_ptr, out_idx[: nnz_s * bs * bs]


def csr_permute(indptr, indices, values, order: torch.Tensor, inv: torch.Tensor):
    """P A P^T as a canonical CSR: row k of the result is row order[k] of A,
    columns mapped through inv (inv[order[k]] = k) and sorted in each row;
    the values (FP64 or FP32) move with their entries."""
    _values_1d(values, "csr_permute")
    dev = _dev(indptr)
    n = indptr.numel() - 1
    nnz = indices.numel()
    lib = _lib.lib()
    ws = workspace(lib.fgb_sell_d16_workspace_bytes(n), dev)
    new_ptr = torch.empty(n + 1, dtype=torch.int64, device=dev)
    new_idx = torch.empty(max(nnz, 1), dtype=torch.int32, device=dev)
    new_val = torch.empty(max(nnz, 1), dtype=values.dtype, device=dev)
    v64, v32 = (values, None) if values.dtype == torch.float64 else (None, values)
    n64, n32 = (new_val, None) if values.dtype == torch.float64 else (None, new_val)
    # the int32 copies are held until the launch is queued (a temporary freed
    # before the call would hand its block to the next allocation)
    o32 = order.to(torch.int32).contiguous()
    i32 = inv.to(torch.int32).contiguous()
    call("fgb_csr_permute", n, ptr(indptr), ptr(indices), ptr(v64), ptr(v32), ptr(o32), ptr(i32), ptr(new_ptr),
         ptr(new_idx), ptr(n64), ptr(n32), ptr(ws), ws.numel(), stream_ptr(dev))
    return new_ptr, new_idx[:nnz], new_val[:nnz]


def assemble_scalar(adj_ptr, adj, c2d, tables: torch.Tensor, factors: torch.Tensor, indptr, indices,
                    values_f32: bool = False, status: Optional[torch.Tensor] = None,
                    accumulate_into: Optional[torch.Tensor] = None, positions: Optional[torch.Tensor] = None):
    """CSR values of sum_t factors[:, t] * tables[t] over the pattern; with
    ``accumulate_into`` (values of an earlier pass) this pass is added to them;
    ``positions`` (from ``build_pattern(..., positions=True)`` of this
    pattern) replaces the per-contribution column search."""
    dev = _dev(c2d)
    n_dof = adj_ptr.numel() - 1
    ldof = c2d.shape[1]
    dtype = factors.dtype
    nt = tables.shape[0]
    if tables.shape[1:] != (ldof, ldof) or factors.shape[1] != nt:
        raise ValueError("table/factor shapes do not match")
    if accumulate_into is not None:
        if accumulate_into.dtype != dtype or accumulate_into.numel() != indices.numel():
            raise ValueError("accumulate_into must hold the pattern's values in the factor dtype")
        values = accumulate_into
    else:
        values = torch.empty(indices.numel(), dtype=dtype, device=dev)
    v32 = torch.empty(indices.numel(), dtype=torch.float32, device=dev) if values_f32 else None
    if positions is not None and (positions.dtype != torch.uint8 or positions.numel() < adj.numel() * ldof):
        raise ValueError("positions must be the uint8 slot map of this pattern (n_adj * ldof entries)")
    lib = _lib.lib()
    ws = workspace(lib.fgb_assemble_workspace_bytes(n_dof), dev)
    own = status is None
    st = status_word(dev) if own else status
    # converted inputs bound to names: two temporaries in one argument list
    # could share a freed block before the launch
    tab_d = tables.to(dev, dtype).contiguous()
    fac_d = factors.contiguous()
    call("fgb_assemble_scalar_acc", dtype_code(dtype), n_dof, ptr(adj_ptr), ptr(adj), ptr(c2d), ldof, nt,
         ptr(tab_d), ptr(fac_d), ptr(indptr), ptr(indices), ptr(positions), ptr(values),
         ptr(v32), 1 if accumulate_into is not None else 0, ptr(st), ptr(ws), ws.numel(), stream_ptr(dev))
    if own:
        check_status_word("fgb_assemble_scalar", st)
    return values, v32


def source_local(cm, mode: int, f_scalar: float, f, wphi, sv, ldof: int) -> torch.Tensor:
    """(NC, ldof) cell vectors of a scalar source (see ``fgb_source_local``)."""
    dev = cm.device
    NC = cm.numel()
    out = torch.empty((NC, ldof), dtype=torch.float64, device=dev)
    cm_d = cm.to(torch.float64).contiguous()
    f_d = f.to(device=dev, dtype=torch.float64).contiguous() if f is not None else None
    call("fgb_source_local", NC, ldof, wphi.shape[0], ptr(cm_d), mode, float(f_scalar), ptr(f_d), ptr(wphi), ptr(sv),
         ptr(out), stream_ptr(dev))
    return out


def source_gather(adj_ptr, adj, ldof: int, cm, mode: int, f_scalar: float, f, wphi, sv,
                  out: Optional[torch.Tensor] = None) -> torch.Tensor:
    """Global vector of a scalar source over the dof adjacency; adds to ``out``
    when given (see ``fgb_source_gather``)."""
    dev = cm.device
    n = adj_ptr.numel() - 1
    acc = out is not None
    if out is None:
        out = torch.empty(n, dtype=torch.float64, device=dev)
    cm_d = cm.to(torch.float64).contiguous()
    f_d = f.to(device=dev, dtype=torch.float64).contiguous() if f is not None else None
    call("fgb_source_gather", n, ptr(adj_ptr), ptr(adj), ldof, wphi.shape[0], ptr(cm_d), mode, float(f_scalar),
         ptr(f_d), ptr(wphi), ptr(sv), ptr(out), 1 if acc else 0, stream_ptr(dev))
    return out


def pcg_multi(indptr, indices, values, dinv, B: torch.Tensor, X: torch.Tensor, atol: float, rtol: float,
              maxit: int):
    """Jacobi-PCG (``dinv`` None: plain CG) on every column of B (n, k),
    FEALPy's multi-right-hand-side recurrence; X (n, k) in/out."""
    dev = B.device
    n, k = B.shape
    lib = _lib.lib()
    nb = lib.fgb_pcg_multi_workspace_bytes(n, k)
    if nb == 0:
        raise ValueError(f"between 1 and 64 right-hand sides are supported, got {k}")
    ws = workspace(nb, dev)
    info = _lib.PcgInfo()
    vals = values.to(torch.float64).contiguous()
    b_d = B.to(torch.float64).contiguous()
    call("fgb_pcg_multi_f64", n, k, ptr(indptr), ptr(indices), ptr(vals), ptr(dinv), ptr(b_d), ptr(X), float(atol),
         float(rtol), int(maxit), ctypes.byref(info), ptr(ws), ws.numel(), stream_ptr(dev))
    _lib.add_launches(info.launches)
    return info


def local_matrices(factors: torch.Tensor, tables: torch.Tensor, out: Optional[torch.Tensor] = None) -> torch.Tensor:
    """(NC, ldof, ldof) local matrices sum_t factors[:, t] * tables[t]; with
    ``out`` (an earlier pass) this pass is added to it."""
    dev = factors.device
    NC, nt = factors.shape
    ldof = tables.shape[1]
    if tables.shape != (nt, ldof, ldof):
        raise ValueError("table/factor shapes do not match")
    acc = out is not None
    if out is None:
        out = torch.empty((NC, ldof, ldof), dtype=factors.dtype, device=dev)
    tab_d = tables.to(dev, factors.dtype).contiguous()
    fac_d = factors.contiguous()
    call("fgb_local_matrices", dtype_code(factors.dtype), NC, ldof, nt, ptr(tab_d), ptr(fac_d), ptr(out),
         1 if acc else 0, stream_ptr(dev))
    return out


def local_elasticity_p1(mesh, plan, priority: bool = False) -> torch.Tensor:
    """(NC, (GD+1) GD, (GD+1) GD) P1 elasticity local matrices from the
    plan's factor channels (its cells); ``priority``: component-major local
    order."""
    dev = _dev(mesh.node)
    gd = plan.gd
    f = cell_factors(mesh, plan.channels, plan.coef_matrix(), torch.float64, cells=plan.cells)
    ld = (gd + 1) * gd
    out = torch.empty((f.shape[0], ld, ld), dtype=torch.float64, device=dev)
    call("fgb_local_elasticity_p1", dtype_code(torch.float64), gd, f.shape[0], ptr(f), 1 if priority else 0,
         ptr(out), stream_ptr(dev))
    return out


def assemble_elasticity_p1(gd, adj_ptr, adj, cell, factors, node_indptr, node_indices, indptr, nnz,
                           values_f32: bool = False, status: Optional[torch.Tensor] = None):
    dev = _dev(cell)
    n_node = adj_ptr.numel() - 1
    dtype = factors.dtype
    values = torch.empty(nnz, dtype=dtype, device=dev)
    v32 = torch.empty(nnz, dtype=torch.float32, device=dev) if values_f32 else None
    lib = _lib.lib()
    ws = workspace(lib.fgb_assemble_workspace_bytes(n_node), dev)
    own = status is None
    st = status_word(dev) if own else status
    fac_d = factors.contiguous()
    call("fgb_assemble_elasticity_p1", dtype_code(dtype), gd, n_node, ptr(adj_ptr), ptr(adj), ptr(cell),
         ptr(fac_d), ptr(node_indptr), ptr(node_indices), ptr(indptr), ptr(values), ptr(v32), ptr(st),
         ptr(ws), ws.numel(), stream_ptr(dev))
    if own:
        check_status_word("fgb_assemble_elasticity_p1", st)
    return values, v32


def dirichlet_apply(indptr, indices, values, is_bd: torch.Tensor, f: Optional[torch.Tensor],
                    uh: Optional[torch.Tensor], matrix: bool = True):
    """Returns (new_indptr, new_indices, new_values, f_new); entries not asked for are None.
    ``uh`` None with ``f`` given: all boundary values zero."""
    _values_1d(values, "dirichlet_apply")
    dev = _dev(indptr)
    n = indptr.numel() - 1
    dt = values.dtype
    isb = is_bd.to(device=dev, dtype=torch.uint8).contiguous()
    row_nnz = torch.empty(n, dtype=torch.int32, device=dev)
    f_out = None
    if f is not None:
        f_out = torch.empty(n, dtype=dt, device=dev)
        f = f.to(dev, dt).contiguous()
        # uh None: homogeneous boundary data (the kernel skips A uh)
        uh = uh.to(dev, dt).contiguous() if uh is not None else None
    call("fgb_dirichlet_count", dtype_code(dt), n, ptr(indptr), ptr(indices), ptr(values), ptr(isb), ptr(f), ptr(uh),
         ptr(f_out), ptr(row_nnz), stream_ptr(dev))
    if not matrix:
        return None, None, None, f_out
    lib = _lib.lib()
    ws = workspace(lib.fgb_scan_workspace_bytes(n), dev)
    new_ptr = torch.empty(n + 1, dtype=torch.int64, device=dev)
    call("fgb_exclusive_scan_i32", ptr(row_nnz), n, ptr(new_ptr), ptr(ws), ws.numel(), stream_ptr(dev))
    nnz = int(new_ptr[n].item())
    new_idx = torch.empty(max(nnz, 1), dtype=torch.int32, device=dev)
    new_val = torch.empty(max(nnz, 1), dtype=dt, device=dev)
    call("fgb_dirichlet_fill", dtype_code(dt), n, ptr(indptr), ptr(indices), ptr(values), ptr(isb), ptr(new_ptr),
         ptr(new_idx), ptr(new_val), stream_ptr(dev))
    return new_ptr, new_idx[:nnz], new_val[:nnz], f_out


def csr_spmv(indptr, indices, values, x, lanes: int = 0, out: Optional[torch.Tensor] = None):
    _values_1d(values, "csr_spmv")
    dev = _dev(indptr)
    n = indptr.numel() - 1
    x = x.to(dev, values.dtype).contiguous()
    y = out if out is not None else torch.empty(n, dtype=values.dtype, device=dev)
    call("fgb_csr_spmv", dtype_code(values.dtype), n, ptr(indptr), ptr(indices), ptr(values), ptr(x), ptr(y), lanes,
         stream_ptr(dev))
    return y


def residual_norm(indptr, indices, values, b, x):
    """(||b - A x||, ||b||) of an FP64 CSR matrix, formed on the device in one
    pass (``fgb_residual_norm``); one host read of the two sums."""
    dev = _dev(indptr)
    n = indptr.numel() - 1
    vals = values.to(torch.float64).contiguous()
    bd = b.to(dev, torch.float64).contiguous()
    xd = x.to(dev, torch.float64).contiguous()
    out = torch.empty(2, dtype=torch.float64, device=dev)
    lib = _lib.lib()
    ws = workspace(lib.fgb_residual_norm_workspace_bytes(), dev)
    call("fgb_residual_norm", n, ptr(indptr), ptr(indices), ptr(vals), ptr(bd), ptr(xd), ptr(out), ptr(ws),
         ws.numel(), stream_ptr(dev))
    rr, bb = out.cpu().tolist()
    return rr ** 0.5, bb ** 0.5


def csr_spmm(indptr, indices, values, X: torch.Tensor) -> torch.Tensor:
    """Y = A X for X (m, k) row-major FP64, k <= 64, in one pass over the matrix."""
    _values_1d(values, "csr_spmm")
    dev = _dev(indptr)
    n = indptr.numel() - 1
    k = X.shape[1]
    X = X.to(dev, torch.float64).contiguous()
    Y = torch.empty((n, k), dtype=torch.float64, device=dev)
    vals = values.contiguous()
    call("fgb_csr_spmm_f64", n, k, ptr(indptr), ptr(indices), ptr(vals), ptr(X), ptr(Y), stream_ptr(dev))
    return Y


def csr_diagonal(indptr, indices, values):
    _values_1d(values, "csr_diagonal")
    dev = _dev(indptr)
    n = indptr.numel() - 1
    d = torch.empty(n, dtype=values.dtype, device=dev)
    dinv = torch.empty(n, dtype=values.dtype, device=dev)
    call("fgb_csr_diagonal", dtype_code(values.dtype), n, ptr(indptr), ptr(indices), ptr(values), ptr(d), ptr(dinv),
         stream_ptr(dev))
    return d, dinv


def pcg_f64(indptr, indices, values, dinv, b, x, atol, rtol, maxit, check_every=16, lanes=0, norm=0, profile=False):
    _values_1d(values, "pcg_f64")
    dev = _dev(indptr)
    n = indptr.numel() - 1
    lib = _lib.lib()
    ws = workspace(lib.fgb_pcg_workspace_bytes(n), dev)
    info = _lib.PcgInfo()
    call("fgb_pcg_f64", n, ptr(indptr), ptr(indices), ptr(values), ptr(dinv), ptr(b), ptr(x), float(atol),
         float(rtol), int(maxit), int(check_every), int(lanes), int(norm), int(bool(profile)), ptr(ws), ws.numel(),
         ctypes.byref(info), stream_ptr(dev))
    _lib.add_launches(info.launches)
    return info


def pcg_mixed(indptr, indices, values64, values32, dinv64, b, x, rtol, delta=0.2, maxit=100000, check_every=32,
              lanes=0, profile=False):
    dev = _dev(indptr)
    n = indptr.numel() - 1
    lib = _lib.lib()
    ws = workspace(lib.fgb_pcg_mixed_workspace_bytes(n), dev)
    info = _lib.PcgInfo()
    call("fgb_pcg_mixed", n, ptr(indptr), ptr(indices), ptr(values64), ptr(values32), ptr(dinv64), ptr(b), ptr(x),
         float(rtol), float(delta), int(maxit), int(check_every), int(lanes), int(bool(profile)), ptr(ws),
         ws.numel(), ctypes.byref(info), stream_ptr(dev))
    _lib.add_launches(info.launches)
    return info


def gather_sum(adj_ptr, adj, local: torch.Tensor, out: Optional[torch.Tensor] = None):
    """out[i] = sum of local.flat[adj[k]] over i's adjacency (deterministic)."""
    dev = _dev(adj_ptr)
    n = adj_ptr.numel() - 1
    local = local.contiguous()
    y = out if out is not None else torch.empty(n, dtype=local.dtype, device=dev)
    call("fgb_gather_sum", dtype_code(local.dtype), n, ptr(adj_ptr), ptr(adj), ptr(local), ptr(y), stream_ptr(dev))
    return y


def mesh_entities(cell: torch.Tensor, n_node: int, local, want_entity2cell: bool):
    """(entity (NE, k), entity2cell (NE, 4) or None, cell2entity (NC, nfc)),
    int32, of the local entities ``local`` (nfc x k vertex indices) of every
    cell (``fgb_topology_count`` + ``fgb_topology_fill``)."""
    import numpy as np
    dev = _dev(cell)
    cell = cell.to(torch.int32).contiguous()
    NC, nv = cell.shape
    loc = np.ascontiguousarray(local, dtype=np.int32)
    nfc, k = loc.shape
    lib = _lib.lib()
    ws = workspace(lib.fgb_topology_workspace_bytes(n_node, NC * nfc), dev)
    st = status_word(dev)
    lp = loc.ctypes.data_as(ctypes.c_void_p)
    ne = ctypes.c_int64(0)
    s = stream_ptr(dev)
    call("fgb_topology_count", NC, nv, ptr(cell), int(n_node), k, nfc, lp, ctypes.byref(ne), ptr(st), ptr(ws),
         ws.numel(), s)
    check_status_word("mesh topology (cell vertex indices)", st)
    NE = int(ne.value)
    entity = torch.empty((NE, k), dtype=torch.int32, device=dev)
    e2c = torch.empty((NE, 4), dtype=torch.int32, device=dev) if want_entity2cell else None
    c2e = torch.empty((NC, nfc), dtype=torch.int32, device=dev)
    call("fgb_topology_fill", NC, nv, ptr(cell), int(n_node), k, nfc, lp, ptr(entity), ptr(e2c), ptr(c2e), ptr(st),
         ptr(ws), ws.numel(), s)
    check_status_word("mesh topology", st)
    return entity, e2c, c2e


def cell_to_ipoint(mesh, p: int) -> torch.Tensor:
    """(NC, ldof) int32 interpolation-point numbering of a mesh on the device
    (``fgb_cell_to_ipoint``): the per-point table is built here from the
    multi-index matrix, the numbering by one thread per (cell, point)."""
    import numpy as np
    from . import simplex as sx
    TD = mesh.TD
    mi = sx.multi_index_matrix(p, TD)
    ldof = mi.shape[0]
    local_edge = [(1, 2), (2, 0), (0, 1)] if TD == 2 else list(mesh.localEdge)
    edge_id = {tuple(sorted(e)): q for q, e in enumerate(local_edge)}
    tab = {name: np.zeros(ldof, dtype=np.int32) for name in ("kind", "a", "b", "le", "ma", "mb", "rank")}
    interior = 0
    for q in range(ldof):
        support = np.nonzero(mi[q] > 0)[0]
        if len(support) == 1:
            tab["kind"][q], tab["a"][q] = 0, support[0]
        elif len(support) == 2:
            a, b = int(support[0]), int(support[1])
            tab["kind"][q], tab["a"][q], tab["b"][q] = 1, a, b
            tab["le"][q], tab["ma"][q], tab["mb"][q] = edge_id[(a, b)], mi[q, a], mi[q, b]
        elif TD == 2:
            tab["kind"][q], tab["rank"][q] = 2, interior
            interior += 1
        else:
            # P3 tetrahedron: the point of the face opposite the vertex whose entry is 0
            tab["kind"][q], tab["le"][q] = 3, int(np.nonzero(mi[q] == 0)[0][0])
    dev = _dev(mesh.cell)
    NC = mesh.number_of_cells()
    out = torch.empty((NC, ldof), dtype=torch.int32, device=dev)
    hp = [tab[k].ctypes.data_as(ctypes.c_void_p) for k in ("kind", "a", "b", "le", "ma", "mb", "rank")]
    c2f = mesh.cell2face if TD == 3 else None
    c2e_d, edge_d = mesh.cell2edge.contiguous(), mesh.edge.contiguous()
    c2f_d = c2f.contiguous() if c2f is not None else None
    call("fgb_cell_to_ipoint", NC, TD, p, ldof, ptr(mesh.cell), ptr(c2e_d),
         ptr(edge_d), ptr(c2f_d), mesh.number_of_nodes(),
         mesh.number_of_edges(), *hp, ptr(out), stream_ptr(dev))
    return out


def cell_apply(c2d, tables: "np.ndarray", factors: torch.Tensor, x: torch.Tensor) -> torch.Tensor:
    """(NC, ldof) cell products K_c x_c (``fgb_cell_apply``) in the factors'
    dtype; ``tables`` is the (nt, ldof, ldof) FP64 table array on the host."""
    import numpy as np
    dev = _dev(c2d)
    NC, ldof = c2d.shape
    nt = factors.shape[1]
    dt = factors.dtype
    tab_host = np.ascontiguousarray(tables, dtype=np.float64)
    if tab_host.shape != (nt, ldof, ldof):
        raise ValueError(f"tables must be ({nt}, {ldof}, {ldof})")
    tab_dev = None if ldof in (3, 4, 6, 10) else torch.as_tensor(tab_host, dtype=dt, device=dev)
    y = torch.empty((NC, ldof), dtype=dt, device=dev)
    c2d_d, fac_d, x_d = c2d.contiguous(), factors.contiguous(), x.to(dt).contiguous()
    call("fgb_cell_apply", dtype_code(dt), NC, ldof, ptr(c2d_d), nt,
         tab_host.ctypes.data_as(ctypes.c_void_p), ptr(tab_dev), ptr(fac_d),
         ptr(x_d), ptr(y), stream_ptr(dev))
    return y


class SellMatrix:
    """Device SELL-32 copy of a CSR matrix (tensors kept alive here) and the
    ``fgb_sell`` descriptor pointing at them.

    With 4-byte columns (``col``) the copy is in the matrix's own numbering.
    The delta-coded copy (``col16`` + ``col0``) is of P A P^T for the
    locality renumbering ``order`` (new row k = old row order[k]); the solver
    and SpMV wrappers below permute vectors into and out of that numbering."""

    def __init__(self, n, n_slices, slice_ptr, perm, col, val64, val32, col16=None, col0=None, order=None,
                 nnz=None, node_triples=False, d15=False):
        self.n, self.n_slices = n, n_slices
        self.slice_ptr, self.perm, self.col, self.val64, self.val32 = slice_ptr, perm, col, val64, val32
        self.col16, self.col0, self.order, self.nnz = col16, col0, order, nnz
        self.node_triples = bool(node_triples)
        self._d15 = bool(d15)
        self.desc = _lib.SellDesc(n, n_slices, slice_ptr.data_ptr(), perm.data_ptr(),
                                  col.data_ptr() if col is not None else None,
                                  val64.data_ptr() if val64 is not None else None,
                                  val32.data_ptr() if val32 is not None else None, 0, 0,
                                  col16.data_ptr() if col16 is not None else None,
                                  col0.data_ptr() if col0 is not None else None, 1 if node_triples else 0,
                                  1 if d15 else 0)

    @property
    def d16(self) -> bool:
        """16-bit steps of a renumbered matrix."""
        return self.col16 is not None and not self._d15

    @property
    def d15(self) -> bool:
        """15-bit steps with long steps, in the matrix's own numbering."""
        return self._d15

    def stored_entries(self) -> int:
        """Slots of the copy without padding: the nonzeros, plus the long-step
        entries of a 15-bit copy; triple slots of a node-triple copy (one
        host read)."""
        ep = getattr(self, "entry_indptr", None)
        return int(ep[-1].item()) if ep is not None else int(self.nnz or 0)

    @property
    def cols(self) -> str:
        """Column storage: 'i32', 'd16', 'd15' or 'triples'."""
        if self.node_triples:
            return "triples"
        return "d15" if self._d15 else ("d16" if self.col16 is not None else "i32")

    @property
    def device(self):
        return self.slice_ptr.device

    @property
    def padded_nnz(self):
        """Stored entries including padding (three per slot for node triples)."""
        if self.node_triples:
            return 3 * self.col.numel()
        return (self.col16 if self.col16 is not None else self.col).numel()

    def to_inner(self, v: torch.Tensor) -> torch.Tensor:
        """A vector in the copy's numbering (a new tensor when renumbered)."""
        if self.order is None or v is None:
            return v
        v = v.contiguous()
        out = torch.empty_like(v)
        call("fgb_permute", dtype_code(v.dtype), self.n, ptr(self.order), ptr(v), ptr(out), 0, stream_ptr(v.device))
        return out

    def to_outer(self, v: torch.Tensor, out: Optional[torch.Tensor] = None) -> torch.Tensor:
        """Back to the matrix's own numbering (into ``out`` if given)."""
        if self.order is None:
            if out is not None and out is not v:
                out.copy_(v)
                return out
            return v
        res = out if out is not None else torch.empty_like(v)
        v_d = v.contiguous()
        call("fgb_permute", dtype_code(v.dtype), self.n, ptr(self.order), ptr(v_d), ptr(res), 1,
             stream_ptr(v.device))
        return res

    def set_launch(self, threads: int = 0, blocks: int = 0):
        """Launch shape of the slice kernels (0, 0 = library defaults)."""
        if threads and (threads % 32 or not 32 <= threads <= 1024):
            raise ValueError("threads must be a multiple of 32 in [32, 1024]")
        if blocks and not 1 <= blocks <= SELL_MAX_BLOCKS:
            raise ValueError(f"blocks must be in [1, {SELL_MAX_BLOCKS}]")
        self.desc.threads, self.desc.blocks = int(threads), int(blocks)

    @property
    def launch(self):
        return int(self.desc.threads), int(self.desc.blocks)


SELL_MAX_BLOCKS = 152 * 8
# (threads, blocks cap) candidates of the slice-kernel autotuner: 8, 4, 2 and
# 1 resident 256/512/1024-thread blocks per SM, plus grid-stride variants
SELL_LAUNCH_CANDIDATES = ((256, 1216), (512, 608), (1024, 304), (1024, 152), (256, 608), (128, 1216))


def sell_autotune(S: SellMatrix, dtype=torch.float32, reps: int = 20, candidates=SELL_LAUNCH_CANDIDATES):
    """Pick the launch shape of the slice kernels by timing the SELL SpMV with
    CUDA events on the current stream (after one warm-up call per shape).
    Sets it on ``S`` and returns ``{(threads, blocks): microseconds}``."""
    dev = S.device
    x = torch.rand(S.n, dtype=dtype, device=dev)
    y = torch.empty(S.n, dtype=dtype, device=dev)
    code = dtype_code(dtype)
    s = torch.cuda.current_stream(dev)
    times = {}
    for t, b in candidates:
        S.set_launch(t, b)
        call("fgb_sell_spmv", code, ctypes.byref(S.desc), ptr(x), ptr(y), stream_ptr(dev))
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(s)
        for _ in range(reps):
            call("fgb_sell_spmv", code, ctypes.byref(S.desc), ptr(x), ptr(y), stream_ptr(dev))
        e1.record(s)
        e1.synchronize()
        times[(t, b)] = 1000.0 * e0.elapsed_time(e1) / reps
    best = min(times, key=times.get)
    S.set_launch(*best)
    return times


# A delta-coded copy is kept when its entries (with bridges) are at most this
# many times the nonzeros: 6 bytes per entry against 8.
D16_MAX_GROWTH = 1.25


def sell_build(indptr, indices, values64=None, values32=None, want64=True, want32=False,
               d16: Optional[bool] = None, blocks: Optional[Sequence[int]] = None,
               triples: bool = False, d15: bool = False) -> SellMatrix:
    """SELL-32 copy of a CSR matrix.  ``d15``: 15-bit column steps with long
    steps in the matrix's own numbering (columns must ascend in every row;
    ``d16`` ignored).  ``d16``: True = delta-coded columns of the renumbered
    matrix, False = 4-byte columns, None = delta-coded when the bridges add
    at most 25% entries (two host reads for the sizes).  ``blocks``: the dof
    block sizes of the space (``dof_blocks()``) for the block-merge
    renumbering; without them the rows are ordered by their smallest column.
    ``triples``: node-triple copy for a vector space with three interleaved
    components (rows a multiple of 3; ``d16`` and ``d15`` ignored)."""
    _values_1d(values64, "sell_build")
    _values_1d(values32, "sell_build")
    dev = _dev(indptr)
    n = indptr.numel() - 1
    lib = _lib.lib()
    if triples:
        return _sell_build_b3(indptr, indices, values64, values32, want64, want32)
    if d15:
        return _sell_build_d15(indptr, indices, values64, values32, want64, want32)
    if d16 is None or d16:
        S = _sell_build_d16(indptr, indices, values64, values32, want64, want32, force=bool(d16), blocks=blocks)
        if S is not None:
            return S
    slots = int(lib.fgb_sell_slots(n))
    n_slices = slots // 32
    perm = torch.empty(slots, dtype=torch.int32, device=dev)
    slice_ptr = torch.empty(n_slices + 1, dtype=torch.int64, device=dev)
    ws = workspace(lib.fgb_sell_workspace_bytes(n), dev)
    call("fgb_sell_plan", n, ptr(indptr), ptr(perm), ptr(slice_ptr), ptr(ws), ws.numel(), stream_ptr(dev))
    total = int(slice_ptr[n_slices].item())
    col = torch.empty(max(total, 1), dtype=torch.int32, device=dev)
    v64 = torch.empty(max(total, 1), dtype=torch.float64, device=dev) if want64 else None
    v32 = torch.empty(max(total, 1), dtype=torch.float32, device=dev) if want32 else None
    call("fgb_sell_fill", n, ptr(indptr), ptr(indices), ptr(values64), ptr(values32), ptr(perm), ptr(slice_ptr),
         ptr(col), ptr(v64), ptr(v32), stream_ptr(dev))
    return SellMatrix(n, n_slices, slice_ptr, perm, col, v64, v32, nnz=indices.numel())


def _sell_build_d16(indptr, indices, values64, values32, want64, want32, force=False,
                    renumber=True, blocks: Optional[Sequence[int]] = None) -> Optional[SellMatrix]:
    """Delta-coded copy of P A P^T (None when not worth it and not forced).
    ``renumber=False`` keeps the matrix's own numbering (columns must be
    ascending in every row; steps above 65535 are bridged)."""
    dev = _dev(indptr)
    n = indptr.numel() - 1
    nnz = indices.numel()
    lib = _lib.lib()
    s = stream_ptr(dev)
    ws = workspace(max(lib.fgb_sell_d16_workspace_bytes(n), lib.fgb_sell_workspace_bytes(n)), dev)
    if renumber:
        order = torch.empty(n, dtype=torch.int32, device=dev)
        inv = torch.empty(n, dtype=torch.int32, device=dev)
        nb = len(blocks) if blocks else 0
        if nb and sum(int(v) for v in blocks) != n:
            raise ValueError("dof blocks do not add up to the matrix size")
        sizes = (ctypes.c_int64 * max(nb, 1))(*[int(v) for v in (blocks or [])])
        call("fgb_sell_renumber", n, ptr(indptr), ptr(indices), nb, sizes, ptr(order), ptr(inv), ptr(ws), ws.numel(),
             s)
        if not nb:
            _lib.add_launches(6)  # key pass, 3 scan kernels, placement, group sort
        p_indptr = torch.empty(n + 1, dtype=torch.int64, device=dev)
        p_indices = torch.empty(max(nnz, 1), dtype=torch.int32, device=dev)
        p64 = torch.empty(max(nnz, 1), dtype=torch.float64, device=dev) if want64 else None
        p32 = torch.empty(max(nnz, 1), dtype=torch.float32, device=dev) if want32 else None
        call("fgb_csr_permute", n, ptr(indptr), ptr(indices), ptr(values64), ptr(values32), ptr(order), ptr(inv),
             ptr(p_indptr), ptr(p_indices), ptr(p64), ptr(p32), ptr(ws), ws.numel(), s)
        del inv
    else:
        order, p_indptr, p_indices, p64, p32 = None, indptr, indices, values64, values32
    b_indptr = torch.empty(n + 1, dtype=torch.int64, device=dev)
    call("fgb_sell_d16_indptr", n, ptr(p_indptr), ptr(p_indices), ptr(b_indptr), ptr(ws), ws.numel(), s)
    if not force and int(b_indptr[n].item()) > D16_MAX_GROWTH * max(nnz, 1):
        return None
    slots = int(lib.fgb_sell_slots(n))
    n_slices = slots // 32
    perm = torch.empty(slots, dtype=torch.int32, device=dev)
    slice_ptr = torch.empty(n_slices + 1, dtype=torch.int64, device=dev)
    call("fgb_sell_plan", n, ptr(b_indptr), ptr(perm), ptr(slice_ptr), ptr(ws), ws.numel(), s)
    total = int(slice_ptr[n_slices].item())
    col0 = torch.empty(slots, dtype=torch.int32, device=dev)
    col16 = torch.empty(max(total, 4), dtype=torch.int16, device=dev)
    v64 = torch.empty(max(total, 1), dtype=torch.float64, device=dev) if want64 else None
    v32 = torch.empty(max(total, 1), dtype=torch.float32, device=dev) if want32 else None
    call("fgb_sell_fill_d16", n, ptr(p_indptr), ptr(p_indices), ptr(p64), ptr(p32), ptr(perm), ptr(slice_ptr),
         ptr(col0), ptr(col16), ptr(v64), ptr(v32), s)
    return SellMatrix(n, n_slices, slice_ptr, perm, None, v64, v32, col16=col16, col0=col0, order=order, nnz=nnz)


def _sell_build_d15(indptr, indices, values64, values32, want64, want32) -> SellMatrix:
    """15-bit column copy in the matrix's own numbering."""
    dev = _dev(indptr)
    n = indptr.numel() - 1
    nnz = indices.numel()
    lib = _lib.lib()
    s = stream_ptr(dev)
    ws = workspace(max(lib.fgb_sell_d16_workspace_bytes(n), lib.fgb_sell_workspace_bytes(n)), dev)
    st = status_word(dev)
    e_indptr = torch.empty(n + 1, dtype=torch.int64, device=dev)
    call("fgb_sell_d15_indptr", n, ptr(indptr), ptr(indices), ptr(e_indptr), ptr(st), ptr(ws), ws.numel(), s)
    slots = int(lib.fgb_sell_slots(n))
    n_slices = slots // 32
    perm = torch.empty(slots, dtype=torch.int32, device=dev)
    slice_ptr = torch.empty(n_slices + 1, dtype=torch.int64, device=dev)
    call("fgb_sell_plan", n, ptr(e_indptr), ptr(perm), ptr(slice_ptr), ptr(ws), ws.numel(), s)
    # one host read for the status of the length pass and the copy's size
    code, total = (int(v) for v in torch.stack([st.to(torch.int64)[0], slice_ptr[n_slices]]).cpu())
    if code:
        raise _lib.FgbError("sell_build(d15): columns must ascend strictly in every row", code)
    col0 = torch.empty(slots, dtype=torch.int32, device=dev)
    col16 = torch.empty(max(total, 4), dtype=torch.int16, device=dev)
    v64 = torch.empty(max(total, 1), dtype=torch.float64, device=dev) if want64 else None
    v32 = torch.empty(max(total, 1), dtype=torch.float32, device=dev) if want32 else None
    call("fgb_sell_fill_d15", n, ptr(indptr), ptr(indices), ptr(values64), ptr(values32), ptr(perm), ptr(slice_ptr),
         ptr(col0), ptr(col16), ptr(v64), ptr(v32), s)
    S = SellMatrix(n, n_slices, slice_ptr, perm, None, v64, v32, col16=col16, col0=col0, nnz=nnz, d15=True)
    S.entry_indptr = e_indptr  # entries per row with the long steps (``stored_entries``)
    return S


def _sell_build_b3(indptr, indices, values64, values32, want64, want32) -> SellMatrix:
    """Node-triple copy: a 4-byte column per run of three consecutive columns."""
    dev = _dev(indptr)
    n = indptr.numel() - 1
    if n % 3:
        raise ValueError("a node-triple copy needs a multiple of 3 rows")
    lib = _lib.lib()
    s = stream_ptr(dev)
    ws = workspace(max(lib.fgb_sell_d16_workspace_bytes(n), lib.fgb_sell_workspace_bytes(n)), dev)
    t_indptr = torch.empty(n + 1, dtype=torch.int64, device=dev)
    call("fgb_sell_b3_indptr", n, ptr(indptr), ptr(indices), ptr(t_indptr), ptr(ws), ws.numel(), s)
    slots = int(lib.fgb_sell_slots(n))
    n_slices = slots // 32
    perm = torch.empty(slots, dtype=torch.int32, device=dev)
    slice_ptr = torch.empty(n_slices + 1, dtype=torch.int64, device=dev)
    call("fgb_sell_plan", n, ptr(t_indptr), ptr(perm), ptr(slice_ptr), ptr(ws), ws.numel(), s)
    total = int(slice_ptr[n_slices].item())
    col = torch.empty(max(total, 4), dtype=torch.int32, device=dev)
    v64 = torch.empty(3 * max(total, 4), dtype=torch.float64, device=dev) if want64 else None
    v32 = torch.empty(3 * max(total, 4), dtype=torch.float32, device=dev) if want32 else None
    call("fgb_sell_fill_b3", n, ptr(indptr), ptr(indices), ptr(values64), ptr(values32), ptr(perm), ptr(slice_ptr),
         ptr(col), ptr(v64), ptr(v32), s)
    S = SellMatrix(n, n_slices, slice_ptr, perm, col, v64, v32, nnz=indices.numel(), node_triples=True)
    S.entry_indptr = t_indptr  # triples per row (``stored_entries`` counts triple slots)
    return S


def sell_spmv(S: SellMatrix, x, dtype=torch.float64):
    """y = A x in the matrix's own numbering."""
    dev = S.device
    x = S.to_inner(x.to(dev, dtype).contiguous())
    y = torch.empty(S.n, dtype=dtype, device=dev)
    call("fgb_sell_spmv", dtype_code(dtype), ctypes.byref(S.desc), ptr(x), ptr(y), stream_ptr(dev))
    return S.to_outer(y)


def pcg_sell_f64(S: SellMatrix, dinv, b, x, atol, rtol, maxit, check_every=16, norm=0, graph=True, profile=False):
    """Jacobi-PCG in FP64 on the SELL copy; dinv, b and x (updated in place)
    in the matrix's own numbering."""
    dev = S.device
    lib = _lib.lib()
    ws = workspace(lib.fgb_pcg_sell_workspace_bytes(S.n), dev)
    info = _lib.PcgInfo()
    di, bi, xi = S.to_inner(dinv), S.to_inner(b), S.to_inner(x)
    call("fgb_pcg_sell_f64", ctypes.byref(S.desc), ptr(di), ptr(bi), ptr(xi), float(atol), float(rtol), int(maxit),
         int(check_every), int(norm), int(bool(graph)), int(bool(profile)), ptr(ws), ws.numel(), ctypes.byref(info),
         stream_ptr(dev))
    S.to_outer(xi, out=x)
    _lib.add_launches(info.launches)
    return info


def pcg_sell_mixed(S: SellMatrix, dinv64, b, x, rtol, delta=0.2, maxit=100000, check_every=32, graph=True,
                   profile=False, barrier_polls=0):
    """FP32 Jacobi-PCG with FP64 reliable updates on the SELL copy; dinv64, b
    and x (updated in place) in the matrix's own numbering.  ``graph``: 0
    host-polled loop, 1 CUDA-graph loop, 2 one persistent cooperative kernel,
    whose grid barriers wait at most ``barrier_polls`` polls (0: the default
    limit) before every block returns and the call raises."""
    dev = S.device
    lib = _lib.lib()
    ws = workspace(lib.fgb_pcg_sell_workspace_bytes(S.n), dev)
    info = _lib.PcgInfo()
    di, bi, xi = S.to_inner(dinv64), S.to_inner(b), S.to_inner(x)
    call("fgb_pcg_sell_mixed_ex", ctypes.byref(S.desc), ptr(di), ptr(bi), ptr(xi), float(rtol), float(delta),
         int(maxit), int(check_every), int(graph), int(bool(profile)), int(barrier_polls), ptr(ws), ws.numel(),
         ctypes.byref(info), stream_ptr(dev))
    S.to_outer(xi, out=x)
    _lib.add_launches(info.launches)
    return info
