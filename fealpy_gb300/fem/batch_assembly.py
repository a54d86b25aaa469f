"""Assembly of many independent systems with a few launches (no FEALPy
counterpart: FEALPy assembles one ``BilinearForm`` at a time, ``fealpy/fem/
bilinear_form.py:46-105``; the batched configuration has hundreds of meshes).

Systems whose forms have the same structure (element type, degree, factor
channels and tables, source quadrature) form a group.  A group is assembled
as one block-diagonal system: the meshes' nodes, cells and dof maps are
concatenated once (offset by the previous meshes' nodes and dofs), and every
assembly stage runs once for the whole group — the dof adjacency and CSR
pattern, one factor launch, one values launch, the right-hand side gather and
the Dirichlet elimination.  ``fgb_csr_split_blocks`` then rebases the union's
columns and row pointers, so that every system's CSR is a view of the union's
arrays in its own numbering.  Each system's matrix, right-hand side and
Dirichlet rows are those of its own ``BilinearForm.assembly`` +
``LinearForm.assembly`` + ``DirichletBC.apply``, bit for bit: every dof's
contributions are summed over the same cells in the same order.
"""
from typing import List, Sequence, Tuple

import torch

from .. import _lib
from .. import kernels as K
from .. import simplex as sx
from ..sparse import CSRTensor
from .integrators import GroupIntegrator, ScalarSourceIntegrator

__all__ = ["BatchAssembler"]


def _source_spec(lf):
    """(constant source value, quadrature order) of a LinearForm made of one
    ScalarSourceIntegrator with a number as source; None otherwise."""
    ints = []
    for it in lf.integrators.values():
        ints.extend(it.ints if isinstance(it, GroupIntegrator) else [it])
    if len(ints) != 1 or not isinstance(ints[0], ScalarSourceIntegrator):
        return None
    src = ints[0]
    if not isinstance(src.source, (int, float)) or src._region is not None:
        return None
    q = lf.space.p + 3 if src.q is None else src.q
    return float(src.source), int(q)


class _Group:
    def __init__(self, key, members):
        self.key = key
        self.members = members  # indices into the system list


class BatchAssembler:
    """``BatchAssembler([(bform, lform, bc), ...])`` then ``assemble(dtype)`` ->
    ``[(A, F), ...]`` in the order given: the Dirichlet-eliminated matrix and
    right-hand side of every system.

    Requirements for the grouped path: scalar Lagrange forms over whole
    meshes (no sub-region), a right-hand side of one ScalarSourceIntegrator
    with a constant source, and homogeneous Dirichlet data (``gd`` 0 or
    None).  Systems outside these fall back to their own forms' assembly."""

    def __init__(self, systems: Sequence[Tuple[object, object, object]]):
        self.systems = list(systems)
        self.device = None
        self.groups: List[_Group] = []
        self.fallback: List[int] = []
        keyed = {}
        for k, (bf, lf, bc) in enumerate(self.systems):
            space = bf.space
            mesh = space.mesh
            self.device = mesh.node.device if self.device is None else self.device
            spec = _source_spec(lf)
            plan = bf._plan()
            gd_zero = bc.gd is None or (isinstance(bc.gd, (int, float)) and float(bc.gd) == 0.0)
            if spec is None or not gd_zero or plan.cells is not None or not hasattr(plan, "tables"):
                self.fallback.append(k)
                continue
            sig = (type(mesh).__name__, mesh.TD, space.p, tuple((c[0], c[1] >= 0, c[2]) for c in plan.channels),
                   plan.tables.tobytes(), spec[1])
            keyed.setdefault(sig, []).append(k)
        for sig, members in keyed.items():
            self.groups.append(self._build_group(sig, members))

    def _build_group(self, sig, members) -> _Group:
        g = _Group(sig, members)
        dev = self.device
        nodes, cells, c2ds, bds, row_off = [], [], [], [], [0]
        node_off = 0
        for k in members:
            bf, lf, bc = self.systems[k]
            space = bf.space
            mesh = space.mesh
            nodes.append(mesh.node)
            cells.append(mesh.cell + node_off)
            c2ds.append(space.cell_to_dof() + row_off[-1])
            bds.append(bc.is_boundary_dof.to(torch.uint8))
            node_off += mesh.node.shape[0]
            row_off.append(row_off[-1] + space.number_of_global_dofs())
        mesh0 = self.systems[members[0]][0].space.mesh
        g.mesh = type(mesh0)(torch.cat(nodes), torch.cat(cells).to(torch.int32))
        g.c2d = torch.cat(c2ds).to(torch.int32).contiguous()
        g.is_bd = torch.cat(bds).contiguous()
        g.row_off_host = row_off
        g.row_off = torch.as_tensor(row_off, dtype=torch.int64, device=dev)
        g.n = row_off[-1]
        # right-hand side table: sum_q w_q phi_i of the source's rule
        space0 = self.systems[members[0]][0].space
        q = sig[-1]
        bcs, ws = mesh0.quadrature_formula(q).get_quadrature_points_and_weights()
        wphi = ws[:, None] * sx.shape_function(bcs, space0.p)
        g.wphi = torch.as_tensor(wphi, dtype=torch.float64, device=dev).contiguous()
        g.sv = torch.as_tensor(wphi.sum(axis=0), dtype=torch.float64, device=dev)
        g.ldof = space0.number_of_local_dofs()
        g.cell_count = [self.systems[k][0].space.mesh.number_of_cells() for k in members]
        return g

    def assemble(self, dtype=torch.float64) -> List[Tuple[CSRTensor, torch.Tensor]]:
        out = [None] * len(self.systems)
        for g in self.groups:
            for k, AF in zip(g.members, self._assemble_group(g, dtype)):
                out[k] = AF
        for k in self.fallback:
            bf, lf, bc = self.systems[k]
            out[k] = bc.apply(bf.assembly(dtype=dtype), lf.assembly())
        return out

    def _assemble_group(self, g: _Group, dtype):
        dev = self.device
        status = _lib.status_word(dev)
        plans = [self.systems[k][0]._plan() for k in g.members]
        srcs = [_source_spec(self.systems[k][1])[0] for k in g.members]
        p0 = plans[0]
        # coefficient rows of the union: each plan's rows concatenated over
        # the members' cells
        n_rows = len(p0.coefs)
        coef = None
        if n_rows:
            rows = []
            for r in range(n_rows):
                parts = []
                for pl, nc in zip(plans, g.cell_count):
                    parts.append(pl.coefs[r].to(device=dev, dtype=torch.float64).reshape(-1)[:nc])
                rows.append(torch.cat(parts))
            coef = torch.stack(rows, 0)
        # one more channel: the signed measure (right-hand side)
        chans = list(p0.channels) + [(_lib.FGB_CH_MEASURE, -1, 1.0)]
        adj_ptr, adj, _ = K.build_adjacency(g.c2d, g.n, status)
        indptr, indices = K.build_pattern(adj_ptr, adj, g.c2d, g.n, status)
        values = None
        passes = [(chans[a:a + _lib.FGB_MAX_CHANNELS], None) for a in range(0, len(chans), _lib.FGB_MAX_CHANNELS)]
        tabs_all = p0.tables
        fac_all = []
        for chs, _ in passes:
            fac_all.append(K.cell_factors(g.mesh, chs, coef, torch.float64, status))
        fac64 = torch.cat(fac_all, 1) if len(fac_all) > 1 else fac_all[0]
        cm = fac64[:, -1]
        fac_mat = fac64[:, :-1].to(dtype).contiguous()
        nt = fac_mat.shape[1]
        for a in range(0, nt, _lib.FGB_MAX_CHANNELS):
            tab = torch.as_tensor(tabs_all[a:a + _lib.FGB_MAX_CHANNELS], dtype=dtype, device=dev)
            values, _ = K.assemble_scalar(adj_ptr, adj, g.c2d, tab, fac_mat[:, a:a + _lib.FGB_MAX_CHANNELS].contiguous(),
                                          indptr, indices, status=status, accumulate_into=values)
        # right-hand side: |T| (sum_q w_q phi_i) f per (cell, local dof),
        # formed and summed per dof as the single-system LinearForm does (the
        # source of every member as a per-cell value: the same products)
        fcell = torch.repeat_interleave(torch.as_tensor(srcs, dtype=torch.float64, device=dev),
                                        torch.as_tensor(g.cell_count, device=dev))
        F = K.source_gather(adj_ptr, adj, g.ldof, cm.contiguous(), 1, 0.0, fcell, g.wphi, g.sv)
        _lib.check_status_word("batched assembly", status)
        # homogeneous boundary data: no u_h (the elimination skips A u_h)
        bptr, bidx, bval, bF = K.dirichlet_apply(indptr, indices, values, g.is_bd, F.to(values.dtype), None)
        # split into the systems' own CSRs
        nsys = len(g.members)
        iptr_out = torch.empty(g.n + nsys, dtype=torch.int64, device=dev)
        st2 = _lib.status_word(dev)
        _lib.call("fgb_csr_split_blocks", nsys, _lib.ptr(g.row_off), _lib.ptr(bptr), _lib.ptr(bidx),
                  _lib.ptr(iptr_out), g.n, _lib.ptr(st2), _lib.stream_ptr(dev))
        starts = bptr[g.row_off].cpu().tolist()  # entry range of every system (one host read)
        _lib.check_status_word("batched assembly split", st2)
        res = []
        ro = g.row_off_host
        for s, k in enumerate(g.members):
            n = ro[s + 1] - ro[s]
            A = CSRTensor(iptr_out[ro[s] + s: ro[s + 1] + s + 1], bidx[starts[s]:starts[s + 1]],
                          bval[starts[s]:starts[s + 1]], (n, n))
            A.dof_blocks = self.systems[k][0].space.dof_blocks()
            res.append((A, bF[ro[s]:ro[s + 1]]))
        return res
