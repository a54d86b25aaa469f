"""``BilinearForm`` / ``LinearForm`` with FEALPy's interface
(``fealpy/fem/form.py``, ``bilinear_form.py``, ``linear_form.py``).

``BilinearForm.assembly`` runs the symbolic phase (dof adjacency + canonical
CSR pattern) and the numeric phase (factor kernel + row-gather assembly) on the
GPU and returns a :class:`~fealpy_gb300.sparse.CSRTensor` whose pattern equals
FEALPy's coalesced CSR and whose values match it to rounding.
"""
from typing import Optional, Sequence

import torch

from ..sparse import CSRTensor
from .. import _lib
from .. import kernels as K
from .integrators import (ElasticityPlan, GroupIntegrator, Integrator, ScalarPlan, ScalarSourceIntegrator,
                          _same_cells)

__all__ = ["BilinearForm", "LinearForm", "symbolic_structure"]


def _mark(marks, label):
    """Record a CUDA event labelled `label` into `marks` (timing instrumentation)."""
    if marks is not None:
        e = torch.cuda.Event(enable_timing=True)
        e.record()
        marks.append((label, e))


def symbolic_structure(c2d: torch.Tensor, n_dof: int, status: Optional[torch.Tensor] = None, marks=None,
                       positions: bool = False):
    """(adj_ptr, adj, indptr, indices) for a cell-to-dof map; with
    ``positions`` a fifth entry, the within-row slot map that lets the numeric
    assembly skip the column search."""
    st = _lib.status_word(c2d.device) if status is None else status
    adj_ptr, adj, _ = K.build_adjacency(c2d, n_dof, st)
    _mark(marks, "adjacency")
    if positions:
        indptr, indices, pos = K.build_pattern(adj_ptr, adj, c2d, n_dof, st, positions=True)
        _mark(marks, "pattern")
        return adj_ptr, adj, indptr, indices, pos
    indptr, indices = K.build_pattern(adj_ptr, adj, c2d, n_dof, st)
    _mark(marks, "pattern")
    return adj_ptr, adj, indptr, indices


class _Form:
    def __init__(self, *space, batch_size: int = 0):
        if len(space) == 0:
            raise ValueError("No space is given.")
        if isinstance(space[0], Sequence):
            space = tuple(space[0])
        if len(space) != 1:
            raise NotImplementedError("forms over two different spaces are not provided")
        if batch_size < 0:
            raise ValueError("batch_size must be non-negative")
        self._spaces = space
        self.integrators = {}
        self.splitters = {}
        self._cursor = 0
        self.batch_size = batch_size

    @property
    def space(self):
        return self._spaces[0]

    def __len__(self):
        return len(self.integrators)

    def add_integrator(self, *I, region=None, splitter=None, group=None):
        if len(I) == 0:
            return self
        if len(I) == 1 and isinstance(I[0], (list, tuple)):
            I = tuple(I[0])
        if len(I) == 1:
            I = I[0]
            if region is not None:
                I.set_region(region)
        else:
            I = GroupIntegrator(*I, region=region)
        self._mf_cache = None  # matrix-free data belongs to the former integrators
        group = f"_group_{self._cursor}" if group is None else group
        self._cursor += 1
        if group in self.integrators:
            self.integrators[group] = self.integrators[group] + I
        else:
            self.integrators[group] = I
        # cell chunking (UniformSplitter) has no effect on a row-gather assembly
        self.splitters[group] = splitter
        return self

    def __lshift__(self, other):
        if isinstance(other, Integrator):
            return self.add_integrator(other)
        return NotImplemented


class BilinearForm(_Form):
    _M = None

    def __init__(self, *space, batch_size: int = 0, reuse_pattern: bool = False):
        super().__init__(*space, batch_size=batch_size)
        self.reuse_pattern = reuse_pattern
        s = self.space
        n = s.number_of_global_dofs()
        self.sparse_shape = (n, n)

    @property
    def shape(self):
        return ((self.batch_size,) if self.batch_size > 0 else ()) + tuple(self.sparse_shape)

    def _members(self):
        """Unbatched forms of the batch members (kept for repeated matrix-free
        products; rebuilt when integrators are added)."""
        cached = getattr(self, "_member_forms", None)
        key = tuple((g, id(it)) for g, it in self.integrators.items())
        if cached is None or cached[0] != key:
            forms = []
            for b in range(self.batch_size):
                f = BilinearForm(self.space)
                for g, it in self.integrators.items():
                    f.integrators[g] = it.batch_member(self.space, b)
                forms.append(f)
            cached = (key, forms)
            self._member_forms = cached
        return cached[1]

    def _plan(self):
        """The merged plan of the form's integrators; scalar integrators over
        different cells (a region per integrator group,
        ``fealpy/fem/integrator.py:141-162``) give a list of plans, one per
        distinct cell set."""
        plans = [it.plan(self.space) for it in self.integrators.values()]
        if not plans:
            raise RuntimeError("no integrator added to the form")
        if not all(isinstance(p, ScalarPlan) for p in plans):
            if len(plans) > 1:
                raise NotImplementedError("only several scalar integrators can share one form")
            return plans[0]
        merged = []
        for p in plans:
            for k, m in enumerate(merged):
                if _same_cells(m.cells, p.cells):
                    merged[k] = m + p
                    break
            else:
                merged.append(p)
        return merged[0] if len(merged) == 1 else merged

    def _symbolic(self, space, c2d, n, marks=None, sub: bool = False, positions: bool = False):
        key = ("symbolic", n, positions)
        cache = getattr(space, "_cache", {})
        if self.reuse_pattern and not sub and key in cache:
            return cache[key]
        out = symbolic_structure(c2d, n, marks=marks, positions=positions)
        if self.reuse_pattern and not sub:
            cache[key] = out
        if not sub and hasattr(space, "_cache"):
            # the dof adjacency depends on the dof map alone: the right-hand
            # side of the same space gathers over it (LinearForm._adjacency)
            space._cache[("adjacency", n)] = (out[0], out[1])
        return out

    def assembly(self, *, format="csr", dtype=torch.float64, emit_f32: bool = False, marks=None):
        """Assemble the global matrix, a CSRTensor (``format="csr"``) or its
        coalesced COOTensor (``format="coo"``; FEALPy
        ``fealpy/fem/bilinear_form.py:83-104``: the kernels emit CSR, the COO
        form is its row expansion).  ``dtype`` float64 (default) or float32
        selects the arithmetic of the factor and assembly kernels;
        ``emit_f32`` also stores a float copy of float64 values on the result
        (used by the mixed-precision solver).  ``marks`` (a list) receives
        labelled CUDA events after each sub-stage (instrumentation)."""
        if format not in ("csr", "coo"):
            raise ValueError(f"Unsupported format {format}.")
        if self.batch_size > 0:
            return self._batched_assembly(format, dtype)
        space = self.space
        plan = self._plan()
        status = _lib.status_word(space.device)
        _mark(marks, "start")
        if isinstance(plan, list):
            # several cell sets: the pattern of their union, then each set's
            # values added into it (its own adjacency, column search)
            full = space.cell_to_dof()
            c2ds = [full if p.cells is None else full[p.cells].contiguous() for p in plan]
            n = space.number_of_global_dofs()
            adj_ptr, adj, indptr, indices = symbolic_structure(torch.cat(c2ds).contiguous(), n, marks=marks)
            mesh = space.mesh
            values = v32 = None
            for g, (p, c2d) in enumerate(zip(plan, c2ds)):
                st = _lib.status_word(space.device)
                g_ptr, g_adj, _ = K.build_adjacency(c2d, n, st)
                _lib.check_status_word("adjacency", st)
                coef = p.coef_matrix()
                passes = p.passes()
                for chans, tabs in passes:
                    fac = K.cell_factors(mesh, chans, coef, dtype, status, cells=p.cells)
                    tab = torch.as_tensor(tabs, dtype=dtype, device=space.device)
                    values, _ = K.assemble_scalar(g_ptr, g_adj, c2d, tab, fac, indptr, indices,
                                                  status=status, accumulate_into=values)
            # the float copy of the totals (a cell set's pass covers its own rows only)
            if emit_f32 and dtype == torch.float64:
                v32 = values.to(torch.float32)
            _mark(marks, "values")
        elif isinstance(plan, ScalarPlan):
            c2d = space.cell_to_dof()
            sub = plan.cells is not None
            if sub:
                # integration over a sub-region: the pattern of its cells only
                # (FEALPy scatters the region's local matrices alone)
                c2d = c2d[plan.cells].contiguous()
            n = space.number_of_global_dofs()
            # a reused pattern also keeps the slot of every contribution in
            # its row (the numeric pass then skips the column search)
            sym = self._symbolic(space, c2d, n, marks, sub, positions=self.reuse_pattern and not sub)
            adj_ptr, adj, indptr, indices = sym[:4]
            pos = sym[4] if len(sym) > 4 else None
            mesh = space.mesh
            coef = plan.coef_matrix()
            passes = plan.passes()
            values = v32 = None
            for k, (chans, tabs) in enumerate(passes):
                # more channels than one factor launch holds (coefficients per
                # quadrature point): passes that add into the values
                fac = K.cell_factors(mesh, chans, coef, dtype, status, cells=plan.cells)
                if k == 0:
                    _mark(marks, "factors")
                tab = torch.as_tensor(tabs, dtype=dtype, device=space.device)
                last = k == len(passes) - 1
                values, v32 = K.assemble_scalar(adj_ptr, adj, c2d, tab, fac, indptr, indices,
                                                values_f32=emit_f32 and dtype == torch.float64 and last,
                                                status=status, accumulate_into=values, positions=pos)
            _mark(marks, "values")
        elif isinstance(plan, ElasticityPlan):
            ss = space.scalar_space
            mesh = ss.mesh
            cell = mesh.cell if plan.cells is None else mesh.cell[plan.cells].contiguous()
            NN = mesh.number_of_nodes()
            adj_ptr, adj, nptr, nidx = self._symbolic(ss, cell, NN, marks, plan.cells is not None)
            # the kernel writes the interleaved layout (3 node + component)
            indptr, indices = K.expand_blocks(NN, plan.gd, False, nptr, nidx)
            n = space.number_of_global_dofs()
            fac = K.cell_factors(mesh, plan.channels, plan.coef_matrix(), dtype, status, cells=plan.cells)
            _mark(marks, "factors")
            values, v32 = K.assemble_elasticity_p1(plan.gd, adj_ptr, adj, cell, fac, nptr, nidx, indptr,
                                                   indices.numel(), values_f32=emit_f32 and dtype == torch.float64,
                                                   status=status)
            if space.dof_priority:
                # component-major layout (shape=(GD, -1)): row comp NN + node
                # is the interleaved row GD node + comp; the permutation keeps
                # every entry's value (the same sum) and sorts the columns
                gd = plan.gd
                k = torch.arange(n, device=space.device, dtype=torch.int64)
                order = (k % NN) * gd + k // NN
                inv = torch.empty_like(order)
                inv[order] = k
                _lib.check_status_word("assembly", status)
                indptr, indices, values = K.csr_permute(indptr, indices, values, order, inv)
                if v32 is not None:
                    v32 = values.to(torch.float32)
            _mark(marks, "values")
        else:
            raise NotImplementedError
        _lib.check_status_word("assembly", status)
        M = CSRTensor(indptr, indices, values, (n, n))
        M.dof_blocks = space.dof_blocks()
        # three interleaved components: the nonzeros come in runs of three
        # consecutive columns (node triples)
        if getattr(space, "dof_priority", True) is False and getattr(space, "dof_numel", 1) == 3:
            M.node_block = 3
        if v32 is not None:
            M._f32 = v32
        self._M = M
        return M.tocoo() if format == "coo" else M

    def _batched_assembly(self, format, dtype):
        """A form with ``batch_size`` B (``fealpy/fem/bilinear_form.py:46-75``):
        integrators with batched coefficients contribute member b's matrix to
        batch member b, the others the same matrix to every member.  One
        pattern for all members (with its slot map), one factor and one values
        pass per member; the result holds values (B, nnz)."""
        space = self.space
        B = self.batch_size
        for it in self.integrators.values():
            nb = it.batch_size(space)
            if nb not in (0, B):
                raise ValueError(f"an integrator has {nb} batch members, the form {B}")
        vals = []
        for b in range(B):
            member = BilinearForm(space, reuse_pattern=True)
            for g, it in self.integrators.items():
                member.integrators[g] = it.batch_member(space, b)
            Mb = member.assembly(dtype=dtype)
            if vals and not (Mb.crow is M0.crow and Mb.col is M0.col):
                raise RuntimeError("batch members assembled on different patterns")
            if not vals:
                M0 = Mb
            vals.append(Mb.values)
        M = CSRTensor(M0.crow, M0.col, torch.stack(vals), M0.shape)
        M.dof_blocks = M0.dof_blocks
        M.node_block = M0.node_block
        self._M = M
        return M.tocoo() if format == "coo" else M

    def __matmul__(self, u):
        """``A @ u``; without an assembled matrix the product is formed matrix
        free, as FEALPy does (``fealpy/fem/bilinear_form.py:126-158``): a
        kernel forms every cell's K_c u_c from the cell factors and the
        tables, and the dof adjacency adds them per dof in cell order.  No
        global matrix is built (``_M`` stays None).  ``u`` may carry a batch
        on the first dimension."""
        if self._M is not None:
            return self._M @ u
        if not isinstance(u, torch.Tensor):
            raise TypeError("u must be a torch tensor")
        if self.batch_size > 0:
            # batched coefficients: (B, n) out, u (n,) or one vector per member (B, n)
            members = self._members()
            if u.ndim == 1:
                return torch.stack([f._matfree(u) for f in members])
            if u.ndim == 2 and u.shape[0] == self.batch_size:
                return torch.stack([f._matfree(v) for f, v in zip(members, u)])
            raise ValueError(f"a batched form multiplies (n,) or ({self.batch_size}, n) vectors")
        if u.ndim >= 2:
            return torch.stack([self._matfree(v) for v in u.reshape(-1, u.shape[-1])]).reshape(
                u.shape[:-1] + (self.shape[0],))
        return self._matfree(u)

    def _region_forms(self):
        """One form per distinct cell set of the integrator groups (kept for
        repeated matrix-free products)."""
        key = tuple((g, id(it)) for g, it in self.integrators.items())
        cached = getattr(self, "_region_cache", None)
        if cached is None or cached[0] != key:
            forms = []
            for g, it in self.integrators.items():
                cells = it.plan(self.space).cells
                for f, c in forms:
                    if _same_cells(c, cells):
                        f.integrators[g] = it
                        break
                else:
                    f = BilinearForm(self.space)
                    f.integrators[g] = it
                    forms.append((f, cells))
            cached = (key, [f for f, _ in forms])
            self._region_cache = cached
        return cached[1]

    def _matfree(self, u):
        plan = self._plan()
        if isinstance(plan, list):
            # integrator groups over different cells: the sum of their products
            out = None
            for f in self._region_forms():
                y = f._matfree(u)
                out = y if out is None else out + y
            return out
        if not isinstance(plan, ScalarPlan):
            raise NotImplementedError("matrix-free products are provided for scalar integrators")
        space = self.space
        dtype = u.dtype if u.dtype in (torch.float32, torch.float64) else torch.float64
        key = ("matfree", dtype)
        cache = getattr(self, "_mf_cache", None)
        if cache is None or cache[0] != key:
            status = _lib.status_word(space.device)
            coef = plan.coef_matrix()
            fac = [(K.cell_factors(space.mesh, chans, coef, dtype, status, cells=plan.cells), tabs)
                   for chans, tabs in plan.passes()]
            _lib.check_status_word("matrix-free factors", status)
            n = space.number_of_global_dofs()
            c2d = space.cell_to_dof() if plan.cells is None else space.cell_to_dof()[plan.cells].contiguous()
            akey = ("adjacency", n)
            if plan.cells is not None:
                st = _lib.status_word(space.device)
                adj_ptr, adj, _ = K.build_adjacency(c2d, n, st)
                _lib.check_status_word("adjacency", st)
                adjacency = (adj_ptr, adj)
            else:
                if akey not in space._cache:
                    st = _lib.status_word(space.device)
                    adj_ptr, adj, _ = K.build_adjacency(c2d, n, st)
                    _lib.check_status_word("adjacency", st)
                    space._cache[akey] = (adj_ptr, adj)
                adjacency = space._cache[akey]
            cache = (key, fac, c2d, adjacency)
            self._mf_cache = cache
        _, fac, c2d, (adj_ptr, adj) = cache
        ud = u.to(device=space.device, dtype=dtype)
        yc = None
        for f, tables in fac:
            y = K.cell_apply(c2d, tables, f, ud)
            yc = y if yc is None else yc + y
        return K.gather_sum(adj_ptr, adj, yc)

    def mult(self, x, out=None):
        y = self @ x
        if out is not None:
            out.copy_(y)
            return out
        return y


class LinearForm(_Form):
    """Right-hand-side vector: scalar sources formed and summed per dof in one
    kernel (``fgb_source_gather``); other integrators' cell vectors summed
    into dofs by the deterministic adjacency gather."""

    def __init__(self, *space, batch_size: int = 0):
        super().__init__(*space, batch_size=batch_size)
        self._V = None

    def assembly(self, *, format="dense") -> torch.Tensor:
        if self.batch_size > 0:
            # batched sources (fealpy/fem/linear_form.py:36-60): one vector per
            # member, (B, n); unbatched integrators repeat over the batch
            space = self.space
            out = []
            for b in range(self.batch_size):
                member = LinearForm(space)
                for g, it in self.integrators.items():
                    nb = it.batch_size(space)
                    if nb not in (0, self.batch_size):
                        raise ValueError(f"an integrator has {nb} batch members, the form {self.batch_size}")
                    member.integrators[g] = it.batch_member(space, b)
                out.append(member.assembly(format=format))
            self._V = torch.stack(out)
            return self._V
        space = self.space
        mesh = space.scalar_space.mesh if hasattr(space, "scalar_space") else space.mesh
        n = space.number_of_global_dofs()
        out = None
        # scalar sources: formed and gathered per dof in one kernel each
        # (fgb_source_gather), no cell-vector array
        rest = []
        for it in self.integrators.values():
            ints = it.ints if isinstance(it, GroupIntegrator) else [it]
            for i in ints:
                if isinstance(i, ScalarSourceIntegrator) and not hasattr(space, "scalar_space"):
                    cells, cm, mode, fs, f, wphi, sv = i.source_data(space)
                    adj_ptr, adj = self._adjacency(space, cells)
                    out = K.source_gather(adj_ptr, adj, space.number_of_local_dofs(), cm, mode, fs, f, wphi, sv,
                                          out=out)
                else:
                    rest.append(i)
        # other integrators: cell vectors grouped by the cells they integrate
        # over (all cells, or a sub-region), one dof gather per group
        groups = []
        for i in rest:
            v = i.assembly(space)
            cells = i.cell_selection(mesh)
            for g in groups:
                if (g[0] is None and cells is None) or (g[0] is not None and cells is not None and
                                                       g[0].shape == cells.shape and torch.equal(g[0], cells)):
                    g[1] = g[1] + v
                    break
            else:
                groups.append([cells, v])
        if not groups and out is None:
            raise RuntimeError("no integrator added to the form")
        for cells, local in groups:
            adj_ptr, adj = self._adjacency(space, cells)
            vec = K.gather_sum(adj_ptr, adj, local.to(torch.float64).contiguous())
            out = vec if out is None else out + vec
        self._V = out
        return self._V

    @staticmethod
    def _adjacency(space, cells):
        """dof -> (cell, local) adjacency of all cells (cached on the space)
        or of a sub-region."""
        n = space.number_of_global_dofs()
        if cells is None:
            key = ("adjacency", n)
            cache = space._cache
            if key not in cache:
                st = _lib.status_word(space.device)
                adj_ptr, adj, _ = K.build_adjacency(space.cell_to_dof(), n, st)
                _lib.check_status_word("adjacency", st)
                cache[key] = (adj_ptr, adj)
            return cache[key]
        st = _lib.status_word(space.device)
        adj_ptr, adj, _ = K.build_adjacency(space.cell_to_dof()[cells].contiguous(), n, st)
        _lib.check_status_word("adjacency", st)
        return adj_ptr, adj
