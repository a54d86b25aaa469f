"""Integrators with FEALPy's interface (``fealpy/fem/integrator.py``,
``scalar_diffusion_integrator.py``, ``scalar_mass_integrator.py``,
``linear_elasticity_integrator.py``, ``scalar_source_integrator.py``).

An operator integrator here does not build local matrices on the assembly
path.  It describes its local matrix as ``sum_t factor_t(cell) * table_t`` (a
*plan*): the factors are per-cell geometric quantities computed by the
``fgb_cell_factors`` kernel (signed measure, Jacobian-inverse metric, times the
coefficient) and the tables are mesh-independent contractions of the basis
gradients with the integrator's own quadrature rule.  ``BilinearForm`` merges
the plans of all integrators on a space into a single factor launch and a
single CSR assembly launch.  ``assembly(space)`` still returns the
(NC, ldof, ldof) local matrices for callers that want them.
"""
from typing import List, Optional, Tuple

import numpy as np
import torch

from .. import _lib
from .. import simplex as sx
from ..functionspace import TensorFunctionSpace
from .. import kernels as K

__all__ = ["Integrator", "GroupIntegrator", "ScalarDiffusionIntegrator", "ScalarMassIntegrator",
           "LinearElasticityIntegrator", "ScalarSourceIntegrator", "VectorSourceIntegrator", "ScalarPlan",
           "ElasticityPlan"]

_S = slice(None)


def _is_full(index) -> bool:
    return index is None or (isinstance(index, slice) and index == slice(None))


class ScalarPlan:
    """Local matrix = sum_t factor_t(c) * tables[t]; channel t = (kind, coef_row, scale)."""

    def __init__(self, channels: List[Tuple[int, int, float]], coefs: List[torch.Tensor], tables: np.ndarray,
                 cells: Optional[torch.Tensor] = None):
        self.channels = channels
        self.coefs = coefs
        self.tables = tables
        self.cells = cells  # sub-region (int64 cell indices) or None

    def __add__(self, other: "ScalarPlan") -> "ScalarPlan":
        if not _same_cells(self.cells, other.cells):
            raise NotImplementedError("integrators of one form integrate over the same cells on the GB300 path")
        off = len(self.coefs)
        ch = list(self.channels) + [(k, (c + off) if c >= 0 else -1, s) for k, c, s in other.channels]
        return ScalarPlan(ch, self.coefs + other.coefs, np.concatenate([self.tables, other.tables], axis=0),
                          self.cells)

    def coef_matrix(self):
        return torch.stack(self.coefs, 0) if self.coefs else None

    def passes(self, limit: int = _lib.FGB_MAX_CHANNELS):
        """The channels in passes of at most ``limit`` (the factor kernel's
        capacity): [(channels, tables)]; coefficient rows keep indexing
        :meth:`coef_matrix`."""
        n = len(self.channels)
        return [(self.channels[a:a + limit], self.tables[a:a + limit]) for a in range(0, n, limit)]


def _same_cells(a: Optional[torch.Tensor], b: Optional[torch.Tensor]) -> bool:
    if a is None or b is None:
        return a is None and b is None
    return a is b or (a.shape == b.shape and bool(torch.equal(a, b)))


class ElasticityPlan:
    """P1 elasticity: factor channels = grad(lambda_{1..GD}) then |T| D00, |T| D_lambda, |T| D_mu."""

    def __init__(self, gd: int, channels, coefs, cells: Optional[torch.Tensor] = None):
        self.gd = gd
        self.channels = channels
        self.coefs = coefs
        self.cells = cells

    def coef_matrix(self):
        return torch.stack(self.coefs, 0) if self.coefs else None


def _cell_coefficient(coef, space, q: int, cells: Optional[torch.Tensor] = None
                      ) -> Tuple[float, Optional[torch.Tensor], Optional[torch.Tensor]]:
    """(scale, per-cell array or None, per-point array or None) from a FEALPy
    CoefLike (``fealpy/utils/utils.py:21-53``): a number, an (NC,) array, an
    (NC, NQ) array of values at the quadrature points of rule ``q``, or a
    callable evaluated there.  Values that agree across each cell's points
    become a per-cell array; otherwise the (NC, NQ) array is returned.  With
    ``cells`` (a sub-region) NC counts the selected cells and callables are
    evaluated on them."""
    mesh = space.mesh
    NC = mesh.number_of_cells() if cells is None else int(cells.numel())
    if coef is None:
        return 1.0, None, None
    if isinstance(coef, (int, float)):
        return float(coef), None, None
    if isinstance(coef, torch.Tensor):
        if coef.numel() == 1:
            return float(coef.reshape(-1)[0].item()), None, None
        if coef.ndim == 1 and coef.shape[0] == NC:
            return 1.0, coef.to(device=mesh.device, dtype=torch.float64), None
        if coef.ndim == 2 and coef.shape[0] == NC:
            val = coef.to(device=mesh.device, dtype=torch.float64)
            NQ = mesh.quadrature_formula(q).number_of_quadrature_points()
            if val.shape[1] == NQ and not bool(torch.all(val == val[:, :1])):
                return 1.0, None, val.contiguous()
            if bool(torch.all(val == val[:, :1])):
                return 1.0, val[:, 0].contiguous(), None
            raise ValueError(f"an (NC, NQ) coefficient needs NQ = {NQ} values per cell for quadrature order {q}")
        raise ValueError("coefficients are a number, (NC,) or (NC, NQ)")
    if isinstance(coef, np.ndarray):
        return _cell_coefficient(torch.as_tensor(coef, device=mesh.device), space, q, cells)
    if callable(coef):
        bcs, _ = mesh.quadrature_formula(q).get_quadrature_points_and_weights()
        index = _S if cells is None else cells
        if getattr(coef, "coordtype", "barycentric") == "cartesian":
            val = coef(mesh.bc_to_point(bcs, index=index))
        else:
            val = coef(torch.as_tensor(bcs, device=mesh.device), index=index)
        return _cell_coefficient(torch.as_tensor(val, device=mesh.device), space, q, cells)
    raise TypeError(f"coef should be int, float, TensorLike or callable, but got {type(coef)}")


class Integrator:
    """Base class: region handling, data cache switch and ``+`` grouping."""
    etype = "cell"

    def __init__(self, keep_data: bool = False):
        self._region = None
        self._cache = {}
        self._keep_data = keep_data

    def keep_data(self, status_on=True):
        self._keep_data = status_on
        if not status_on:
            self._cache.clear()
        return self

    def clear(self):
        self._cache.clear()

    def set_region(self, region):
        self._region = region
        self.clear()
        return self

    def get_region(self):
        return self._region

    def _check_region(self):
        """Kept for callers of the former interface: sub-regions are supported."""
        return None

    def cell_selection(self, mesh) -> Optional[torch.Tensor]:
        """The cells integrated over as an int64 index tensor on the mesh's
        device, or None for all cells: ``region`` (index or boolean tensor, or
        a callable of the mesh; ``fealpy/fem/integrator.py:141-162``) or, for
        the integrators that take it, ``index`` (``scalar_mass_integrator.py``,
        ``linear_elasticity_integrator.py``)."""
        sel = self._region
        if sel is None:
            idx = getattr(self, "index", None)
            if _is_full(idx):
                return None
            sel = idx
        if callable(sel) and not isinstance(sel, (torch.Tensor, np.ndarray)):
            sel = sel(mesh)
        NC = mesh.number_of_cells()
        if isinstance(sel, slice):
            return torch.arange(NC, device=mesh.device)[sel]
        t = torch.as_tensor(sel, device=mesh.device)
        if t.dtype == torch.bool:
            if t.numel() != NC:
                raise ValueError("a boolean region has one entry per cell")
            return torch.nonzero(t).reshape(-1)
        t = t.reshape(-1).to(torch.int64)
        if t.numel() and (int(t.min()) < 0 or int(t.max()) >= NC):
            raise IndexError("region cell index out of range")
        return t

    def __add__(self, other):
        if isinstance(other, Integrator):
            return GroupIntegrator(self, other)
        return NotImplemented

    __iadd__ = __add__

    # batched coefficients (``batched=True``: a leading batch axis on the
    # coefficient, ``fealpy/functional.py:68-106``) -----------------------
    def batch_size(self, space) -> int:
        """Batch members of the coefficient (0: not batched)."""
        return 0

    def batch_member(self, space, b: int) -> "Integrator":
        """The integrator of batch member ``b`` (unbatched); an unbatched
        integrator is the same for every member."""
        return self

    def __call__(self, *args, **kwargs):
        return self.assembly(*args, **kwargs)

    def to_global_dof(self, space, /, indices=None):
        c2d = space.cell_to_dof()
        sel = self.cell_selection(space.mesh)
        if sel is not None:
            c2d = c2d[sel]
        return c2d if indices is None else c2d[indices]

    def __repr__(self):
        return self.__class__.__name__


class _OperatorIntegrator(Integrator):
    def plan(self, space):
        raise NotImplementedError

    def assembly(self, space, /, indices=None):
        """Local matrices (NC, ldof, ldof), FP64 (a convenience; the CSR path
        never materialises them); (B, NC, ldof, ldof) with batched
        coefficients."""
        nb = self.batch_size(space)
        if nb:
            return torch.stack([self.batch_member(space, b).assembly(space, indices) for b in range(nb)])
        plan = self.plan(space)
        mesh = space.mesh
        coef = plan.coef_matrix()
        out = None
        for chans, tabs in plan.passes():
            f = K.cell_factors(mesh, chans, coef, torch.float64, cells=plan.cells)
            out = K.local_matrices(f, torch.as_tensor(tabs, dtype=torch.float64, device=mesh.device), out)
        return out if indices is None else out[indices]


class _BatchedCoef:
    """Batched coefficients of a scalar integrator (the attribute named by
    ``_batched_attr``: the coefficient, or a source's values): a number per
    member (B,), a per-cell array (B, NC), values at the quadrature points
    (B, NC, NQ), or a callable returning one of those at the quadrature
    points."""
    _batched_attr = "coef"

    def _batched_values(self, space) -> torch.Tensor:
        coef = getattr(self, self._batched_attr)
        mesh = space.mesh
        if callable(coef) and not isinstance(coef, (torch.Tensor, np.ndarray)):
            key = ("batched_coef", id(space))
            if key not in self._cache:
                q = space.p + 3 if self.q is None else self.q
                bcs, _ = mesh.quadrature_formula(q).get_quadrature_points_and_weights()
                cells = self.cell_selection(mesh)
                index = _S if cells is None else cells
                if getattr(coef, "coordtype", "barycentric") == "cartesian":
                    val = coef(mesh.bc_to_point(bcs, index=index))
                else:
                    val = coef(torch.as_tensor(bcs, device=mesh.device), index=index)
                self._cache[key] = torch.as_tensor(val, device=mesh.device)
            return self._cache[key]
        if isinstance(coef, (torch.Tensor, np.ndarray)):
            return torch.as_tensor(coef, device=mesh.device)
        raise ValueError("a batched coefficient is a tensor (or a callable) with the batch on its first axis")

    def batch_size(self, space) -> int:
        if not self.batched:
            return 0
        val = self._batched_values(space)
        if val.ndim < 1 or val.shape[0] < 1:
            raise ValueError("a batched coefficient has the batch on its first axis")
        return int(val.shape[0])

    def batch_member(self, space, b: int):
        if not self.batched:
            return self
        import copy
        member = copy.copy(self)
        member._cache = {}
        member.batched = False
        setattr(member, self._batched_attr, self._batched_values(space)[b])
        return member


class ScalarDiffusionIntegrator(_BatchedCoef, _OperatorIntegrator):
    """``(coef grad u, grad v)`` on simplex Lagrange spaces."""

    def __init__(self, coef=None, q: Optional[int] = None, *, region=None, batched: bool = False, method=None):
        super().__init__()
        if method not in (None, "fast"):
            raise NotImplementedError(f"assembly variant {method!r} is not provided on the GB300 path")
        self.coef = coef
        self.q = q
        self.batched = batched
        self.set_region(region)

    def plan(self, space) -> ScalarPlan:
        self._check_region()
        if self.batched:
            raise ValueError("a batched integrator is assembled per batch member (a form with batch_size)")
        mesh = space.mesh
        TD = mesh.TD
        q = space.p + 3 if self.q is None else self.q
        cells = self.cell_selection(mesh)
        scale, arr, arrq = _cell_coefficient(self.coef, space, q, cells)
        pairs = sx.metric_pairs(TD)
        if arrq is not None:
            # a coefficient per quadrature point: one channel per (point,
            # metric entry) with that point's table
            coefs = [arrq[:, iq].contiguous() for iq in range(arrq.shape[1])]
            ch = [(_lib.FGB_CH_METRIC + k * 3 + l, iq, 1.0) for iq in range(arrq.shape[1]) for k, l in pairs]
            return ScalarPlan(ch, coefs, sx.diffusion_tables_q(TD, space.p, q), cells)
        coefs = [arr] if arr is not None else []
        ci = 0 if arr is not None else -1
        ch = [(_lib.FGB_CH_METRIC + k * 3 + l, ci, scale) for k, l in pairs]
        return ScalarPlan(ch, coefs, sx.diffusion_tables(TD, space.p, q), cells)


class ScalarMassIntegrator(_BatchedCoef, _OperatorIntegrator):
    """``(coef u, v)`` on simplex Lagrange spaces."""

    def __init__(self, coef=None, q: Optional[int] = None, *, index=_S, batched: bool = False, method=None):
        super().__init__()
        if method is not None:
            raise NotImplementedError(f"assembly variant {method!r} is not provided on the GB300 path")
        self.coef = coef
        self.q = q
        self.batched = batched
        self.index = index

    def plan(self, space) -> ScalarPlan:
        self._check_region()
        if self.batched:
            raise ValueError("a batched integrator is assembled per batch member (a form with batch_size)")
        mesh = space.mesh
        q = space.p + 3 if self.q is None else self.q
        cells = self.cell_selection(mesh)
        scale, arr, arrq = _cell_coefficient(self.coef, space, q, cells)
        if arrq is not None:
            coefs = [arrq[:, iq].contiguous() for iq in range(arrq.shape[1])]
            ch = [(_lib.FGB_CH_MEASURE, iq, 1.0) for iq in range(arrq.shape[1])]
            return ScalarPlan(ch, coefs, sx.mass_tables_q(mesh.TD, space.p, q), cells)
        coefs = [arr] if arr is not None else []
        ch = [(_lib.FGB_CH_MEASURE, 0 if arr is not None else -1, scale)]
        return ScalarPlan(ch, coefs, sx.mass_table(mesh.TD, space.p, q), cells)


class LinearElasticityIntegrator(_OperatorIntegrator):
    """Linear elasticity on a ``TensorFunctionSpace`` of P1 Lagrange functions:
    interleaved components (``shape=(-1, GD)``, ``dof_priority=False``) or
    component-major (``shape=(GD, -1)``; the form permutes the interleaved
    matrix)."""

    def __init__(self, material, q: Optional[int] = None, *, index=_S, method=None):
        super().__init__()
        # FEALPy's 'voigt' (B^T D B, fealpy/fem/linear_elasticity_integrator.py:214-226)
        # and 'fast' (:265-) variants form the default variant's matrix (on P1
        # tetrahedra, both dof orders, they agree with it to 2.3e-15 relative in
        # the reference itself), so they name the same kernel here
        if method not in (None, "assembly", "voigt", "fast"):
            raise NotImplementedError(f"assembly variant {method!r} is not provided on the GB300 path")
        self.material = material
        self.q = q
        self.index = index

    def assembly(self, space, /, indices=None):
        """Local matrices ((NC, (GD+1) GD, (GD+1) GD), FP64) in the space's
        local dof order (interleaved or component-major)."""
        out = K.local_elasticity_p1(space.scalar_space.mesh, self.plan(space, local=True),
                                    priority=bool(space.dof_priority))
        return out if indices is None else out[indices]

    def plan(self, space, local: bool = False) -> ElasticityPlan:
        self._check_region()
        if not isinstance(space, TensorFunctionSpace):
            raise TypeError("LinearElasticityIntegrator needs a TensorFunctionSpace")
        ss = space.scalar_space
        mesh = ss.mesh
        gd = mesh.GD
        if ss.p != 1:
            raise NotImplementedError("the GB300 elasticity kernel covers P1 spaces")
        q = ss.p + 3 if self.q is None else self.q
        _, ws = mesh.quadrature_formula(q).get_quadrature_points_and_weights()
        wsum = float(np.sum(ws))
        D = torch.as_tensor(self.material.elastic_matrix(), dtype=torch.float64, device=mesh.device)
        if D.ndim != 4 or D.shape[1] != 1:
            raise ValueError(f"elastic matrix must be (NC or 1, 1, {2 * gd}, {2 * gd})")
        if gd == 3:
            d01, dmu = D[:, 0, 0, 1], D[:, 0, 5, 5]
            d00 = 2.0 * dmu + d01
        else:
            d00, d01, dmu = D[:, 0, 0, 0], D[:, 0, 0, 1], D[:, 0, 2, 2]
        cells = self.cell_selection(mesh)
        chans = [(_lib.FGB_CH_GRAD + k * 3 + a, -1, 1.0) for k in range(gd) for a in range(gd)]
        coefs = []
        for v in (d00, d01, dmu):
            if v.numel() == 1:
                chans.append((_lib.FGB_CH_MEASURE, -1, float(v.item()) * wsum))
            else:
                if cells is not None and v.numel() == mesh.number_of_cells():
                    v = v[cells]  # per-cell material of the whole mesh, restricted to the region
                chans.append((_lib.FGB_CH_MEASURE, len(coefs), wsum))
                coefs.append(v.contiguous())
        return ElasticityPlan(gd, chans, coefs, cells)


class GroupIntegrator(Integrator):
    """Several integrators sharing one dof map; their local matrices add."""

    def __init__(self, *ints, region=None):
        super().__init__()
        self.ints = []
        if not ints:
            raise ValueError("No integrators provided.")
        for it in ints:
            if isinstance(it, GroupIntegrator):
                self.ints.extend(it.ints)
            elif isinstance(it, Integrator):
                self.ints.append(it)
            else:
                raise TypeError(f"Unsupported type {type(it).__name__} found in the inputs.")
        if region is not None:
            self.set_region(region)

    def __iter__(self):
        return iter(self.ints)

    def __len__(self):
        return len(self.ints)

    def __getitem__(self, i):
        return self.ints[i]

    def __iadd__(self, other):
        if isinstance(other, GroupIntegrator):
            self.ints.extend(other.ints)
        elif isinstance(other, Integrator):
            self.ints.append(other)
        else:
            return NotImplemented
        return self

    def set_region(self, region):
        for it in self.ints:
            it.set_region(region)
        return super().set_region(region)

    def to_global_dof(self, space, /, indices=None):
        return self.ints[0].to_global_dof(space, indices)

    def batch_size(self, space) -> int:
        sizes = {it.batch_size(space) for it in self.ints} - {0}
        if len(sizes) > 1:
            raise ValueError(f"grouped integrators have different batch sizes {sorted(sizes)}")
        return sizes.pop() if sizes else 0

    def batch_member(self, space, b: int):
        if not self.batch_size(space):
            return self
        return GroupIntegrator(*[it.batch_member(space, b) for it in self.ints])

    def plan(self, space):
        plans = [it.plan(space) for it in self.ints]
        out = plans[0]
        for p in plans[1:]:
            if not (isinstance(out, ScalarPlan) and isinstance(p, ScalarPlan)):
                raise NotImplementedError("only scalar integrators can be grouped")
            out = out + p
        return out

    def assembly(self, space, /, indices=None):
        nb = self.batch_size(space)
        if nb:
            return torch.stack([self.batch_member(space, b).assembly(space, indices) for b in range(nb)])
        out = self.ints[0].assembly(space, indices)
        for it in self.ints[1:]:
            out = out + it.assembly(space, indices)
        return out


# ---------------------------------------------------------------------------
# source integrators (right-hand sides)
# ---------------------------------------------------------------------------
def _source_values(source, mesh, bcs, index=_S):
    """Source values at quadrature points: (NC, NQ) or broadcastable (NC: the
    cells of ``index``)."""
    if isinstance(source, (int, float)):
        return float(source)
    if isinstance(source, torch.Tensor):
        return source.to(device=mesh.device, dtype=torch.float64)
    if callable(source):
        if getattr(source, "coordtype", "barycentric") == "cartesian":
            return torch.as_tensor(source(mesh.bc_to_point(bcs, index=index)), dtype=torch.float64,
                                   device=mesh.device)
        return torch.as_tensor(source(torch.as_tensor(bcs, device=mesh.device), index=index), dtype=torch.float64,
                               device=mesh.device)
    raise TypeError(f"source should be int, float, TensorLike or callable, but got {type(source)}")


class ScalarSourceIntegrator(_BatchedCoef, Integrator):
    """``(f, v)`` (``fealpy/fem/scalar_source_integrator.py:13-90``); with
    ``batched=True`` the source has a leading batch axis (a form with
    ``batch_size``)."""
    _batched_attr = "source"

    def __init__(self, source=None, q: Optional[int] = None, *, region=None, batched: bool = False, method=None):
        super().__init__()
        self.source = source
        self.q = q
        self.batched = batched
        self.set_region(region)

    def source_data(self, space):
        """(cells or None, signed measures, mode, number, values, w phi table,
        its column sums) of this source for ``fgb_source_local/gather``:
        mode 0 a number, 1 one value per cell, 2 one per quadrature point."""
        if self.batched:
            raise ValueError("a batched source is assembled per batch member (a form with batch_size)")
        mesh = space.mesh
        q = space.p + 3 if self.q is None else self.q
        bcs, ws = mesh.quadrature_formula(q).get_quadrature_points_and_weights()
        cells = self.cell_selection(mesh)
        index = _S if cells is None else cells
        cm = mesh.entity_measure("cell", index=index)
        wphi_np = ws[:, None] * sx.shape_function(bcs, space.p)                       # (NQ, ldof)
        wphi = torch.as_tensor(wphi_np, dtype=torch.float64, device=mesh.device).contiguous()
        sv = torch.as_tensor(wphi_np.sum(axis=0), dtype=torch.float64, device=mesh.device)
        f = _source_values(self.source, mesh, bcs, index)
        NC = cm.shape[0]
        if isinstance(f, float):
            return cells, cm, 0, f, None, wphi, sv
        if f.numel() == 1:
            return cells, cm, 0, float(f.reshape(-1)[0].item()), None, wphi, sv
        if f.ndim == 1 and f.shape[0] == NC:
            return cells, cm, 1, 0.0, f, wphi, sv
        f = torch.broadcast_to(f, (NC, len(ws))).contiguous()
        return cells, cm, 2, 0.0, f, wphi, sv

    def assembly(self, space, /, indices=None) -> torch.Tensor:
        """Cell vectors (NC, ldof) of the source (``fgb_source_local``)."""
        _, cm, mode, fs, f, wphi, sv = self.source_data(space)
        out = K.source_local(cm, mode, fs, f, wphi, sv, space.number_of_local_dofs())
        return out if indices is None else out[indices]


class VectorSourceIntegrator(Integrator):
    """``(f, v)`` for a vector source on a TensorFunctionSpace (interleaved)."""

    def __init__(self, source=None, q: Optional[int] = None, *, region=None, method=None):
        super().__init__()
        self.source = source
        self.q = q
        self.set_region(region)

    def assembly(self, space, /, indices=None) -> torch.Tensor:
        """Cell vectors (NC, ldof * GD): per component the scalar source
        kernel (``fgb_source_local``; a constant component as a number, a
        callable's values per quadrature point, a (NC, GD) tensor per cell),
        laid out as the space numbers its components (interleaved or
        component-major), as ``fealpy/fem/vector_source_integrator.py`` does."""
        self._check_region()
        ss = space.scalar_space
        mesh = ss.mesh
        gd = space.dof_numel
        q = ss.p + 3 if self.q is None else self.q
        bcs, ws = mesh.quadrature_formula(q).get_quadrature_points_and_weights()
        cells = self.cell_selection(mesh)
        index = _S if cells is None else cells
        cm = mesh.entity_measure("cell", index=index)
        NC = cm.shape[0]
        wphi_np = ws[:, None] * sx.shape_function(bcs, ss.p)                       # (NQ, ldof)
        wphi = torch.as_tensor(wphi_np, dtype=torch.float64, device=mesh.device).contiguous()
        sv = torch.as_tensor(wphi_np.sum(axis=0), dtype=torch.float64, device=mesh.device)
        ldof = ss.number_of_local_dofs()
        f = self.source
        comps = []
        if callable(f):
            fq = torch.broadcast_to(_source_values(f, mesh, bcs, index), (NC, len(ws), gd))
            for d in range(gd):
                comps.append(K.source_local(cm, 2, 0.0, fq[..., d].contiguous(), wphi, sv, ldof))
        else:
            ft = torch.as_tensor(f, dtype=torch.float64)
            if ft.ndim == 2 and ft.shape == (NC, gd):
                ft = ft.to(mesh.device)
                for d in range(gd):
                    comps.append(K.source_local(cm, 1, 0.0, ft[:, d].contiguous(), wphi, sv, ldof))
            else:
                fv = ft.reshape(-1).cpu().tolist()
                if len(fv) != gd:
                    raise ValueError(f"a constant vector source needs {gd} components")
                for d in range(gd):
                    comps.append(K.source_local(cm, 0, float(fv[d]), None, wphi, sv, ldof))
        loc = torch.stack(comps, dim=-1)                                           # (NC, ldof, gd)
        if space.dof_priority:
            loc = loc.transpose(1, 2)
        return loc.reshape(NC, -1)
