"""Lagrange and tensor function spaces (``fealpy/functionspace/lagrange_fe_space.py``,
``fealpy/functionspace/tensor_space.py``) on the meshes of :mod:`fealpy_gb300.mesh`."""
from math import prod
from typing import Callable, Optional, Tuple

import torch


__all__ = ["LagrangeFESpace", "TensorFunctionSpace"]

_S = slice(None)


class LagrangeFESpace:
    """Continuous P-k Lagrange space (``ctype='C'``) on a simplex mesh."""

    def __init__(self, mesh, p: int = 1, ctype: str = "C"):
        if ctype != "C":
            raise NotImplementedError("only continuous Lagrange spaces are provided")
        self.mesh = mesh
        self.p = p
        self.ctype = ctype
        self.ftype = mesh.ftype
        self.itype = mesh.itype
        self.device = mesh.device
        self.TD = mesh.top_dimension()
        self.GD = mesh.geo_dimension()
        self._c2d = None
        self._cache = {}

    def __str__(self):
        return "Lagrange finite element space on linear mesh!"

    # sizes and maps ------------------------------------------------------
    def number_of_local_dofs(self, doftype="cell") -> int:
        return self.mesh.number_of_local_ipoints(self.p, doftype)

    def number_of_global_dofs(self) -> int:
        return self.mesh.number_of_global_ipoints(self.p)

    def dof_blocks(self):
        """Sizes of the contiguous dof ranges (vertex, edge, face and cell
        dofs) in global dof order."""
        return self.mesh.ipoint_blocks(self.p)

    def cell_to_dof(self, index=_S) -> torch.Tensor:
        if self._c2d is None:
            self._c2d = self.mesh.cell_to_ipoint(self.p).contiguous()
        return self._c2d[index]

    def interpolation_points(self) -> torch.Tensor:
        return self.mesh.interpolation_points(self.p)

    def face_dof_mask(self):
        return self.mesh.face_dof_mask(self.p)

    def is_boundary_dof(self, threshold=None, method=None) -> torch.Tensor:
        """Dofs on boundary facets (``fealpy/functionspace/dofs.py:23-55``).

        ``method`` None/'centroid' filters boundary facets by ``threshold`` at
        their barycentres; 'interp' filters the boundary dofs by ``threshold`` at
        their interpolation points.  A boolean tensor of length gdof is returned
        unchanged."""
        gdof = self.number_of_global_dofs()
        if isinstance(threshold, torch.Tensor):
            if threshold.dtype == torch.bool and threshold.numel() == gdof:
                return threshold
            raise ValueError(f"Unknown threshold: {threshold}")
        mesh = self.mesh
        bdf = mesh.boundary_face_index()
        if callable(threshold) and (method in (None, "centroid")):
            bc = mesh.entity_barycenter("face" if mesh.TD == 3 else "edge", bdf)
            bdf = bdf[torch.as_tensor(threshold(bc), device=bdf.device)]
        f2c = mesh.face2cell[bdf].to(torch.int64)
        cells, lfaces = f2c[:, 0], f2c[:, 2]
        on_face = self.face_dof_mask()[lfaces]                       # (nbf, ldof)
        dofs = self.cell_to_dof()[cells].to(torch.int64)[on_face]
        flag = torch.zeros(gdof, dtype=torch.bool, device=self.device)
        if callable(threshold) and method == "interp":
            ip = self.interpolation_points()[dofs]
            dofs = dofs[torch.as_tensor(threshold(ip), device=dofs.device)]
        flag[dofs] = True
        return flag

    def boundary_interpolate(self, gd, uh: Optional[torch.Tensor] = None, *, threshold=None, method=None):
        """Set boundary values into ``uh`` (``lagrange_fe_space.py:109-142``);
        returns ``(uh, isDDof)``."""
        isDDof = self.is_boundary_dof(threshold=threshold, method="interp")
        if uh is None:
            uh = torch.zeros(self.number_of_global_dofs(), dtype=self.ftype, device=self.device)
        if isinstance(gd, torch.Tensor):
            uh[..., isDDof] = gd[isDDof].to(uh.dtype)
        elif callable(gd):
            ip = self.interpolation_points()[isDDof]
            uh[..., isDDof] = torch.as_tensor(gd(ip), dtype=uh.dtype, device=uh.device)
        elif isinstance(gd, (int, float)):
            uh[..., isDDof] = float(gd)
        else:
            raise TypeError("gd must be a tensor, a number or a callable")
        return uh, isDDof

    set_dirichlet_bc = boundary_interpolate

    def interpolate(self, u: Callable) -> torch.Tensor:
        return torch.as_tensor(u(self.interpolation_points()), dtype=self.ftype, device=self.device)

    def array(self, dim=None, dtype=None):
        shape = (self.number_of_global_dofs(),) if dim is None else (self.number_of_global_dofs(), dim)
        return torch.zeros(shape, dtype=dtype or self.ftype, device=self.device)

    function = array

    # basis ---------------------------------------------------------------
    def basis(self, bc, index=_S):
        return self.mesh.shape_function(bc, self.p)[None, ...]

    def grad_basis(self, bc, index=_S, variable="x"):
        return self.mesh.grad_shape_function(bc, self.p, index=index, variables=variable)


class TensorFunctionSpace:
    """Vector/tensor space built from a scalar space (``tensor_space.py:13-38``).
    ``shape=(-1, GD)`` is the interleaved layout ``dof = GD*node + comp``
    (``dof_priority=False``); ``shape=(GD, -1)`` is component-major."""

    def __init__(self, scalar_space: LagrangeFESpace, shape: Tuple[int, ...]):
        self.scalar_space = scalar_space
        self.shape = tuple(shape)
        if len(shape) < 2:
            raise ValueError("shape must be a tuple of at least two element")
        if shape[0] == -1:
            self.dof_shape = tuple(shape[1:])
            self.dof_priority = False
        elif shape[-1] == -1:
            self.dof_shape = tuple(shape[:-1])
            self.dof_priority = True
        else:
            raise ValueError("`-1` is required as the first or last element")
        self.p = scalar_space.p
        self._cache = {}

    @property
    def mesh(self):
        return self.scalar_space.mesh

    @property
    def device(self):
        return self.scalar_space.device

    @property
    def ftype(self):
        return self.scalar_space.ftype

    @property
    def itype(self):
        return self.scalar_space.itype

    @property
    def dof_numel(self) -> int:
        return prod(self.dof_shape)

    def number_of_global_dofs(self) -> int:
        return self.dof_numel * self.scalar_space.number_of_global_dofs()

    def number_of_local_dofs(self, doftype="cell") -> int:
        return self.dof_numel * self.scalar_space.number_of_local_dofs(doftype)

    def dof_blocks(self):
        """Contiguous dof ranges: the scalar blocks scaled by the number of
        components (interleaved layout), or repeated per component
        (component-major layout)."""
        sb = self.scalar_space.dof_blocks()
        if self.dof_priority:
            return sb * self.dof_numel
        return [self.dof_numel * v for v in sb]

    def _expand(self, to_dof: torch.Tensor) -> torch.Tensor:
        n = self.dof_numel
        sg = self.scalar_space.number_of_global_dofs()
        d = to_dof.to(torch.int64)
        comp = torch.arange(n, device=d.device)
        if self.dof_priority:
            out = comp[:, None] * sg + d[:, None, :]          # (NC, n, ldof)
        else:
            out = d[:, :, None] * n + comp[None, None, :]     # (NC, ldof, n)
        return out.reshape(d.shape[0], -1).to(torch.int32)

    def cell_to_dof(self, index=_S):
        return self._expand(self.scalar_space.cell_to_dof())[index]

    def interpolation_points(self):
        return self.scalar_space.interpolation_points()

    def is_boundary_dof(self, threshold=None, method="interp") -> torch.Tensor:
        ss = self.scalar_space
        sg = ss.number_of_global_dofs()
        n = self.dof_numel
        if isinstance(threshold, torch.Tensor):
            if threshold.dtype == torch.bool and threshold.numel() == self.number_of_global_dofs():
                return threshold
            raise ValueError("len(threshold) must equal tensorspace gdof")
        if threshold is None or callable(threshold):
            s = ss.is_boundary_dof(threshold, method=method)
            if self.dof_priority:
                return s[None, :].expand(n, sg).reshape(-1).clone()
            return s[:, None].expand(sg, n).reshape(-1).clone()
        if isinstance(threshold, tuple):
            parts = [ss.is_boundary_dof(t, method=method) for t in threshold]
            if self.dof_priority:
                return torch.cat(parts)
            return torch.stack(parts, dim=1).reshape(-1)
        raise ValueError(f"Unknown type of threshold {type(threshold)}")

    def boundary_interpolate(self, gd, uh=None, *, threshold=None, method=None):
        isb = self.is_boundary_dof(threshold=threshold, method="interp")
        if uh is None:
            uh = torch.zeros(self.number_of_global_dofs(), dtype=self.ftype, device=self.device)
        ss = self.scalar_space
        n = self.dof_numel
        sg = ss.number_of_global_dofs()
        if isinstance(gd, (int, float)):
            uh[isb] = float(gd)
        elif isinstance(gd, torch.Tensor):
            uh[isb] = gd.reshape(-1)[isb].to(uh.dtype)
        elif callable(gd):
            ip = ss.interpolation_points()
            val = torch.as_tensor(gd(ip), dtype=uh.dtype, device=uh.device).reshape(sg, n)
            full = val.T.reshape(-1) if self.dof_priority else val.reshape(-1)
            uh[isb] = full[isb]
        else:
            raise TypeError("gd must be a number, tensor or callable")
        return uh, isb

    def array(self, dtype=None):
        return torch.zeros(self.number_of_global_dofs(), dtype=dtype or self.ftype, device=self.device)

    function = array
