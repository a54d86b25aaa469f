"""``DirichletBC`` with FEALPy's interface (``fealpy/fem/dirichlet_bc.py:13-229``)."""
from typing import Optional

import torch

from ..sparse import CSRTensor
from .. import kernels as K

__all__ = ["DirichletBC"]


class DirichletBC:
    """Dirichlet condition by symmetric elimination: boundary rows and columns
    are removed from ``A`` and replaced by a unit diagonal, and
    ``f <- f - A u_D`` with ``f[bd] = u_D[bd]``."""

    def __init__(self, space, gd=None, *, threshold=None, method=None):
        if isinstance(space, tuple):
            raise NotImplementedError("DirichletBC over a tuple of spaces is not provided")
        self.space = space
        self.gd = gd
        self.threshold = threshold
        self.method = method
        self.bctype = "Dirichlet"
        self.gdof = space.number_of_global_dofs()
        if isinstance(threshold, torch.Tensor):
            self.is_boundary_dof = threshold
        else:
            self.is_boundary_dof = space.is_boundary_dof(threshold=threshold, method=method)
        self.boundary_dof_index = torch.nonzero(self.is_boundary_dof).reshape(-1)

    def check_matrix(self, matrix):
        if not isinstance(matrix, CSRTensor):
            raise ValueError("The type of matrix must be CSRTensor.")
        matrix._single("DirichletBC.apply")
        if matrix.shape[0] != matrix.shape[1]:
            raise ValueError("The matrix must be a square matrix.")
        if matrix.shape[0] != self.gdof:
            raise ValueError("The matrix size must match the gdof of the space.")
        return matrix

    def check_vector(self, vector):
        if not isinstance(vector, torch.Tensor):
            raise ValueError("The type of vector must be a tensor.")
        if vector.ndim != 1:
            raise ValueError("The vector must be 1-D.")
        if vector.shape[0] != self.gdof:
            raise ValueError("The vector size must match the gdof of the space.")
        return vector

    def _boundary_values(self, f, uh, gd):
        """u_h with the boundary values interpolated; None for homogeneous data
        (``gd`` the number 0 and no ``uh``), which lets the elimination skip
        the product A u_h (it is zero)."""
        gd = self.gd if gd is None else gd
        if gd is None:
            raise RuntimeError("The boundary condition is None.")
        if uh is None and isinstance(gd, (int, float)) and float(gd) == 0.0:
            return None
        if uh is None:
            uh = torch.zeros_like(f)
        uh, _ = self.space.boundary_interpolate(gd=gd, uh=uh, threshold=self.threshold, method=self.method)
        return uh

    def apply(self, A: CSRTensor, f: torch.Tensor, uh: Optional[torch.Tensor] = None, gd=None, *, check=True):
        if check:
            self.check_matrix(A)
            self.check_vector(f)
        uh = self._boundary_values(f, uh, gd)
        ptr_, idx, val, f_new = K.dirichlet_apply(A.crow, A.col, A.values, self.is_boundary_dof, f, uh, matrix=True)
        out = CSRTensor(ptr_, idx, val, A.shape)
        out.dof_blocks = getattr(A, "dof_blocks", None)
        out.node_block = getattr(A, "node_block", 1)
        return out, f_new

    def apply_matrix(self, matrix: CSRTensor, *, check=True) -> CSRTensor:
        A = self.check_matrix(matrix) if check else matrix
        ptr_, idx, val, _ = K.dirichlet_apply(A.crow, A.col, A.values, self.is_boundary_dof, None, None, matrix=True)
        out = CSRTensor(ptr_, idx, val, A.shape)
        out.dof_blocks = getattr(A, "dof_blocks", None)
        out.node_block = getattr(A, "node_block", 1)
        return out

    def apply_vector(self, vector, matrix, uh=None, gd=None, *, check=True):
        A = self.check_matrix(matrix) if check else matrix
        f = self.check_vector(vector) if check else vector
        uh = self._boundary_values(f, uh, gd)
        _, _, _, f_new = K.dirichlet_apply(A.crow, A.col, A.values, self.is_boundary_dof, f, uh, matrix=False)
        return f_new
