"""CSR sparse tensor with FEALPy's ``CSRTensor`` interface
(``fealpy/sparse/csr_tensor.py:16-590``), backed by the GB300 SpMV kernel."""
from typing import Optional, Tuple

import torch

from . import kernels as K

__all__ = ["CSRTensor", "spdiags"]


class CSRTensor:
    """Compressed sparse rows: ``crow`` int64 (n+1), ``col`` int32 (nnz),
    ``values`` (nnz,) float.  Matrices produced by this package are canonical
    (columns strictly ascending within a row, duplicates summed)."""

    def __init__(self, crow: torch.Tensor, col: torch.Tensor, values: Optional[torch.Tensor],
                 spshape: Optional[Tuple[int, int]] = None):
        self._crow = crow
        self._col = col
        self._values = values
        # sizes of the contiguous dof ranges of the space the matrix was
        # assembled on (vertex, edge, face, cell dofs), or None
        self.dof_blocks = None
        # 3 when the nonzeros come in runs of three consecutive columns (a
        # vector space with three interleaved components), else 1
        self.node_block = 1
        if spshape is None:
            spshape = (crow.shape[0] - 1, int(col.max().item()) + 1 if col.numel() else 0)
        self._spshape = tuple(int(s) for s in spshape)
        if crow.ndim != 1 or col.ndim != 1:
            raise ValueError("crow and col must be 1-D")
        if self._spshape[0] != crow.shape[0] - 1:
            raise ValueError("crow.shape[0] - 1 must be equal to spshape[0]")
        if values is not None and values.shape[-1] != col.shape[-1]:
            raise ValueError("values must have the same size as col")
        self._f32 = None      # optional float copy of the values (mixed precision)
        self._dinv = None     # cached inverse diagonal

    # data access ---------------------------------------------------------
    @property
    def crow(self):
        return self._crow

    @property
    def col(self):
        return self._col

    @property
    def values(self):
        return self._values

    indptr = crow
    indices = col
    data = values

    @property
    def nnz(self):
        return self._col.shape[-1]

    @property
    def shape(self):
        return self._spshape

    @property
    def sparse_shape(self):
        return self._spshape

    @property
    def dtype(self):
        return self._values.dtype

    @property
    def device(self):
        return self._crow.device

    @property
    def itype(self):
        return self._col.dtype

    @property
    def row(self):
        counts = self._crow[1:] - self._crow[:-1]
        return torch.repeat_interleave(torch.arange(self._spshape[0], device=self.device), counts)

    def values_context(self):
        return {"dtype": self._values.dtype, "device": self._values.device}

    def __repr__(self):
        return f"CSRTensor(shape={self.shape}, nnz={self.nnz}, dtype={self._values.dtype}, device={self.device})"

    # conversions ------------------------------------------------------------
    def to_dense(self):
        out = torch.zeros(self._spshape, dtype=self._values.dtype, device=self.device)
        out[self.row, self._col.long()] = self._values
        return out

    def to_scipy(self):
        from scipy.sparse import csr_matrix
        return csr_matrix((self._values.cpu().numpy(), self._col.cpu().numpy(), self._crow.cpu().numpy()),
                          shape=self._spshape)

    @classmethod
    def from_scipy(cls, mat, device="cuda"):
        return cls(torch.as_tensor(mat.indptr, dtype=torch.int64, device=device),
                   torch.as_tensor(mat.indices, dtype=torch.int32, device=device),
                   torch.as_tensor(mat.data, device=device), mat.shape)

    def tocsr(self, copy=False):
        return self.copy() if copy else self

    def copy(self):
        return CSRTensor(self._crow.clone(), self._col.clone(),
                         None if self._values is None else self._values.clone(), self._spshape)

    def astype(self, dtype=None, *, copy=True):
        return CSRTensor(self._crow, self._col, self._values.to(dtype), self._spshape)

    def device_put(self, device=None):
        return CSRTensor(self._crow.to(device), self._col.to(device), self._values.to(device), self._spshape)

    # arithmetic ---------------------------------------------------------------
    def values_f32(self) -> torch.Tensor:
        """Float copy of the values (computed once and cached)."""
        if self._f32 is None:
            self._f32 = self._values.to(torch.float32)
        return self._f32

    def matmul(self, other):
        if isinstance(other, CSRTensor):
            raise NotImplementedError("sparse-sparse products are not on the GB300 path")
        if not isinstance(other, torch.Tensor):
            raise TypeError(f"Unsupported type {type(other).__name__} in matmul")
        if other.ndim == 1:
            return K.csr_spmv(self._crow, self._col, self._values, other)
        if other.ndim == 2:
            cols = [K.csr_spmv(self._crow, self._col, self._values, other[:, k].contiguous())
                    for k in range(other.shape[1])]
            return torch.stack(cols, dim=1)
        raise ValueError("`other` must be a 1-D or 2-D tensor")

    __matmul__ = matmul

    def diags(self) -> "CSRTensor":
        """Diagonal part (FEALPy ``CSRTensor.diags``); every row of an
        assembled FE matrix has its diagonal entry."""
        d, _ = K.csr_diagonal(self._crow, self._col, self._values)
        n = self._spshape[0]
        crow = torch.arange(n + 1, dtype=torch.int64, device=self.device)
        col = torch.arange(n, dtype=torch.int32, device=self.device)
        out = CSRTensor(crow, col, d, self._spshape)
        return out

    def diagonal_inverse(self) -> torch.Tensor:
        if self._dinv is None:
            _, self._dinv = K.csr_diagonal(self._crow, self._col, self._values)
        return self._dinv

    def is_diagonal(self) -> bool:
        n = self._spshape[0]
        if self.nnz != n or self._spshape[0] != self._spshape[1]:
            return False
        return bool(torch.equal(self._col.long(), torch.arange(n, device=self.device)))

    def neg(self):
        return CSRTensor(self._crow, self._col, -self._values, self._spshape)

    __neg__ = neg

    def mul(self, scalar):
        if isinstance(scalar, (int, float)):
            return CSRTensor(self._crow, self._col, self._values * scalar, self._spshape)
        raise NotImplementedError("only scalar scaling is provided")

    __mul__ = mul
    __rmul__ = mul


def spdiags(data: torch.Tensor, diags: int, M: int, N: int, format="csr") -> CSRTensor:
    """Diagonal CSR keeping only nonzero entries (``fealpy/sparse/ops.py:18-86``, diags=0)."""
    if diags != 0 or M != N:
        raise NotImplementedError("only the main diagonal of a square matrix is provided")
    nz = torch.nonzero(data).reshape(-1)
    counts = torch.zeros(M, dtype=torch.int64, device=data.device)
    counts[nz] = 1
    crow = torch.cat([torch.zeros(1, dtype=torch.int64, device=data.device), torch.cumsum(counts, 0)])
    return CSRTensor(crow, nz.to(torch.int32), data[nz], (M, N))
