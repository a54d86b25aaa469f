"""CSR sparse tensor with FEALPy's ``CSRTensor`` interface
(``fealpy/sparse/csr_tensor.py:16-590``), backed by the GB300 SpMV kernel."""
from typing import Optional, Tuple

import torch

from . import kernels as K

__all__ = ["CSRTensor", "COOTensor", "spdiags"]


class CSRTensor:
    """Compressed sparse rows: ``crow`` int64 (n+1), ``col`` int32 (nnz),
    ``values`` (nnz,) float, or (B, nnz) for a batch of B matrices on one
    pattern (a form with batched coefficients).  Matrices produced by this
    package are canonical (columns strictly ascending within a row,
    duplicates summed)."""

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
    def is_batched(self) -> bool:
        return self._values is not None and self._values.ndim > 1

    @property
    def dense_shape(self):
        return tuple(self._values.shape[:-1]) if self.is_batched else ()

    @property
    def shape(self):
        return self.dense_shape + self._spshape

    @property
    def sparse_shape(self):
        return self._spshape

    def _single(self, what: str):
        if self.is_batched:
            raise ValueError(f"{what} takes one matrix; a batched matrix's member b is "
                             "CSRTensor(A.crow, A.col, A.values[b], A.sparse_shape)")

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
        out = torch.zeros(self.dense_shape + self._spshape, dtype=self._values.dtype, device=self.device)
        out[..., self.row, self._col.long()] = self._values
        return out

    def to_scipy(self):
        self._single("to_scipy")
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

    def tocoo(self, *, copy=False) -> "COOTensor":
        """Coordinate form of the same entries in the same order
        (``fealpy/sparse/csr_tensor.py:149-155``); a canonical CSR gives a
        coalesced COO."""
        indices = torch.stack([self.row, self._col.long()], dim=0)
        values = self._values.clone() if (copy and self._values is not None) else self._values
        return COOTensor(indices, values, self._spshape, is_coalesced=True)

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
        self._single("the FP32 solver copy")
        if self._f32 is None:
            self._f32 = self._values.to(torch.float32)
        return self._f32

    def matmul(self, other):
        if isinstance(other, CSRTensor):
            raise NotImplementedError("sparse-sparse products are not on the GB300 path")
        if not isinstance(other, torch.Tensor):
            raise TypeError(f"Unsupported type {type(other).__name__} in matmul")
        if self.is_batched:
            # one product per member: a vector for all members (B, n), or one
            # vector per member (B, m) -> (B, n)
            vals = self._values.reshape(-1, self.nnz)
            if other.ndim == 1:
                out = [K.csr_spmv(self._crow, self._col, v.contiguous(), other) for v in vals]
            elif other.ndim == 2 and other.shape[0] == vals.shape[0] and other.shape[1] == self._spshape[1]:
                out = [K.csr_spmv(self._crow, self._col, v.contiguous(), x.contiguous())
                       for v, x in zip(vals, other)]
            else:
                raise ValueError("a batched matrix multiplies a vector (m,) or one vector per member (B, m)")
            return torch.stack(out).reshape(self.dense_shape + (self._spshape[0],))
        if other.ndim == 1:
            return K.csr_spmv(self._crow, self._col, self._values, other)
        if other.ndim == 2:
            if self._values.dtype == torch.float64 and 1 <= other.shape[1] <= 64:
                # all columns in one pass over the matrix
                return K.csr_spmm(self._crow, self._col, self._values, other)
            cols = [K.csr_spmv(self._crow, self._col, self._values, other[:, k].contiguous())
                    for k in range(other.shape[1])]
            return torch.stack(cols, dim=1)
        raise ValueError("`other` must be a 1-D or 2-D tensor")

    __matmul__ = matmul

    def diags(self) -> "CSRTensor":
        """Diagonal part (FEALPy ``CSRTensor.diags``); every row of an
        assembled FE matrix has its diagonal entry."""
        self._single("diags")
        d, _ = K.csr_diagonal(self._crow, self._col, self._values)
        n = self._spshape[0]
        crow = torch.arange(n + 1, dtype=torch.int64, device=self.device)
        col = torch.arange(n, dtype=torch.int32, device=self.device)
        out = CSRTensor(crow, col, d, self._spshape)
        return out

    def diagonal_inverse(self) -> torch.Tensor:
        self._single("diagonal_inverse")
        if self._dinv is None:
            _, self._dinv = K.csr_diagonal(self._crow, self._col, self._values)
        return self._dinv

    def is_diagonal(self) -> bool:
        if self.is_batched:
            return False
        n = self._spshape[0]
        if self.nnz != n or self._spshape[0] != self._spshape[1]:
            return False
        return bool(torch.equal(self._col.long(), torch.arange(n, device=self.device)))

    def neg(self):
        return CSRTensor(self._crow, self._col, -self._values, self._spshape)

    __neg__ = neg

    # FEALPy's element-wise arithmetic and sparse utilities
    # (``fealpy/sparse/csr_tensor.py:218-420``, operators
    # ``fealpy/sparse/sparse_tensor.py:131-216``) ------------------------------
    @property
    def nonzero_slice(self):
        return self.row, self._col.long()

    def _vals(self):
        return self._values if self._values is not None else torch.ones(self.nnz, dtype=torch.float64,
                                                                         device=self.device)

    def _same_pattern(self, other: "CSRTensor") -> bool:
        if self._crow is other._crow and self._col is other._col:
            return True
        return (self.nnz == other.nnz and torch.equal(self._crow, other._crow)
                and torch.equal(self._col, other._col))

    def add(self, other, alpha=1):
        """``self + alpha * other``: a CSRTensor for a CSRTensor (the union of
        the two patterns, duplicates summed; two matrices of one pattern, such
        as two forms assembled on one space, add their values) or a number
        (added to the stored entries); a dense tensor for a dense tensor."""
        if isinstance(other, CSRTensor):
            if tuple(self.shape) != tuple(other.shape):
                raise ValueError(f"shapes {self.shape} and {other.shape} do not match")
            if self._same_pattern(other):
                return CSRTensor(self._crow, self._col, self._vals() + alpha * other._vals(), self._spshape)
            indices = torch.cat([torch.stack(self.nonzero_slice), torch.stack(other.nonzero_slice)], dim=1)
            values = torch.cat([self._vals(), alpha * other._vals()])
            return COOTensor(indices, values, self._spshape).tocsr()
        if isinstance(other, torch.Tensor):
            if tuple(other.shape) != tuple(self.shape):
                raise ValueError(f"shapes {self.shape} and {tuple(other.shape)} do not match")
            out = other * alpha
            out = out.to(torch.promote_types(out.dtype, self._vals().dtype)).clone()
            nz = (Ellipsis,) + self.nonzero_slice     # (row, col) of every member; no duplicates
            out[nz] = out[nz] + self._vals().to(out.dtype)
            return out
        if isinstance(other, (int, float)):
            return CSRTensor(self._crow.clone(), self._col.clone(), self._vals() + alpha * other, self._spshape)
        raise TypeError(f"Unsupported type {type(other).__name__} in addition")

    def __add__(self, other):
        return self.add(other)

    __radd__ = __add__

    def __sub__(self, other):
        return self.add(other, alpha=-1)

    def __rsub__(self, other):
        return self.neg().add(other)

    def mul(self, other):
        """Element-wise product with a number or a dense tensor (the stored
        entries only)."""
        if isinstance(other, (int, float)):
            if self._values is None:
                raise ValueError("Cannot multiply CSRTensor without value with scalar")
            return CSRTensor(self._crow, self._col, self._values * other, self._spshape)
        if isinstance(other, torch.Tensor):
            if tuple(other.shape) != tuple(self.shape):
                raise ValueError(f"shapes {self.shape} and {tuple(other.shape)} do not match")
            vals = other[(Ellipsis,) + self.nonzero_slice]
            if self._values is not None:
                vals = self._values * vals
            return CSRTensor(self._crow, self._col, vals, self._spshape)
        if isinstance(other, CSRTensor):
            raise NotImplementedError("element-wise products of two sparse matrices are not provided")
        raise TypeError(f"Unsupported type {type(other).__name__} in multiplication")

    __mul__ = mul
    __rmul__ = mul

    def div(self, other):
        """Element-wise quotient by a number or a dense tensor (a vector of
        length rows or columns broadcasts along that axis)."""
        if self._values is None:
            raise ValueError("Cannot divide CSRTensor without value")
        if isinstance(other, (int, float)):
            return CSRTensor(self._crow, self._col, self._values / other, self._spshape)
        if isinstance(other, torch.Tensor):
            if other.ndim == 1:
                if other.shape[0] == self._spshape[0]:
                    return CSRTensor(self._crow, self._col, self._values / other[self.row], self._spshape)
                if other.shape[0] == self._spshape[1]:
                    return CSRTensor(self._crow, self._col, self._values / other[self._col.long()], self._spshape)
            if tuple(other.shape) != tuple(self.shape):
                raise ValueError(f"shapes {self.shape} and {tuple(other.shape)} do not match")
            return CSRTensor(self._crow, self._col, self._values / other[(Ellipsis,) + self.nonzero_slice],
                             self._spshape)
        raise TypeError(f"Unsupported type {type(other).__name__} in division")

    __truediv__ = div

    def pow(self, other):
        if self._values is None:
            raise ValueError("Cannot power CSRTensor without value with tensor")
        if isinstance(other, (int, float)):
            return CSRTensor(self._crow, self._col, self._values ** other, self._spshape)
        if isinstance(other, torch.Tensor):
            if tuple(other.shape) != tuple(self.shape):
                raise ValueError(f"shapes {self.shape} and {tuple(other.shape)} do not match")
            return CSRTensor(self._crow, self._col, self._values ** other[(Ellipsis,) + self.nonzero_slice],
                             self._spshape)
        raise TypeError(f"Unsupported type {type(other).__name__} in power")

    __pow__ = pow

    def partial(self, index) -> "CSRTensor":
        """The stored entries selected by a boolean mask (or an index) over
        the nonzeros, rows kept."""
        sel = torch.zeros(self.nnz, dtype=torch.bool, device=self.device)
        sel[index] = True
        cum = torch.zeros(self.nnz + 1, dtype=torch.int64, device=self.device)
        torch.cumsum(sel, 0, out=cum[1:])
        crow = cum[self._crow]
        values = None if self._values is None else self._values[sel]
        return CSRTensor(crow, self._col[sel], values, self._spshape)

    def tril(self, k: int = 0) -> "CSRTensor":
        return self.partial(self.row + k >= self._col.long())

    def triu(self, k: int = 0) -> "CSRTensor":
        return self.partial(self._col.long() - k >= self.row)

    def sum(self, axis=0):
        """Row sums (axis 0, the product with a vector of ones, as FEALPy
        forms it) or column sums (axis 1)."""
        if axis == 0:
            return self @ torch.ones(self._spshape[1], dtype=self._vals().dtype, device=self.device)
        if axis == 1:
            v = self._vals()
            out = torch.zeros(v.shape[:-1] + (self._spshape[1],), dtype=v.dtype, device=self.device)
            return out.index_add_(-1, self._col.long(), v)
        raise ValueError("axis must be 0 or 1")

    @property
    def T(self) -> "CSRTensor":
        """The transpose (through the coordinate form, as FEALPy forms it)."""
        row, col = self.nonzero_slice
        return COOTensor(torch.stack([col, row]), self._values, (self._spshape[1], self._spshape[0])).tocsr()


class COOTensor:
    """Coordinate sparse matrix with FEALPy's ``COOTensor`` interface
    (``fealpy/sparse/coo_tensor.py:14-213``): ``indices`` (2, nnz) int64 rows
    and columns, ``values`` (nnz,) or None.  Products go through the CSR form
    (``tocsr``) and its SpMV kernel."""

    def __init__(self, indices: torch.Tensor, values: Optional[torch.Tensor],
                 spshape: Optional[Tuple[int, int]] = None, *, is_coalesced: Optional[bool] = None):
        if not isinstance(indices, torch.Tensor):
            raise TypeError(f"indices must be a Tensor, but got {type(indices)}")
        if indices.ndim != 2 or indices.shape[0] != 2:
            raise ValueError("indices must be shaped (2, nnz)")
        if values is not None:
            if not isinstance(values, torch.Tensor):
                raise TypeError(f"values must be a Tensor or None, but got {type(values)}")
            if values.ndim < 1 or values.shape[-1] != indices.shape[1]:
                raise ValueError("values must be shaped (..., nnz) like the indices")
        self._indices = indices
        self._values = values
        self.is_coalesced = is_coalesced
        if spshape is None:
            spshape = tuple(int(v) + 1 for v in indices.max(dim=1).values.tolist()) if indices.numel() else (0, 0)
        if len(spshape) != 2:
            raise ValueError("a COO matrix has two sparse dimensions")
        self._spshape = tuple(int(s) for s in spshape)

    @property
    def indices(self):
        return self._indices

    @property
    def values(self):
        return self._values

    data = values

    @property
    def row(self):
        return self._indices[0]

    @property
    def col(self):
        return self._indices[1]

    @property
    def nnz(self):
        return self._indices.shape[1]

    @property
    def dense_shape(self):
        return tuple(self._values.shape[:-1]) if self._values is not None else ()

    @property
    def shape(self):
        return self.dense_shape + self._spshape

    @property
    def sparse_shape(self):
        return self._spshape

    @property
    def dtype(self):
        return None if self._values is None else self._values.dtype

    @property
    def itype(self):
        return self._indices.dtype

    @property
    def device(self):
        return self._indices.device

    def __repr__(self):
        return f"COOTensor(shape={self.shape}, nnz={self.nnz}, dtype={self.dtype}, device={self.device})"

    def coalesce(self, accumulate: bool = True) -> "COOTensor":
        """Entries sorted by (row, column) with duplicates summed
        (``fealpy/sparse/coo_tensor.py:184-213``); a matrix without values
        gets the multiplicity of each position (``accumulate``) or stays
        without values."""
        if self.is_coalesced or self.nnz == 0:
            return self
        key = self._indices[0] * self._spshape[1] + self._indices[1]
        uniq, inv = torch.unique(key, sorted=True, return_inverse=True)
        indices = torch.stack([uniq // self._spshape[1], uniq % self._spshape[1]], dim=0)
        if self._values is None and not accumulate:
            return COOTensor(indices, None, self._spshape, is_coalesced=True)
        src = self._values if self._values is not None else torch.ones(self.nnz, dtype=torch.int64,
                                                                       device=self.device)
        values = torch.zeros(src.shape[:-1] + (uniq.numel(),), dtype=src.dtype,
                             device=self.device).index_add_(-1, inv, src)
        return COOTensor(indices, values, self._spshape, is_coalesced=True)

    def tocoo(self, *, copy=False):
        return self.copy() if copy else self

    def tocsr(self, *, copy=False) -> CSRTensor:
        """CSR form of the coalesced entries (``fealpy/sparse/coo_tensor.py:137``)."""
        c = self.coalesce()
        counts = torch.bincount(c.row, minlength=self._spshape[0])
        crow = torch.zeros(self._spshape[0] + 1, dtype=torch.int64, device=self.device)
        torch.cumsum(counts, 0, out=crow[1:])
        values = c.values if c.values is not None else torch.ones(c.nnz, dtype=torch.float64, device=self.device)
        if copy and c is self:
            values = values.clone()
        return CSRTensor(crow, c.col.to(torch.int32), values, self._spshape)

    def to_dense(self):
        values = self._values if self._values is not None else torch.ones(self.nnz, dtype=torch.float64,
                                                                           device=self.device)
        out = torch.zeros(values.shape[:-1] + (self._spshape[0] * self._spshape[1],), dtype=values.dtype,
                          device=self.device)
        out.index_add_(-1, self._indices[0] * self._spshape[1] + self._indices[1], values)
        return out.reshape(values.shape[:-1] + self._spshape)

    def copy(self):
        return COOTensor(self._indices.clone(), None if self._values is None else self._values.clone(),
                         self._spshape, is_coalesced=self.is_coalesced)

    def astype(self, dtype=None, *, copy=True):
        values = torch.ones(self.nnz, dtype=dtype, device=self.device) if self._values is None \
            else self._values.to(dtype)
        return COOTensor(self._indices, values, self._spshape, is_coalesced=self.is_coalesced)

    def device_put(self, device=None):
        return COOTensor(self._indices.to(device), None if self._values is None else self._values.to(device),
                         self._spshape, is_coalesced=self.is_coalesced)

    def matmul(self, other):
        return self.tocsr().matmul(other)

    __matmul__ = matmul


def spdiags(data: torch.Tensor, diags: int, M: int, N: int, format="csr") -> CSRTensor:
    """Diagonal CSR keeping only nonzero entries (``fealpy/sparse/ops.py:18-86``, diags=0)."""
    if diags != 0 or M != N:
        raise NotImplementedError("only the main diagonal of a square matrix is provided")
    nz = torch.nonzero(data).reshape(-1)
    counts = torch.zeros(M, dtype=torch.int64, device=data.device)
    counts[nz] = 1
    crow = torch.cat([torch.zeros(1, dtype=torch.int64, device=data.device), torch.cumsum(counts, 0)])
    return CSRTensor(crow, nz.to(torch.int32), data[nz], (M, N))
