"""GB300-native implementation of FEALPy's Lagrange assemble + Dirichlet + Jacobi-PCG path.

The public modules mirror FEALPy's: ``mesh`` (TriangleMesh, TetrahedronMesh),
``functionspace`` (LagrangeFESpace, TensorFunctionSpace), ``fem``
(BilinearForm, LinearForm, integrators, DirichletBC), ``sparse`` (CSRTensor, COOTensor),
``solver`` (cg, cg_mixed, JacobiPreconditioner), ``amg`` (GAMGSolver,
AMGPreconditioner: the multigrid for cg's M slot) and ``material``.  Assembly,
boundary conditions, SpMV and CG run as hand-written sm_103a kernels reached
through the C ABI of ``fealpy_gb300/_lib/libfealpy_gb300.so``.
"""
from .mesh import TriangleMesh, TetrahedronMesh
from .functionspace import LagrangeFESpace, TensorFunctionSpace
from .sparse import CSRTensor, COOTensor
from .solver import cg, cg_mixed, JacobiPreconditioner
from .amg import GAMGSolver, AMGPreconditioner
from .material import LinearElasticMaterial
from . import fem

__version__ = "0.1.0"

__all__ = ["TriangleMesh", "TetrahedronMesh", "LagrangeFESpace", "TensorFunctionSpace", "CSRTensor", "COOTensor",
           "cg", "cg_mixed", "JacobiPreconditioner", "GAMGSolver", "AMGPreconditioner", "LinearElasticMaterial", "fem"]
