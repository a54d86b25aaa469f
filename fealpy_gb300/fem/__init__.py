"""Forms, integrators and boundary conditions (the ``fealpy.fem`` subset on the GB300 path)."""
from .integrators import (Integrator, GroupIntegrator, ScalarDiffusionIntegrator, ScalarMassIntegrator,
                          LinearElasticityIntegrator, ScalarSourceIntegrator, VectorSourceIntegrator)
from .forms import BilinearForm, LinearForm
from .dirichlet_bc import DirichletBC

__all__ = ["Integrator", "GroupIntegrator", "ScalarDiffusionIntegrator", "ScalarMassIntegrator",
           "LinearElasticityIntegrator", "ScalarSourceIntegrator", "VectorSourceIntegrator", "BilinearForm",
           "LinearForm", "DirichletBC"]
