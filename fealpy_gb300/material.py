"""``LinearElasticMaterial`` (``fealpy/material/elastic_material.py:184-319``):
Lame parameters to the Voigt elasticity matrix D."""
from typing import Optional

import torch

__all__ = ["LinearElasticMaterial"]


class LinearElasticMaterial:
    def __init__(self, name: str = "material", elastic_modulus: Optional[float] = None,
                 poisson_ratio: Optional[float] = None, lame_lambda: Optional[float] = None,
                 shear_modulus: Optional[float] = None, density: Optional[float] = None, hypo: str = "3D",
                 device=None, cell_scale: Optional[torch.Tensor] = None):
        """``cell_scale`` (NC,) multiplies D cell by cell, giving the
        (NC, 1, k, k) elastic matrix FEALPy's integrator accepts for
        heterogeneous materials."""
        self.name = name
        self.hypo = hypo
        self.device = device
        if elastic_modulus is not None and poisson_ratio is not None and lame_lambda is None and shear_modulus is None:
            E, nu = float(elastic_modulus), float(poisson_ratio)
            lam = nu * E / ((1 + nu) * (1 - 2 * nu))
            mu = E / (2 * (1 + nu))
        elif lame_lambda is not None and shear_modulus is not None:
            lam, mu = float(lame_lambda), float(shear_modulus)
            E = mu * (3 * lam + 2 * mu) / (lam + mu)
            nu = lam / (2 * (lam + mu))
        else:
            raise ValueError("You must provide either (elastic_modulus, poisson_ratio) or "
                             "(lame_lambda, shear_modulus).")
        self.E, self.nu, self.lam, self.mu, self.rho = E, nu, lam, mu, density
        if hypo == "3D":
            D = [[2 * mu + lam, lam, lam, 0, 0, 0], [lam, 2 * mu + lam, lam, 0, 0, 0],
                 [lam, lam, 2 * mu + lam, 0, 0, 0], [0, 0, 0, mu, 0, 0], [0, 0, 0, 0, mu, 0], [0, 0, 0, 0, 0, mu]]
            self.D = torch.tensor(D, dtype=torch.float64, device=device)
        elif hypo == "plane_strain":
            self.D = torch.tensor([[2 * mu + lam, lam, 0], [lam, 2 * mu + lam, 0], [0, 0, mu]], dtype=torch.float64,
                                  device=device)
        elif hypo == "plane_stress":
            self.D = E / (1 - nu ** 2) * torch.tensor([[1, nu, 0], [nu, 1, 0], [0, 0, (1 - nu) / 2]],
                                                       dtype=torch.float64, device=device)
        else:
            raise NotImplementedError("Only 3D, plane_stress, and plane_strain are supported.")
        self.cell_scale = cell_scale

    @property
    def lame_lambda(self):
        return self.lam

    @property
    def shear_modulus(self):
        return self.mu

    def elastic_matrix(self, bcs=None) -> torch.Tensor:
        D = self.D[None, None, ...]
        if self.cell_scale is not None:
            s = self.cell_scale.to(dtype=torch.float64, device=self.D.device)
            D = s[:, None, None, None] * D
        return D
