"""Time the oracle port against the reference FEALPy itself, stage by stage, on
the bench workload's law (P2 diffusion + mass on a jittered tetrahedral box,
lognormal per-cell coefficient, f = 1, u = 0, q = 4, Jacobi-PCG to 1e-10),
to show that the port's costs track the reference numpy path it restates.

Run where the reference checkout is importable (it does not exist on the GPU
hosts, where the bench times the port):

    python tests/golden/time_port_vs_reference.py /path/to/fealpy-checkout

Writes tests/golden/port_vs_reference_timing.json: per size, per stage, the
best of three single-process runs of each implementation and their ratio
(port / reference).  Stages: assembly (BilinearForm.assembly: local matrices
and the COO coalesce to CSR), dirichlet (DirichletBC.apply), pcg (cg with
the Jacobi preconditioner).
"""
import json
import os
import platform
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))


def best_of(fn, reps=3):
    best, out = None, None
    for _ in range(reps):
        t0 = time.perf_counter()
        out = fn()
        dt = time.perf_counter() - t0
        best = dt if best is None else min(best, dt)
    return best, out


def main(ref_root):
    sys.path.insert(0, HERE)
    sys.path.insert(0, ROOT)
    import refshim
    refshim.install(ref_root)
    from fealpy.backend import backend_manager as bm
    bm.set_backend("numpy")
    from fealpy.mesh import TetrahedronMesh
    from fealpy.functionspace import LagrangeFESpace
    from fealpy.fem import (BilinearForm, LinearForm, ScalarDiffusionIntegrator, ScalarMassIntegrator,
                            ScalarSourceIntegrator, DirichletBC)
    from fealpy.solver import cg
    from fealpy.sparse import CSRTensor
    from fealpy.decorator import cartesian
    from fealpy_gb300.workloads import diffusion_mass_tet_box
    from oracle import fem_oracle as O

    @cartesian
    def zero(p):
        return np.zeros(p.shape[:-1], dtype=np.float64)

    record = {"host": platform.processor() or platform.machine(), "python": platform.python_version(),
              "numpy": np.__version__, "threads": "default (BLAS threads the einsum)", "sizes": {}}
    for n in (16, 24):
        node, cell, kappa = diffusion_mass_tet_box(n)
        mesh = TetrahedronMesh(node, cell)
        space = LagrangeFESpace(mesh, p=2)
        space.cell_to_dof()

        def ref_asm():
            bf = BilinearForm(space)
            bf.add_integrator(ScalarDiffusionIntegrator(coef=kappa, q=4), ScalarMassIntegrator(coef=1.0, q=4))
            return bf.assembly()

        t_asm, A = best_of(ref_asm)
        lf = LinearForm(space)
        lf.add_integrator(ScalarSourceIntegrator(1.0, q=4))
        F = lf.assembly()
        bc = DirichletBC(space, gd=zero)
        t_bc, (A2, F2) = best_of(lambda: bc.apply(A, F.copy()))
        d = A2.diags()
        M = CSRTensor(d.crow, d.col, 1.0 / d.values, A2.shape)
        t_cg, (x, info) = best_of(lambda: cg(A2, F2, M=M, atol=1e-30, rtol=1e-10, returninfo=True))

        topo = O.construct(cell)
        c2d = O.cell_to_dof(cell, topo, node.shape[0], 2)
        N = O.n_global_dofs(cell, topo, node.shape[0], 2)

        def port_asm():
            K = O.diffusion_local(node, cell, 2, 4, kappa) + O.mass_local(node, cell, 2, 4, 1.0)
            return O.coalesce_to_csr(c2d, K, N)

        p_asm, (crow, col, val) = best_of(port_asm)
        Fp = O.source_vector(node, cell, c2d, 2, N, np.ones((cell.shape[0], 20)), 4)
        is_bd = O.boundary_dof_flag(cell, topo, c2d, 2, N)
        p_bc, ((bcrow, bcol, bval), Fb) = best_of(lambda: O.dirichlet_apply(crow, col, val, is_bd, Fp, np.zeros(N)))
        p_cg, (xp, pinfo) = best_of(lambda: O.jacobi_cg(bcrow, bcol, bval, Fb, atol=1e-30, rtol=1e-10))
        err = float(np.max(np.abs(xp - np.asarray(x))) / np.max(np.abs(np.asarray(x))))
        rec = {"gdof": int(N), "reference_s": {"assembly": t_asm, "dirichlet": t_bc, "pcg": t_cg},
               "port_s": {"assembly": p_asm, "dirichlet": p_bc, "pcg": p_cg},
               "port_over_reference": {"assembly": p_asm / t_asm, "dirichlet": p_bc / t_bc, "pcg": p_cg / t_cg,
                                       "total": (p_asm + p_bc + p_cg) / (t_asm + t_bc + t_cg)},
               "iterations": {"reference": int(info["niter"]), "port": int(pinfo["niter"])},
               "solution_rel_diff": err}
        record["sizes"][f"{n}^3"] = rec
        print(n, json.dumps(rec))
    with open(os.path.join(HERE, "port_vs_reference_timing.json"), "w") as fh:
        json.dump(record, fh, indent=1)


if __name__ == "__main__":
    args = [a for a in sys.argv[1:] if not a.startswith("--")]
    root = args[0] if args else os.environ.get("FEALPY_REFERENCE")
    if not root:
        raise SystemExit("usage: time_port_vs_reference.py /path/to/fealpy-checkout (or set FEALPY_REFERENCE)")
    main(root)
