"""Generate the golden fixtures of ``tests/golden/*.npz`` by running the reference
FEALPy (numpy backend, unmodified) through its public API.

Run in an environment where the reference checkout is importable:

    python tests/golden/make_golden.py /path/to/fealpy-checkout            # small cases, C1
    python tests/golden/make_golden.py --configs /path/to/fealpy-checkout  # mid-size config laws
    python tests/golden/make_golden.py --coef /path/to/fealpy-checkout     # (NC, NQ) coefficients
    python tests/golden/make_golden.py --batched /path/to/fealpy-checkout  # batched coefficients
    python tests/golden/make_golden.py --layouts /path/to/fealpy-checkout  # component-major elasticity
    python tests/golden/make_golden.py --regions /path/to/fealpy-checkout  # groups over different regions

The fixtures hold only inputs and outputs of the reference (meshes, dof maps,
local matrices, CSR matrices, vectors, iteration counts, quadrature tables and
the reference's own known-answer data), never its source.  Every random input
is seeded here and stored in the fixture, so tests read it back instead of
regenerating it.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def canonical(crow, col, val):
    """Sort the columns inside each row (the reference's tocsr may leave them in
    unstable-argsort order); returns (crow, col, val) in canonical order."""
    crow = np.asarray(crow, dtype=np.int64)
    col = np.asarray(col)
    val = np.asarray(val)
    row = np.repeat(np.arange(len(crow) - 1), np.diff(crow))
    order = np.lexsort((col, row))
    return crow, col[order].astype(np.int32), val[order]


def jitter(node, is_bd, h, amp, rng):
    out = node.copy()
    d = rng.uniform(-amp * h, amp * h, size=node.shape)
    out[~is_bd] += d[~is_bd]
    return out


def main(ref_root):
    sys.path.insert(0, HERE)
    import refshim
    refshim.install(ref_root)
    from fealpy.backend import backend_manager as bm
    bm.set_backend("numpy")
    from fealpy.mesh import TriangleMesh, TetrahedronMesh
    from fealpy.functionspace import LagrangeFESpace, TensorFunctionSpace
    from fealpy.fem import (BilinearForm, LinearForm, ScalarDiffusionIntegrator, ScalarMassIntegrator,
                            LinearElasticityIntegrator, ScalarSourceIntegrator, VectorSourceIntegrator, DirichletBC)
    from fealpy.solver import cg
    from fealpy.material import LinearElasticMaterial
    from fealpy.sparse import CSRTensor
    from fealpy.quadrature import TriangleQuadrature, TetrahedronQuadrature
    from fealpy.decorator import cartesian

    def jacobi(A):
        d = A.diags()
        return CSRTensor(d.crow, d.col, 1.0 / d.values, A.shape)

    # ------------------------------------------------------------------ C1
    mesh = TriangleMesh.from_box([0, 1, 0, 1], 64, 64)
    space = LagrangeFESpace(mesh, p=1)

    @cartesian
    def solution(p):
        return np.sin(np.pi * p[..., 0]) * np.sin(np.pi * p[..., 1])

    @cartesian
    def source(p):
        return 2 * np.pi ** 2 * solution(p)

    bf = BilinearForm(space)
    bf.add_integrator(ScalarDiffusionIntegrator(coef=1, q=3))
    A = bf.assembly()
    lf = LinearForm(space)
    lf.add_integrator(ScalarSourceIntegrator(source, q=3))
    F = lf.assembly()
    bc = DirichletBC(space, gd=solution)
    A2, F2 = bc.apply(A, F)
    uh, info = cg(A2, F2, M=jacobi(A2), atol=1e-30, rtol=1e-10, returninfo=True)
    c0, c1, c2 = canonical(A.crow, A.col, A.values)
    p0, p1, p2 = canonical(A2.crow, A2.col, A2.values)
    np.savez_compressed(os.path.join(HERE, "c1_poisson_tri_p1_64.npz"),
                        node=mesh.node, cell=mesh.cell, cell2dof=space.cell_to_dof(),
                        crow=c0, col=c1, val=c2, F=F, is_bd=bc.is_boundary_dof,
                        bc_crow=p0, bc_col=p1, bc_val=p2, bc_F=F2, uh=uh,
                        niter=np.int64(info["niter"]), residual=np.float64(info["residual"]))
    print("C1", A.nnz, A2.nnz, info["niter"])

    # ------------------------------------------- small jittered scalar cases
    rng = np.random.default_rng(20251204)
    cases = {}
    for tag, (kind, dims, p, q) in {
        "tri_p1": ("tri", (4, 3), 1, None), "tri_p2": ("tri", (4, 3), 2, None), "tri_p3": ("tri", (3, 3), 3, None),
        "tet_p1": ("tet", (3, 2, 2), 1, None), "tet_p2": ("tet", (2, 2, 2), 2, 4),
    }.items():
        if kind == "tri":
            m0 = TriangleMesh.from_box([0, 1, 0, 1], *dims)
            h = 1.0 / max(dims)
            node = jitter(m0.node, m0.boundary_node_flag(), h, 0.15, rng)
            mesh = TriangleMesh(node, m0.cell)
        else:
            m0 = TetrahedronMesh.from_box([0, 1, 0, 1, 0, 1], *dims)
            h = 1.0 / max(dims)
            node = jitter(m0.node, m0.boundary_node_flag(), h, 0.2, rng)
            mesh = TetrahedronMesh(node, m0.cell)
        space = LagrangeFESpace(mesh, p=p)
        NC = mesh.number_of_cells()
        kappa = np.exp(rng.normal(0.0, 1.0, NC))
        rho = 1.0
        di = ScalarDiffusionIntegrator(coef=kappa, q=q)
        mi = ScalarMassIntegrator(coef=rho, q=q)
        Kd = di.assembly(space)
        Km = mi.assembly(space)
        bf = BilinearForm(space)
        bf.add_integrator(ScalarDiffusionIntegrator(coef=kappa, q=q), ScalarMassIntegrator(coef=rho, q=q))
        A = bf.assembly()
        f = rng.normal(size=space.number_of_global_dofs())
        gdv = rng.normal(size=space.number_of_global_dofs())
        bc = DirichletBC(space, gd=gdv)
        A2, F2 = bc.apply(A, f.copy())
        uh, info = cg(A2, F2, M=jacobi(A2), atol=1e-30, rtol=1e-10, returninfo=True)
        c0, c1, c2 = canonical(A.crow, A.col, A.values)
        p0, p1, p2 = canonical(A2.crow, A2.col, A2.values)
        np.savez_compressed(os.path.join(HERE, f"small_{tag}.npz"),
                            node=mesh.node, cell=mesh.cell, p=np.int64(p), q=np.int64(-1 if q is None else q),
                            kappa=kappa, cell2dof=space.cell_to_dof(), edge=mesh.edge, face2cell=mesh.face2cell,
                            ipoints=space.interpolation_points(), K_diff=Kd, K_mass=Km,
                            crow=c0, col=c1, val=c2, f=f, gd=gdv, is_bd=bc.is_boundary_dof,
                            bc_crow=p0, bc_col=p1, bc_val=p2, bc_F=F2, uh=uh, niter=np.int64(info["niter"]),
                            residual=np.float64(info["residual"]))
        print(tag, A.nnz, A2.nnz, info["niter"])

    # ------------------------------------------------ P1 elasticity (tets)
    m0 = TetrahedronMesh.from_box([0, 1, 0, 1, 0, 1], 4, 3, 3)
    node = jitter(m0.node, m0.boundary_node_flag(), 0.25, 0.2, rng)
    mesh = TetrahedronMesh(node, m0.cell)
    NC = mesh.number_of_cells()
    scale = np.exp(rng.normal(0.0, 0.5, NC))

    class ScaledMaterial(LinearElasticMaterial):
        def __init__(self, s, **kw):
            super().__init__(**kw)
            self._s = s

        def elastic_matrix(self, bcs=None):
            return self._s[:, None, None, None] * super().elastic_matrix(bcs)

    mat = ScaledMaterial(scale, name="m", lame_lambda=1.0, shear_modulus=0.5)
    ts = TensorFunctionSpace(LagrangeFESpace(mesh, p=1), (-1, 3))
    KK = LinearElasticityIntegrator(mat, q=4).assembly(ts)
    bf = BilinearForm(ts)
    bf.add_integrator(LinearElasticityIntegrator(mat, q=4))
    A = bf.assembly()
    lf = LinearForm(ts)
    @cartesian
    def body_force(p):
        out = np.zeros(p.shape[:-1] + (3,), dtype=np.float64)
        out[..., 2] = -1.0
        return out

    lf.add_integrator(VectorSourceIntegrator(source=body_force, q=4))
    F = lf.assembly()

    @cartesian
    def clamp(p):
        return np.abs(p[..., 0]) < 1e-12

    @cartesian
    def zero_disp(p):
        return np.zeros(p.shape[:-1] + (3,), dtype=np.float64)

    bc = DirichletBC(ts, gd=zero_disp, threshold=clamp)
    A2, F2 = bc.apply(A, F)
    uh, info = cg(A2, F2, M=jacobi(A2), atol=1e-30, rtol=1e-10, returninfo=True)
    c0, c1, c2 = canonical(A.crow, A.col, A.values)
    p0, p1, p2 = canonical(A2.crow, A2.col, A2.values)
    np.savez_compressed(os.path.join(HERE, "small_elasticity_tet_p1.npz"),
                        node=mesh.node, cell=mesh.cell, scale=scale, cell2dof=ts.cell_to_dof(), KK=KK,
                        crow=c0, col=c1, val=c2, F=F, is_bd=bc.is_boundary_dof,
                        bc_crow=p0, bc_col=p1, bc_val=p2, bc_F=F2, uh=uh, niter=np.int64(info["niter"]))
    print("elasticity", A.nnz, A2.nnz, info["niter"])

    # ------------------------------------------- reference known answers
    sys.path.insert(0, os.path.join(ref_root, "test", "fem"))
    import scalar_diffusion_integrator_data as sdd
    import scalar_mass_integrator_data as smd
    dd = sdd.triangle_mesh_one_box[0]
    md = smd.triangle_mesh_one_box[0]
    np.savez_compressed(os.path.join(HERE, "reference_known_answers.npz"),
                        diffusion_args=np.asarray(dd["args"][0] + [dd["args"][1], dd["args"][2]], dtype=np.float64),
                        diffusion_cell_matrix=np.asarray(dd["assembly_cell_matrix"]),
                        mass_args=np.asarray(md["args"][0] + [md["args"][1], md["args"][2]], dtype=np.float64),
                        mass_cell_matrix=np.asarray(md["assembly_cell_matrix"]))

    # ------------------------------------------------- quadrature tables
    tabs = {}
    for q in range(1, 10):
        b, w = TriangleQuadrature(q).get_quadrature_points_and_weights()
        tabs[f"tri_{q}_bcs"], tabs[f"tri_{q}_ws"] = np.asarray(b), np.asarray(w)
    for q in range(1, 8):
        b, w = TetrahedronQuadrature(q).get_quadrature_points_and_weights()
        tabs[f"tet_{q}_bcs"], tabs[f"tet_{q}_ws"] = np.asarray(b), np.asarray(w)
    np.savez_compressed(os.path.join(HERE, "quadrature_tables.npz"), **tabs)
    print("done")


def config_cases(ref_root):
    """Mid-size cases of the benchmark configurations' laws, run through the
    reference (numpy backend) with the same seeded generators as the GPU
    workloads (``fealpy_gb300.workloads``):

    * ``cfg_c2_tet_p2_8``: P2 diffusion + mass on the 8^3 tetrahedral box,
      interior nodes jittered by U(+-0.2h), lognormal(0, 1) per-cell diffusion,
      reaction 1, f = 1, u = 0, q = 4 (4,913 dofs, 3,375 interior);
    * ``cfg_c3_tri_p3_32``: P3 diffusion on the 32x32 triangle box, jitter
      U(+-0.15h), a 4x4 checkerboard coefficient log-uniform in [0.1, 10],
      q = p + 3, f = 1, u = 0 (9,409 dofs);
    * ``cfg_c5_elasticity_8``: P1 vector elasticity on the 8^3 tetrahedral box,
      lambda = 1, mu = 0.5 scaled per cell by lognormal(0, 0.5), clamped at
      x = 0, body force (0, 0, -1), q = 4 (2,187 dofs).

    Each fixture holds the inputs and the reference's pre- and post-Dirichlet
    CSR (canonical order), right-hand sides, Jacobi-PCG solution (rtol 1e-10)
    and iteration count."""
    sys.path.insert(0, HERE)
    sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
    import refshim
    refshim.install(ref_root)
    from fealpy.backend import backend_manager as bm
    bm.set_backend("numpy")
    from fealpy.mesh import TriangleMesh, TetrahedronMesh
    from fealpy.functionspace import LagrangeFESpace, TensorFunctionSpace
    from fealpy.fem import (BilinearForm, LinearForm, ScalarDiffusionIntegrator, ScalarMassIntegrator,
                            LinearElasticityIntegrator, ScalarSourceIntegrator, VectorSourceIntegrator, DirichletBC)
    from fealpy.solver import cg
    from fealpy.material import LinearElasticMaterial
    from fealpy.sparse import CSRTensor
    from fealpy.decorator import cartesian
    from fealpy_gb300 import workloads as W

    def jacobi(A):
        d = A.diags()
        return CSRTensor(d.crow, d.col, 1.0 / d.values, A.shape)

    @cartesian
    def zero(p):
        return np.zeros(p.shape[:-1], dtype=np.float64)

    def scalar_case(name, mesh, p, q, integrators, extra):
        space = LagrangeFESpace(mesh, p=p)
        bf = BilinearForm(space)
        bf.add_integrator(*integrators)
        A = bf.assembly()
        lf = LinearForm(space)
        lf.add_integrator(ScalarSourceIntegrator(1.0, q=q))
        F = lf.assembly()
        bc = DirichletBC(space, gd=zero)
        A2, F2 = bc.apply(A, F.copy())
        uh, info = cg(A2, F2, M=jacobi(A2), atol=1e-30, rtol=1e-10, returninfo=True)
        c0, c1, c2 = canonical(A.crow, A.col, A.values)
        p0, p1, p2 = canonical(A2.crow, A2.col, A2.values)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), node=mesh.node, cell=mesh.cell, p=np.int64(p),
                            q=np.int64(q), cell2dof=space.cell_to_dof(), crow=c0, col=c1, val=c2, F=F,
                            is_bd=bc.is_boundary_dof, bc_crow=p0, bc_col=p1, bc_val=p2, bc_F=F2, uh=uh,
                            niter=np.int64(info["niter"]), **extra)
        print(name, space.number_of_global_dofs(), A.nnz, A2.nnz, info["niter"])

    # C2 law: the bench generator at 8^3
    node, cell, kappa = W.diffusion_mass_tet_box(8)
    mesh = TetrahedronMesh(node, cell)
    scalar_case("cfg_c2_tet_p2_8", mesh, 2, 4,
                [ScalarDiffusionIntegrator(coef=kappa, q=4), ScalarMassIntegrator(coef=1.0, q=4)],
                {"kappa": kappa})

    # C3 law: a P3 mesh of the batched generator's law at nx = 32
    rng = np.random.default_rng(32)
    values = np.exp(rng.uniform(np.log(0.1), np.log(10.0), size=16))
    node, cell = W.tri_box_arrays(32, 32)
    node = W.jitter_interior(node, 1.0 / 32, 0.15, seed=int(rng.integers(0, 2 ** 31 - 1)))
    kappa = W.checkerboard_cells(node, cell, values)
    mesh = TriangleMesh(node, cell)
    scalar_case("cfg_c3_tri_p3_32", mesh, 3, 6, [ScalarDiffusionIntegrator(coef=kappa, q=6)], {"kappa": kappa})

    # C5 law: the elasticity generator at 8^3
    node, cell, scale = W.elasticity_tet_box(8)
    mesh = TetrahedronMesh(node, cell)

    class ScaledMaterial(LinearElasticMaterial):
        def __init__(self, s, **kw):
            super().__init__(**kw)
            self._s = s

        def elastic_matrix(self, bcs=None):
            return self._s[:, None, None, None] * super().elastic_matrix(bcs)

    mat = ScaledMaterial(scale, name="m", lame_lambda=1.0, shear_modulus=0.5)
    ts = TensorFunctionSpace(LagrangeFESpace(mesh, p=1), (-1, 3))
    bf = BilinearForm(ts)
    bf.add_integrator(LinearElasticityIntegrator(mat, q=4))
    A = bf.assembly()

    @cartesian
    def body_force(p):
        out = np.zeros(p.shape[:-1] + (3,), dtype=np.float64)
        out[..., 2] = -1.0
        return out

    @cartesian
    def clamp(p):
        return np.abs(p[..., 0]) < 1e-12

    @cartesian
    def zero_disp(p):
        return np.zeros(p.shape[:-1] + (3,), dtype=np.float64)

    lf = LinearForm(ts)
    lf.add_integrator(VectorSourceIntegrator(source=body_force, q=4))
    F = lf.assembly()
    bc = DirichletBC(ts, gd=zero_disp, threshold=clamp)
    A2, F2 = bc.apply(A, F)
    uh, info = cg(A2, F2, M=jacobi(A2), atol=1e-30, rtol=1e-10, returninfo=True)
    c0, c1, c2 = canonical(A.crow, A.col, A.values)
    p0, p1, p2 = canonical(A2.crow, A2.col, A2.values)
    np.savez_compressed(os.path.join(HERE, "cfg_c5_elasticity_8.npz"), node=mesh.node, cell=mesh.cell, scale=scale,
                        cell2dof=ts.cell_to_dof(), crow=c0, col=c1, val=c2, F=F, is_bd=bc.is_boundary_dof,
                        bc_crow=p0, bc_col=p1, bc_val=p2, bc_F=F2, uh=uh, niter=np.int64(info["niter"]))
    print("cfg_c5_elasticity_8", ts.number_of_global_dofs(), A.nnz, A2.nnz, info["niter"])


def coef_cases(ref_root):
    """Coefficients that vary inside a cell (``fealpy/utils/utils.py:21-53``
    hands (NC, NQ) values to ``bilinear_integral``): per seeded jittered mesh,
    a diffusion coefficient given as a cartesian function (1 + x^2 + y z or
    1 + x^2 + y in 2-D) and a mass coefficient given as an (NC, NQ) array
    (uniform in [0.5, 2]), on P2 triangles (4x3 box) and P2 tetrahedra (2^3
    box), q = 4.  Each fixture ``coefq_<tag>`` holds the inputs, the
    reference's local matrices of both integrators and its CSR of their sum
    (canonical order)."""
    sys.path.insert(0, HERE)
    import refshim
    refshim.install(ref_root)
    from fealpy.backend import backend_manager as bm
    bm.set_backend("numpy")
    from fealpy.mesh import TriangleMesh, TetrahedronMesh
    from fealpy.functionspace import LagrangeFESpace
    from fealpy.fem import BilinearForm, ScalarDiffusionIntegrator, ScalarMassIntegrator
    from fealpy.decorator import cartesian

    @cartesian
    def kappa2(p):
        return 1.0 + p[..., 0] ** 2 + p[..., 1]

    @cartesian
    def kappa3(p):
        return 1.0 + p[..., 0] ** 2 + p[..., 1] * p[..., 2]

    rng = np.random.default_rng(20261204)
    for tag, kind, dims, p, q in (("tri_p2", "tri", (4, 3), 2, 4), ("tet_p2", "tet", (2, 2, 2), 2, 4)):
        if kind == "tri":
            m0 = TriangleMesh.from_box([0, 1, 0, 1], *dims)
            node = jitter(m0.node, m0.boundary_node_flag(), 1.0 / max(dims), 0.15, rng)
            mesh, kappa = TriangleMesh(node, m0.cell), kappa2
        else:
            m0 = TetrahedronMesh.from_box([0, 1, 0, 1, 0, 1], *dims)
            node = jitter(m0.node, m0.boundary_node_flag(), 1.0 / max(dims), 0.2, rng)
            mesh, kappa = TetrahedronMesh(node, m0.cell), kappa3
        space = LagrangeFESpace(mesh, p=p)
        NC = mesh.number_of_cells()
        NQ = mesh.quadrature_formula(q).number_of_quadrature_points()
        rho = rng.uniform(0.5, 2.0, size=(NC, NQ))
        Kd = ScalarDiffusionIntegrator(coef=kappa, q=q).assembly(space)
        Km = ScalarMassIntegrator(coef=rho, q=q).assembly(space)
        bf = BilinearForm(space)
        bf.add_integrator(ScalarDiffusionIntegrator(coef=kappa, q=q), ScalarMassIntegrator(coef=rho, q=q))
        A = bf.assembly()
        c0, c1, c2 = canonical(A.crow, A.col, A.values)
        np.savez_compressed(os.path.join(HERE, f"coefq_{tag}.npz"), node=mesh.node, cell=mesh.cell, p=np.int64(p),
                            q=np.int64(q), rho=rho, K_diff=Kd, K_mass=Km, crow=c0, col=c1, val=c2)
        print("coefq", tag, NC, NQ, A.nnz)
        if tag == "tet_p2":
            # several right-hand sides of the last matrix (fealpy/solver/cg.py:60-123),
            # with and without the Jacobi preconditioner
            from fealpy.solver import cg
            from fealpy.sparse import CSRTensor
            Bm = rng.normal(size=(A.shape[0], 3))
            d = A.diags()
            Mj = CSRTensor(d.crow, d.col, 1.0 / d.values, A.shape)
            xj, ij = cg(A, Bm.copy(), M=Mj, atol=1e-30, rtol=1e-10, returninfo=True)
            xp, ip = cg(A, Bm.copy(), atol=1e-30, rtol=1e-10, returninfo=True)
            np.savez_compressed(os.path.join(HERE, "cg_multi_rhs.npz"), crow=c0, col=c1, val=c2, B=Bm,
                                x_jacobi=xj, niter_jacobi=np.int64(ij["niter"]),
                                residual_jacobi=np.float64(ij["residual"]), x_plain=xp,
                                niter_plain=np.int64(ip["niter"]), residual_plain=np.float64(ip["residual"]))
            print("cg multi rhs", ij["niter"], ip["niter"])

    # integration over a sub-region (fealpy/fem/integrator.py:141-162): the
    # cells whose centroid has x < 0.55 (region= for diffusion, index= for
    # mass) on P2 triangles.  (A ScalarSourceIntegrator with region= and a
    # LinearElasticityIntegrator with index= do not run in the reference: the
    # former's to_global_dof ignores the region, the latter sizes its local
    # matrices by all cells.)

    m0 = TriangleMesh.from_box([0, 1, 0, 1], 5, 4)
    mesh = TriangleMesh(jitter(m0.node, m0.boundary_node_flag(), 0.2, 0.15, rng), m0.cell)
    reg = np.nonzero(mesh.entity_barycenter("cell")[:, 0] < 0.55)[0]
    space = LagrangeFESpace(mesh, p=2)
    bf = BilinearForm(space)
    bf.add_integrator(ScalarDiffusionIntegrator(coef=kappa2, q=4, region=reg),
                      ScalarMassIntegrator(coef=2.0, q=4, index=reg))
    A = bf.assembly()
    c0, c1, c2 = canonical(A.crow, A.col, A.values)
    np.savez_compressed(os.path.join(HERE, "region_cases.npz"), node=mesh.node, cell=mesh.cell, region=reg,
                        crow=c0, col=c1, val=c2)
    print("region", len(reg), mesh.number_of_cells(), A.nnz)


def batched_cases(ref_root):
    """A form with batched coefficients (``fealpy/fem/bilinear_form.py:46-75``,
    ``fealpy/functional.py:68-106``): on P2 triangles (3x3 box, jittered),
    batch size 3, a diffusion coefficient per member and cell (B, NC)
    (lognormal) in one group and a mass coefficient per member (B,) in
    another (the reference stacks groups without a batch over the batch, and
    refuses batched and unbatched integrators in one group), q = 4.  The
    fixture ``batched_tri_p2`` holds the inputs, the reference's batched
    local diffusion matrices (B, NC, 6, 6), its CSR with values (B, nnz) in
    canonical order (the numpy backend has no product of a batched matrix:
    ``fealpy/backend/numpy_backend.py:181-199``), and the batched right-hand
    side (B, n) of a source given per member and cell."""
    sys.path.insert(0, HERE)
    import refshim
    refshim.install(ref_root)
    from fealpy.backend import backend_manager as bm
    bm.set_backend("numpy")
    from fealpy.mesh import TriangleMesh
    from fealpy.functionspace import LagrangeFESpace
    from fealpy.fem import BilinearForm, ScalarDiffusionIntegrator, ScalarMassIntegrator

    rng = np.random.default_rng(20261205)
    m0 = TriangleMesh.from_box([0, 1, 0, 1], 3, 3)
    mesh = TriangleMesh(jitter(m0.node, m0.boundary_node_flag(), 1.0 / 3, 0.15, rng), m0.cell)
    space = LagrangeFESpace(mesh, p=2)
    B, NC = 3, mesh.number_of_cells()
    kappa = np.exp(rng.normal(size=(B, NC)))
    rho = rng.uniform(0.5, 2.0, size=B)
    Kd = ScalarDiffusionIntegrator(coef=kappa, q=4, batched=True).assembly(space)
    bf = BilinearForm(space, batch_size=B)
    bf.add_integrator(ScalarDiffusionIntegrator(coef=kappa, q=4, batched=True))
    bf.add_integrator(ScalarMassIntegrator(coef=rho, q=4, batched=True))
    A = bf.assembly()
    crow = np.asarray(A.crow, dtype=np.int64)
    row = np.repeat(np.arange(len(crow) - 1), np.diff(crow))
    order = np.lexsort((np.asarray(A.col), row))
    # batched right-hand side: a source per member and cell (B, NC)
    from fealpy.fem import LinearForm, ScalarSourceIntegrator
    fsrc = rng.normal(size=(B, NC))
    lf = LinearForm(space, batch_size=B)
    lf.add_integrator(ScalarSourceIntegrator(source=fsrc, q=4, batched=True))
    Fb = lf.assembly()
    np.savez_compressed(os.path.join(HERE, "batched_tri_p2.npz"), node=mesh.node, cell=mesh.cell, kappa=kappa,
                        rho=rho, K_diff=Kd, crow=crow, col=np.asarray(A.col)[order].astype(np.int32),
                        val=np.asarray(A.values)[:, order], source=fsrc, F=np.asarray(Fb))
    print("batched", B, NC, A.nnz, np.asarray(A.values).shape, np.asarray(Fb).shape)


def layout_cases(ref_root):
    """P1 elasticity in the component-major layout (``TensorFunctionSpace``
    ``shape=(3, -1)``, ``fealpy/functionspace/tensor_space.py:29-31``) on the
    mesh, per-cell material scale and q of ``small_elasticity_tet_p1``: the
    reference's local matrices and CSR (canonical order) in that layout."""
    sys.path.insert(0, HERE)
    import refshim
    refshim.install(ref_root)
    from fealpy.backend import backend_manager as bm
    bm.set_backend("numpy")
    from fealpy.mesh import TetrahedronMesh
    from fealpy.functionspace import LagrangeFESpace, TensorFunctionSpace
    from fealpy.material import LinearElasticMaterial
    from fealpy.fem import BilinearForm, LinearElasticityIntegrator

    z = np.load(os.path.join(HERE, "small_elasticity_tet_p1.npz"))
    mesh = TetrahedronMesh(z["node"], z["cell"])
    scale = z["scale"]

    class ScaledMaterial(LinearElasticMaterial):
        def __init__(self, s, **kw):
            super().__init__(**kw)
            self._s = s

        def elastic_matrix(self, bcs=None):
            return self._s[:, None, None, None] * super().elastic_matrix(bcs)

    mat = ScaledMaterial(scale, name="m", lame_lambda=1.0, shear_modulus=0.5)
    ts = TensorFunctionSpace(LagrangeFESpace(mesh, p=1), (3, -1))
    KK = LinearElasticityIntegrator(mat, q=4).assembly(ts)
    bf = BilinearForm(ts)
    bf.add_integrator(LinearElasticityIntegrator(mat, q=4))
    A = bf.assembly()
    c0, c1, c2 = canonical(A.crow, A.col, A.values)
    np.savez_compressed(os.path.join(HERE, "elasticity_component_major.npz"), cell2dof=ts.cell_to_dof(), KK=KK,
                        crow=c0, col=c1, val=c2)
    print("component-major elasticity", A.shape, A.nnz)


def multi_region_cases(ref_root):
    """Integrator groups over different regions of one form
    (``fealpy/fem/integrator.py:141-162``, ``fealpy/fem/form.py:92-122``): on
    P2 triangles (5x4 box, jittered), a diffusion group with a cartesian
    coefficient over the cells with centroid x < 0.55, a diffusion group
    (coefficient 3) over the cells with centroid x > 0.35 (the regions
    overlap) and a mass group (coefficient 2, ``index=``; the reference's
    mass integrator takes no ``region``) over the same cells, q = 4.  The fixture ``multi_region_tri_p2`` holds
    the inputs and the reference's CSR (canonical order)."""
    sys.path.insert(0, HERE)
    import refshim
    refshim.install(ref_root)
    from fealpy.backend import backend_manager as bm
    bm.set_backend("numpy")
    from fealpy.mesh import TriangleMesh
    from fealpy.functionspace import LagrangeFESpace
    from fealpy.fem import BilinearForm, ScalarDiffusionIntegrator, ScalarMassIntegrator
    from fealpy.decorator import cartesian

    @cartesian
    def kappa(p):
        return 1.0 + p[..., 0] ** 2 + p[..., 1]

    rng = np.random.default_rng(20261206)
    m0 = TriangleMesh.from_box([0, 1, 0, 1], 5, 4)
    mesh = TriangleMesh(jitter(m0.node, m0.boundary_node_flag(), 0.2, 0.15, rng), m0.cell)
    xc = mesh.entity_barycenter("cell")[:, 0]
    reg1, reg2 = np.nonzero(xc < 0.55)[0], np.nonzero(xc > 0.35)[0]
    space = LagrangeFESpace(mesh, p=2)
    bf = BilinearForm(space)
    bf.add_integrator(ScalarDiffusionIntegrator(coef=kappa, q=4), region=reg1)
    bf.add_integrator(ScalarDiffusionIntegrator(coef=3.0, q=4), region=reg2)
    bf.add_integrator(ScalarMassIntegrator(coef=2.0, q=4, index=reg2))
    A = bf.assembly()
    c0, c1, c2 = canonical(A.crow, A.col, A.values)
    np.savez_compressed(os.path.join(HERE, "multi_region_tri_p2.npz"), node=mesh.node, cell=mesh.cell, reg1=reg1,
                        reg2=reg2, crow=c0, col=c1, val=c2)
    print("multi-region", len(reg1), len(reg2), mesh.number_of_cells(), A.nnz)


def _reference_root(argv):
    root = argv[0] if argv else os.environ.get("FEALPY_REFERENCE")
    if not root:
        raise SystemExit("usage: make_golden.py [--configs] /path/to/fealpy-checkout "
                         "(or set FEALPY_REFERENCE)")
    return root


if __name__ == "__main__":
    args = [a for a in sys.argv[1:] if not a.startswith("--")]
    if "--configs" in sys.argv[1:]:
        config_cases(_reference_root(args))
    elif "--coef" in sys.argv[1:]:
        coef_cases(_reference_root(args))
    elif "--batched" in sys.argv[1:]:
        batched_cases(_reference_root(args))
    elif "--layouts" in sys.argv[1:]:
        layout_cases(_reference_root(args))
    elif "--regions" in sys.argv[1:]:
        multi_region_cases(_reference_root(args))
    else:
        main(_reference_root(args))
