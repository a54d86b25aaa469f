"""Pin the CPU oracle against fixtures produced by running the reference FEALPy
(tests/golden/make_golden.py).  No GPU needed."""
import os

import numpy as np
import pytest

from oracle import fem_oracle as O
from fealpy_gb300.quadrature import simplex_quadrature
from fealpy_gb300 import simplex as sx

RTOL = 1e-12


def load(golden_dir, name):
    return np.load(os.path.join(golden_dir, name))


def rel_err(a, b):
    scale = max(np.max(np.abs(b)), 1e-300)
    return np.max(np.abs(np.asarray(a) - np.asarray(b))) / scale


def test_quadrature_tables_match_reference(golden_dir):
    z = load(golden_dir, "quadrature_tables.npz")
    for TD, name, qs in ((2, "tri", range(1, 10)), (3, "tet", range(1, 8))):
        for q in qs:
            b, w = simplex_quadrature(TD, q)
            rb, rw = z[f"{name}_{q}_bcs"], z[f"{name}_{q}_ws"]
            assert b.shape == rb.shape, (name, q)
            # the same points in the same order (per-point coefficient arrays
            # are indexed in FEALPy's order)
            assert np.max(np.abs(b - rb)) < 2e-15, (name, q)
            assert np.max(np.abs(w - rw)) < 2e-15, (name, q)


def test_multi_index_and_basis_agree():
    for TD in (2, 3):
        for p in (1, 2, 3, 4):
            assert np.array_equal(O.multi_index_matrix(p, TD), sx.multi_index_matrix(p, TD))
            bcs, _ = simplex_quadrature(TD, 4)
            assert np.allclose(O.simplex_shape_function(bcs, p), sx.shape_function(bcs, p), atol=1e-13)
            assert np.allclose(O.simplex_grad_shape_function(bcs, p), sx.grad_shape_function(bcs, p), atol=1e-12)


def test_reference_known_answers(golden_dir):
    """test/fem/test_scalar_{diffusion,mass}_integrator.py: P2 on the 1x1 box, q=3."""
    z = load(golden_dir, "reference_known_answers.npz")
    node, cell = O.tri_from_box([0, 1, 0, 1], 1, 1)
    topo = O.construct(cell)
    K = O.diffusion_local(node, cell, 2, 3)
    M = O.mass_local(node, cell, 2, 3)
    np.testing.assert_array_almost_equal(K, z["diffusion_cell_matrix"], decimal=6)
    np.testing.assert_array_almost_equal(M, z["mass_cell_matrix"], decimal=6)


@pytest.mark.parametrize("tag", ["tri_p1", "tri_p2", "tri_p3", "tet_p1", "tet_p2"])
def test_small_cases(golden_dir, tag):
    z = load(golden_dir, f"small_{tag}.npz")
    node, cell, p = z["node"], z["cell"], int(z["p"])
    q = None if int(z["q"]) < 0 else int(z["q"])
    topo = O.construct(cell)
    assert np.array_equal(topo["edge"], z["edge"])
    assert np.array_equal(topo["face2cell"], z["face2cell"])
    NN = node.shape[0]
    c2d = O.cell_to_dof(cell, topo, NN, p)
    assert np.array_equal(c2d, z["cell2dof"])
    n = O.n_global_dofs(cell, topo, NN, p)
    Kd = O.diffusion_local(node, cell, p, q, z["kappa"])
    Km = O.mass_local(node, cell, p, q, 1.0)
    assert rel_err(Kd, z["K_diff"]) < RTOL
    assert rel_err(Km, z["K_mass"]) < RTOL
    crow, col, val = O.coalesce_to_csr(c2d, Kd + Km, n)
    assert np.array_equal(crow, z["crow"]) and np.array_equal(col, z["col"])
    assert rel_err(val, z["val"]) < RTOL
    is_bd = O.boundary_dof_flag(cell, topo, c2d, p, n)
    assert np.array_equal(is_bd, z["is_bd"])
    uh = np.zeros(n)
    uh[is_bd] = z["gd"][is_bd]
    (bcrow, bcol, bval), F = O.dirichlet_apply(crow, col, val, is_bd, z["f"], uh)
    assert np.array_equal(bcrow, z["bc_crow"]) and np.array_equal(bcol, z["bc_col"])
    assert rel_err(bval, z["bc_val"]) < RTOL
    assert rel_err(F, z["bc_F"]) < RTOL
    x, info = O.jacobi_cg(bcrow, bcol, bval, F, atol=1e-30, rtol=1e-10)
    assert abs(info["niter"] - int(z["niter"])) <= 1
    assert rel_err(x, z["uh"]) < 1e-8


def test_c1_full_pipeline(golden_dir):
    z = load(golden_dir, "c1_poisson_tri_p1_64.npz")
    node, cell = O.tri_from_box([0, 1, 0, 1], 64, 64)
    assert np.array_equal(node, z["node"]) and np.array_equal(cell, z["cell"])

    def u(p):
        return np.sin(np.pi * p[..., 0]) * np.sin(np.pi * p[..., 1])

    topo = O.construct(cell)
    c2d = O.cell_to_dof(cell, topo, node.shape[0], 1)
    n = node.shape[0]
    gd = u(node)
    out = O.poisson_pipeline(node, cell, 1, kappa=None, q=3, f_at_q=lambda x: 2 * np.pi ** 2 * u(x), gd_dofs=gd)
    assert np.array_equal(out["crow"], z["crow"]) and np.array_equal(out["col"], z["col"])
    assert rel_err(out["val"], z["val"]) < RTOL
    assert rel_err(out["F"], z["F"]) < RTOL
    assert np.array_equal(out["is_bd"], z["is_bd"])
    assert np.array_equal(out["bc_crow"], z["bc_crow"]) and np.array_equal(out["bc_col"], z["bc_col"])
    assert rel_err(out["bc_val"], z["bc_val"]) < RTOL
    assert rel_err(out["bc_F"], z["bc_F"]) < RTOL
    assert out["info"]["niter"] == int(z["niter"])
    assert rel_err(out["x"], z["uh"]) < 1e-9


def test_elasticity_case(golden_dir):
    z = load(golden_dir, "small_elasticity_tet_p1.npz")
    node, cell, s = z["node"], z["cell"], z["scale"]
    KK = O.elasticity_local(node, cell, 1.0 * s, 0.5 * s, q=4)
    assert rel_err(KK, z["KK"]) < RTOL
    c2d = O.vector_elasticity_dofs(cell)
    assert np.array_equal(c2d, z["cell2dof"])
    n = 3 * node.shape[0]
    crow, col, val = O.coalesce_to_csr(c2d, KK, n)
    assert np.array_equal(crow, z["crow"]) and np.array_equal(col, z["col"])
    assert rel_err(val, z["val"]) < RTOL
    is_bd = z["is_bd"]
    (bcrow, bcol, bval), F = O.dirichlet_apply(crow, col, val, is_bd, z["F"], np.zeros(n))
    assert np.array_equal(bcrow, z["bc_crow"]) and np.array_equal(bcol, z["bc_col"])
    assert rel_err(bval, z["bc_val"]) < RTOL
    assert rel_err(F, z["bc_F"]) < RTOL
    x, info = O.jacobi_cg(bcrow, bcol, bval, F, atol=1e-30, rtol=1e-10)
    assert abs(info["niter"] - int(z["niter"])) <= 1
    assert rel_err(x, z["uh"]) < 1e-8


@pytest.mark.parametrize("name", ["cfg_c2_tet_p2_8", "cfg_c3_tri_p3_32"])
def test_config_law_scalar_cases(golden_dir, name):
    """Mid-size cases of the C2 (P2 tet 8^3, diffusion + mass) and C3 (P3
    triangles 32x32, checkerboard coefficient) laws: the oracle's full
    pipeline against the reference's outputs."""
    z = load(golden_dir, name + ".npz")
    node, cell, p, q = z["node"], z["cell"], int(z["p"]), int(z["q"])
    rho = 1.0 if cell.shape[1] == 4 else None
    out = O.poisson_pipeline(node, cell, p, kappa=z["kappa"], rho=rho, q=q, rtol=1e-10)
    assert np.array_equal(out["c2d"], z["cell2dof"])
    assert np.array_equal(out["crow"], z["crow"]) and np.array_equal(out["col"], z["col"])
    assert rel_err(out["val"], z["val"]) < RTOL
    assert rel_err(out["F"], z["F"]) < RTOL
    assert np.array_equal(out["is_bd"], z["is_bd"])
    assert np.array_equal(out["bc_crow"], z["bc_crow"]) and np.array_equal(out["bc_col"], z["bc_col"])
    assert rel_err(out["bc_val"], z["bc_val"]) < RTOL
    assert rel_err(out["bc_F"], z["bc_F"]) < RTOL
    assert abs(out["info"]["niter"] - int(z["niter"])) <= 1
    assert rel_err(out["x"], z["uh"]) < 1e-9


def test_config_law_elasticity_case(golden_dir):
    """Mid-size case of the C5 law (P1 elasticity 8^3, per-cell scaled
    material, x = 0 clamp, body force -z): the oracle's pipeline against the
    reference's outputs."""
    z = load(golden_dir, "cfg_c5_elasticity_8.npz")
    node, cell, s = z["node"], z["cell"], z["scale"]
    out = O.elasticity_pipeline(node, cell, 1.0 * s, 0.5 * s, q=4, clamp=lambda x: np.abs(x[..., 0]) < 1e-12)
    assert np.array_equal(out["c2d"], z["cell2dof"])
    assert np.array_equal(out["crow"], z["crow"]) and np.array_equal(out["col"], z["col"])
    assert rel_err(out["val"], z["val"]) < RTOL
    assert rel_err(out["F"], z["F"]) < RTOL
    assert np.array_equal(out["is_bd"], z["is_bd"])
    assert np.array_equal(out["bc_crow"], z["bc_crow"]) and np.array_equal(out["bc_col"], z["bc_col"])
    assert rel_err(out["bc_val"], z["bc_val"]) < RTOL
    assert rel_err(out["bc_F"], z["bc_F"]) < RTOL
    assert abs(out["info"]["niter"] - int(z["niter"])) <= 1
    assert rel_err(out["x"], z["uh"]) < 1e-9


def test_batched_form_case(golden_dir):
    """The oracle, member by member, against the reference's batched form:
    a batch member's matrix is the unbatched assembly with that member's
    coefficients (``fealpy/functional.py:68-106``), the batched right-hand
    side likewise."""
    z = load(golden_dir, "batched_tri_p2.npz")
    node, cell = z["node"], z["cell"]
    topo = O.construct(cell)
    NN = node.shape[0]
    c2d = O.cell_to_dof(cell, topo, NN, 2)
    n = O.n_global_dofs(cell, topo, NN, 2)
    Kd = np.stack([O.diffusion_local(node, cell, 2, 4, k) for k in z["kappa"]])
    assert rel_err(Kd, z["K_diff"]) < RTOL
    NQ = O._rule(2, 2, 4)[1].shape[0]
    for b in range(z["kappa"].shape[0]):
        K = O.diffusion_local(node, cell, 2, 4, z["kappa"][b]) + O.mass_local(node, cell, 2, 4, z["rho"][b])
        crow, col, val = O.coalesce_to_csr(c2d, K, n)
        assert np.array_equal(crow, z["crow"]) and np.array_equal(col, z["col"])
        assert rel_err(val, z["val"][b]) < RTOL
        fq = np.repeat(z["source"][b][:, None], NQ, axis=1)
        assert rel_err(O.source_vector(node, cell, c2d, 2, n, fq, q=4), z["F"][b]) < RTOL


def test_elasticity_component_major_case(golden_dir):
    """The oracle's interleaved elasticity matrix with rows and columns
    renumbered component-major (dof comp NN + node) against the reference's
    shape=(3, -1) matrix."""
    z0 = load(golden_dir, "small_elasticity_tet_p1.npz")
    z = load(golden_dir, "elasticity_component_major.npz")
    node, cell, s = z0["node"], z0["cell"], z0["scale"]
    NN = node.shape[0]
    KK = O.elasticity_local(node, cell, 1.0 * s, 0.5 * s, q=4)
    crow, col, val = O.coalesce_to_csr(O.vector_elasticity_dofs(cell), KK, 3 * NN)
    new_of = (np.arange(3 * NN) % 3) * NN + np.arange(3 * NN) // 3      # interleaved -> component-major
    c2d_cm = new_of[O.vector_elasticity_dofs(cell)]
    assert np.array_equal(np.sort(c2d_cm, axis=1), np.sort(z["cell2dof"], axis=1))
    rows = new_of[np.repeat(np.arange(3 * NN), np.diff(crow))]
    cols = new_of[col]
    order = np.lexsort((cols, rows))
    crow_cm = np.concatenate([[0], np.cumsum(np.bincount(rows, minlength=3 * NN))])
    assert np.array_equal(crow_cm, z["crow"]) and np.array_equal(cols[order], z["col"])
    assert rel_err(val[order], z["val"]) < RTOL
