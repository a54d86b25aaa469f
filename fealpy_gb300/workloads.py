"""Seeded synthetic inputs for the benchmark configurations (no dataset involved).

All random draws use numpy's ``default_rng`` with fixed seeds so that the GPU
path and the CPU oracle receive bit-identical meshes and coefficients.

* ``poisson_tri_box``: P1 Poisson on ``TriangleMesh.from_box([0,1]^2, n, n)``
  (the 64x64 case is the reference's CPU-runnable configuration).
* ``diffusion_mass_tet_box``: P2 diffusion + mass on a ``TetrahedronMesh``
  box of n^3 cubes (6 tetrahedra each) with interior nodes jittered uniformly
  by +-0.2h (``default_rng(1)``), a lognormal(0, 1) per-cell diffusion
  coefficient (``default_rng(0)``), reaction coefficient 1, f = 1, u = 0 on
  the boundary, quadrature index 4.
* ``elasticity_tet_box``: P1 vector elasticity on an n^3 tetrahedral box,
  lambda = 1, mu = 0.5, both scaled per cell by exp(N(0, 0.5))
  (``default_rng(4)``), clamped at x = 0, body force (0, 0, -1).
* ``batched_tri_meshes``: 256 independent Poisson problems on
  ``TriangleMesh.from_box([0,1]^2, nx, nx)`` with nx = round(exp(U(ln 16,
  ln 512))), degree p ~ U{1, 2, 3}, interior nodes jittered by U(+-0.15h), a
  coefficient piecewise constant on a 4x4 checkerboard of the unit square with
  values log-uniform in [0.1, 10] (``default_rng(2)``), quadrature p + 3,
  f = 1, u = 0 on the boundary.
* ``serving_requests``: the request stream of the serving loop: Poisson
  arrival times at a given rate, 70% 2-D P1/P2 Poisson on jittered triangle
  boxes and 30% 3-D P1 Poisson on tetrahedral boxes, dof counts log-uniform
  in [1e3, 2e6] mapped to the nearest box size, lognormal(0, 1) cell
  coefficients (``default_rng(3)``).
"""
import numpy as np

__all__ = ["tri_box_arrays", "tet_box_arrays", "jitter_interior", "lognormal_cells", "diffusion_mass_tet_box",
           "elasticity_tet_box", "batched_tri_meshes", "serving_requests", "tri_box_dofs", "tet_box_dofs"]


def _linspace(a, b, num):
    return np.linspace(a, b, num)


def tri_box_arrays(nx, ny, box=(0.0, 1.0, 0.0, 1.0)):
    x = _linspace(box[0], box[1], nx + 1)
    y = _linspace(box[2], box[3], ny + 1)
    X, Y = np.meshgrid(x, y, indexing="ij")
    node = np.stack([X.ravel(), Y.ravel()], axis=1)
    idx = np.arange((nx + 1) * (ny + 1), dtype=np.int32).reshape(nx + 1, ny + 1)
    c0 = np.stack([idx[1:, :-1].T.ravel(), idx[1:, 1:].T.ravel(), idx[:-1, :-1].T.ravel()], 1)
    c1 = np.stack([idx[:-1, 1:].T.ravel(), idx[:-1, :-1].T.ravel(), idx[1:, 1:].T.ravel()], 1)
    return node, np.concatenate([c0, c1], axis=0).astype(np.int32)


def tet_box_arrays(nx, ny, nz, box=(0.0, 1.0, 0.0, 1.0, 0.0, 1.0)):
    x = _linspace(box[0], box[1], nx + 1)
    y = _linspace(box[2], box[3], ny + 1)
    z = _linspace(box[4], box[5], nz + 1)
    X, Y, Z = np.meshgrid(x, y, z, indexing="ij")
    node = np.stack([X.ravel(), Y.ravel(), Z.ravel()], axis=1)
    idx = np.arange(node.shape[0], dtype=np.int32).reshape(nx + 1, ny + 1, nz + 1)
    nyz = (ny + 1) * (nz + 1)
    c0 = idx[:-1, :-1, :-1]
    c1 = c0 + nyz
    c2 = c1 + nz + 1
    c3 = c0 + nz + 1
    c4 = c0 + 1
    c5 = c4 + nyz
    c6 = c5 + nz + 1
    c7 = c4 + nz + 1
    cube = np.stack([c.ravel() for c in (c0, c1, c2, c3, c4, c5, c6, c7)], axis=1)
    local = np.array([[0, 1, 2, 6], [0, 5, 1, 6], [0, 4, 5, 6], [0, 7, 4, 6], [0, 3, 7, 6], [0, 2, 3, 6]])
    return node, np.ascontiguousarray(cube[:, local].reshape(-1, 4)).astype(np.int32)


def jitter_interior(node, h, amp, seed):
    """Move every node strictly inside the unit box by U(-amp*h, amp*h) per coordinate."""
    rng = np.random.default_rng(seed)
    d = rng.uniform(-amp * h, amp * h, size=node.shape)
    inside = np.all((node > 1e-12) & (node < 1.0 - 1e-12), axis=1)
    out = node.copy()
    out[inside] += d[inside]
    return out


def lognormal_cells(nc, sigma, seed):
    return np.exp(np.random.default_rng(seed).normal(0.0, sigma, nc))


def diffusion_mass_tet_box(n):
    node, cell = tet_box_arrays(n, n, n)
    node = jitter_interior(node, 1.0 / n, 0.2, seed=1)
    kappa = lognormal_cells(cell.shape[0], 1.0, seed=0)
    return node, cell, kappa


def elasticity_tet_box(n):
    node, cell = tet_box_arrays(n, n, n)
    scale = lognormal_cells(cell.shape[0], 0.5, seed=4)
    return node, cell, scale


def checkerboard_cells(node, cell, values):
    """Per-cell value of a 4x4 checkerboard on the unit square (cell barycentre)."""
    bc = node[cell].mean(axis=1)
    ix = np.clip((bc[:, 0] * 4).astype(np.int64), 0, 3)
    iy = np.clip((bc[:, 1] * 4).astype(np.int64), 0, 3)
    return values[iy * 4 + ix]


def batched_tri_meshes(count=256, seed=2):
    """The batched configuration: a list of dicts (nx, p, node, cell, kappa)."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        nx = int(round(np.exp(rng.uniform(np.log(16.0), np.log(512.0)))))
        p = int(rng.integers(1, 4))
        values = np.exp(rng.uniform(np.log(0.1), np.log(10.0), size=16))
        jseed = int(rng.integers(0, 2 ** 31 - 1))
        node, cell = tri_box_arrays(nx, nx)
        node = jitter_interior(node, 1.0 / nx, 0.15, seed=jseed)
        out.append({"nx": nx, "p": p, "node": node, "cell": cell,
                    "kappa": checkerboard_cells(node, cell, values)})
    return out


def tri_box_dofs(nx, p):
    return (p * nx + 1) ** 2


def tet_box_dofs(n):
    return (n + 1) ** 3


def serving_requests(count, rate, seed=3, dof_range=(1e3, 2e6)):
    """Requests (arrival time in s, kind, size, degree, coefficient seed).
    kind 'tri' (70%: P1 or P2 on an nx x nx triangle box) or 'tet' (30%: P1
    on an n^3 tetrahedral box); the box size is the one whose dof count is
    nearest to a log-uniform draw in ``dof_range``."""
    rng = np.random.default_rng(seed)
    t = np.cumsum(rng.exponential(1.0 / rate, size=count))
    reqs = []
    for i in range(count):
        target = np.exp(rng.uniform(np.log(dof_range[0]), np.log(dof_range[1])))
        if rng.uniform() < 0.7:
            p = int(rng.integers(1, 3))
            nx = max(2, int(round((np.sqrt(target) - 1) / p)))
            reqs.append({"t": float(t[i]), "kind": "tri", "n": nx, "p": p, "seed": int(rng.integers(0, 2 ** 31 - 1)),
                         "dofs": tri_box_dofs(nx, p)})
        else:
            n = max(2, int(round(target ** (1.0 / 3.0) - 1)))
            reqs.append({"t": float(t[i]), "kind": "tet", "n": n, "p": 1, "seed": int(rng.integers(0, 2 ** 31 - 1)),
                         "dofs": tet_box_dofs(n)})
    return reqs
