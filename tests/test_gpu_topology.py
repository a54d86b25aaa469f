"""Mesh topology and dof numbering on the device (fgb_topology_*,
fgb_cell_to_ipoint) against the reference's fixtures (edges, face2cell and
cell2dof that FEALPy itself produced) and, bit for bit, against the host-side
construction (torch sorts: FEALPy's lexsort/flocc written out) on larger and
irregular meshes: Kuhn tetrahedral boxes, triangle boxes with P1-P4, a
300-triangle fan (a vertex group above the first-pass capacity) and a
shuffled, jittered tetrahedral mesh."""
import os

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def cuda():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch.device("cuda:0")


def same(a, b):
    a = a.detach().cpu().numpy() if isinstance(a, torch.Tensor) else np.asarray(a)
    b = b.detach().cpu().numpy() if isinstance(b, torch.Tensor) else np.asarray(b)
    return a.shape == b.shape and np.array_equal(a, b)


def _compare(cls, node, cell, ps):
    dev = cuda()
    import fealpy_gb300 as F
    g = cls(torch.as_tensor(node, device=dev), torch.as_tensor(cell, device=dev))
    h = cls(torch.as_tensor(node), torch.as_tensor(cell))
    for name in ("face", "face2cell", "cell2face", "edge", "cell2edge"):
        assert same(getattr(g, name), getattr(h, name)), name
    for p in ps:
        assert same(F.LagrangeFESpace(g, p).cell_to_dof(), F.LagrangeFESpace(h, p).cell_to_dof()), p


@pytest.mark.parametrize("tag", ["tri_p1", "tri_p2", "tri_p3", "tet_p1", "tet_p2"])
def test_topology_against_reference_fixtures(golden_dir, tag):
    dev = cuda()
    import fealpy_gb300 as F
    z = np.load(os.path.join(golden_dir, f"small_{tag}.npz"))
    cls = F.TriangleMesh if z["cell"].shape[1] == 3 else F.TetrahedronMesh
    mesh = cls(torch.as_tensor(z["node"], device=dev), torch.as_tensor(z["cell"], dtype=torch.int32, device=dev))
    assert same(mesh.edge, z["edge"])
    assert same(mesh.face2cell, z["face2cell"])
    assert same(F.LagrangeFESpace(mesh, int(z["p"])).cell_to_dof(), z["cell2dof"])


def test_topology_config_fixtures(golden_dir):
    dev = cuda()
    import fealpy_gb300 as F
    for name, cls, p in (("cfg_c2_tet_p2_8.npz", F.TetrahedronMesh, 2), ("cfg_c3_tri_p3_32.npz", F.TriangleMesh, 3)):
        z = np.load(os.path.join(golden_dir, name))
        mesh = cls(torch.as_tensor(z["node"], device=dev), torch.as_tensor(z["cell"], dtype=torch.int32, device=dev))
        assert same(F.LagrangeFESpace(mesh, p).cell_to_dof(), z["cell2dof"]), name


def test_topology_matches_host_construction():
    from fealpy_gb300 import TriangleMesh, TetrahedronMesh
    from fealpy_gb300.workloads import tet_box_arrays, tri_box_arrays, jitter_interior
    node, cell = tet_box_arrays(7, 5, 6)
    _compare(TetrahedronMesh, node, cell, (1, 2, 3))
    node, cell = tri_box_arrays(13, 9)
    _compare(TriangleMesh, node, cell, (1, 2, 3, 4))
    # a fan of 300 triangles: vertex 0 owns 300 edges (600 occurrences)
    m = 300
    ang = np.linspace(0, 2 * np.pi, m, endpoint=False)
    fan_node = np.concatenate([[[0.0, 0.0]], np.c_[np.cos(ang), np.sin(ang)]], axis=0)
    fan_cell = np.array([[0, 1 + k, 1 + (k + 1) % m] for k in range(m)], dtype=np.int32)
    _compare(TriangleMesh, fan_node, fan_cell, (1, 2, 3))
    # cells in a shuffled order with rotated vertex orders: first occurrences
    # and orientations differ from the structured ordering
    rng = np.random.default_rng(5)
    node, cell = tet_box_arrays(6, 6, 6)
    node = jitter_interior(node, 1 / 6, 0.2, 3)
    cell = cell[rng.permutation(cell.shape[0])]
    rot = rng.integers(0, 4, size=cell.shape[0])
    cell = np.stack([np.roll(c, r) for c, r in zip(cell, rot)]).astype(np.int32)
    _compare(TetrahedronMesh, node, cell, (1, 2, 3))
