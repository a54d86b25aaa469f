"""Triangle and tetrahedron meshes with FEALPy's topology and dof numbering.

Meshes hold torch tensors (``node`` float64 (NN, GD), ``cell`` int32 (NC, TD+1))
on any device; the assembly path requires CUDA.  Topology follows
``MeshDS.construct`` (``fealpy/mesh/mesh_data_structure.py:428-464``): the
unique edges/faces are the lexicographically sorted unique vertex tuples
(``flocc``, ``fealpy/mesh/utils.py:81-110``), each stored in the orientation of
its first occurrence in cell order, with ``face2cell = [first cell, last cell,
first local index, last local index]``.  Interpolation-point (dof) numbering
follows ``cell_to_ipoint`` (``fealpy/mesh/triangle_mesh.py:218-270``,
``fealpy/mesh/tetrahedron_mesh.py:388-441``): vertices, then ``p-1`` points per
edge ordered from ``edge[:,0]`` to ``edge[:,1]``, then face and cell interior
points.  On a CUDA device the topology and the numbering are built by the
library's kernels (``fgb_topology_*``, ``fgb_cell_to_ipoint``); meshes held in
host memory use the same construction written with torch sorts (host-side
checks).  Mesh set-up is not part of the timed assemble/solve path; the
end-to-end bench leg includes it.
"""

import numpy as np
import torch

from . import simplex as sx
from .quadrature import TriangleQuadrature, TetrahedronQuadrature

__all__ = ["TriangleMesh", "TetrahedronMesh"]

_S = slice(None)


def _linspace(a: float, b: float, num: int, device) -> torch.Tensor:
    # numpy.linspace arithmetic (i*step + start, last point = stop) so that
    # node coordinates are bit-identical to FEALPy's numpy backend
    if num == 1:
        return torch.tensor([float(a)], dtype=torch.float64, device=device)
    step = (float(b) - float(a)) / (num - 1)
    y = torch.arange(num, dtype=torch.float64, device=device) * step + float(a)
    y[-1] = float(b)
    return y


def _lexsort_rows(keys: torch.Tensor) -> torch.Tensor:
    """Stable lexicographic argsort of the rows of an int64 (N, K) tensor
    (first column most significant), by successive stable sorts."""
    order = torch.arange(keys.shape[0], device=keys.device)
    for col in range(keys.shape[1] - 1, -1, -1):
        k = keys[order, col]
        _, idx = torch.sort(k, stable=True)
        order = order[idx]
    return order


def _flocc(rows: torch.Tensor):
    """First/last occurrence of each unique row of an integer (N, K) tensor and
    the map original row -> unique index (FEALPy's ``flocc``)."""
    keys = rows.to(torch.int64)
    order = _lexsort_rows(keys)
    srt = keys[order]
    diff = torch.any(srt[1:] != srt[:-1], dim=1)
    true = torch.ones(1, dtype=torch.bool, device=rows.device)
    flag = torch.cat([true, diff, true])
    group = torch.cumsum(flag[:-1].to(torch.int64), 0) - 1
    i0 = order[flag[:-1]]
    i1 = order[flag[1:]]
    j = torch.empty_like(order)
    j[order] = group
    return i0, i1, j


class _SimplexMesh:
    TD = 0
    localEdge = None
    localFace = None

    def __init__(self, node: torch.Tensor, cell: torch.Tensor):
        if node.dtype != torch.float64:
            raise TypeError("node must be float64")
        self.node = node
        self.cell = cell.to(torch.int32).contiguous()
        self.itype = torch.int32
        self.ftype = torch.float64
        self.device = node.device
        self.GD = node.shape[1]
        self.meshdata = {}
        self.celldata = {}
        self.nodedata = {}
        self.construct()

    # -- topology ---------------------------------------------------------
    def construct(self):
        if self.device.type == "cuda":
            # device kernels (fgb_topology_*): per-vertex grouping of the
            # local entities, ranked sorted tuples, first/last occurrences
            from .kernels import mesh_entities
            NN = self.number_of_nodes()
            self.face, self.face2cell, self.cell2face = mesh_entities(
                self.cell, NN, np.asarray(self.localFace, dtype=np.int32), True)
            if self.TD == 3:
                self.edge, _, self.cell2edge = mesh_entities(self.cell, NN, np.asarray(self.localEdge,
                                                                                      dtype=np.int32), False)
            else:
                self.edge = self.face
                self.cell2edge = self.cell2face
                self.edge2cell = self.face2cell
            return
        # meshes held in host memory (host-side checks): the same construction
        # with torch sorts
        NC = self.cell.shape[0]
        lf = torch.tensor(self.localFace, dtype=torch.int64, device=self.device)
        total_face = self.cell[:, lf].reshape(-1, lf.shape[1])
        i0, i1, j = _flocc(torch.sort(total_face, dim=1).values)
        NFC = lf.shape[0]
        self.face = total_face[i0].contiguous()
        self.cell2face = j.reshape(NC, NFC).to(torch.int32)
        self.face2cell = torch.stack([i0 // NFC, i1 // NFC, i0 % NFC, i1 % NFC], dim=1).to(torch.int32)
        if self.TD == 3:
            le = torch.tensor(self.localEdge, dtype=torch.int64, device=self.device)
            total_edge = self.cell[:, le].reshape(-1, 2)
            e0, _, ej = _flocc(torch.sort(total_edge, dim=1).values)
            self.edge = total_edge[e0].contiguous()
            self.cell2edge = ej.reshape(NC, le.shape[0]).to(torch.int32)
        else:
            self.edge = self.face
            self.cell2edge = self.cell2face
            self.edge2cell = self.face2cell

    # -- counts and entities ---------------------------------------------
    def geo_dimension(self):
        return self.GD

    def top_dimension(self):
        return self.TD

    def number_of_nodes(self):
        return self.node.shape[0]

    def number_of_cells(self):
        return self.cell.shape[0]

    def number_of_edges(self):
        return self.edge.shape[0]

    def number_of_faces(self):
        return self.face.shape[0]

    def count(self, etype):
        return {"cell": self.number_of_cells(), "face": self.number_of_faces(), "edge": self.number_of_edges(),
                "node": self.number_of_nodes()}[etype] if isinstance(etype, str) else \
            [self.number_of_nodes(), self.number_of_edges(), self.number_of_faces(), self.number_of_cells()][etype]

    def entity(self, etype, index=_S):
        name = etype if isinstance(etype, str) else {0: "node", 1: "edge", 2: "face" if self.TD == 3 else "cell",
                                                     3: "cell"}[etype]
        return {"node": self.node, "edge": self.edge, "face": self.face, "cell": self.cell}[name][index]

    def cell_to_face(self):
        return self.cell2face

    def cell_to_edge(self):
        return self.cell2edge

    def face_to_cell(self):
        return self.face2cell

    def boundary_face_flag(self):
        return self.face2cell[:, 0] == self.face2cell[:, 1]

    def boundary_face_index(self):
        return torch.nonzero(self.boundary_face_flag()).reshape(-1)

    def boundary_node_flag(self):
        flag = torch.zeros(self.number_of_nodes(), dtype=torch.bool, device=self.device)
        flag[self.face[self.boundary_face_flag()].reshape(-1).long()] = True
        return flag

    def entity_barycenter(self, etype, index=_S):
        ent = self.entity(etype, index)
        return self.node[ent.long()].mean(dim=1)

    def multi_index_matrix(self, p, TD=None):
        return torch.from_numpy(sx.multi_index_matrix(p, self.TD if TD is None else TD)).to(self.device)

    def quadrature_formula(self, q, etype="cell"):
        if etype not in ("cell", self.TD):
            raise NotImplementedError("only cell quadrature is provided")
        return TriangleQuadrature(q) if self.TD == 2 else TetrahedronQuadrature(q)

    def bc_to_point(self, bcs, index=_S):
        bcs_t = torch.as_tensor(bcs, dtype=torch.float64, device=self.device)
        pts = self.node[self.cell[index].long()]          # (NC, TD+1, GD)
        return torch.einsum("cvd,qv->cqd", pts, bcs_t)

    # -- measures and barycentric gradients (GPU kernels) -------------------
    def entity_measure(self, etype="cell", index=_S):
        if etype not in ("cell", self.TD):
            raise NotImplementedError("only cell measures are provided")
        from .kernels import cell_factors
        from . import _lib
        m = cell_factors(self, [(_lib.FGB_CH_MEASURE, -1, 1.0)], None, torch.float64)[:, 0]
        return m[index]

    def grad_lambda(self, index=_S):
        from .kernels import cell_factors
        from . import _lib
        TD = self.TD
        chans = [(_lib.FGB_CH_GRAD + k * 3 + a, -1, 1.0) for k in range(TD) for a in range(TD)]
        g = cell_factors(self, chans, None, torch.float64).reshape(-1, TD, TD)
        g0 = -g.sum(dim=1, keepdim=True)
        return torch.cat([g0, g], dim=1)[index]

    def shape_function(self, bcs, p=1):
        return torch.from_numpy(sx.shape_function(np.asarray(bcs), p)).to(self.device)

    def grad_shape_function(self, bcs, p=1, index=_S, variables="x"):
        R = torch.from_numpy(sx.grad_shape_function(np.asarray(bcs), p)).to(self.device)  # (NQ, ldof, TD+1)
        if variables == "u":
            return R
        Dl = self.grad_lambda(index)
        return torch.einsum("qjb,cbm->cqjm", R, Dl)

    # -- interpolation points / dofs ---------------------------------------
    def number_of_local_ipoints(self, p, iptype="cell"):
        td = {"cell": self.TD, "face": self.TD - 1, "edge": 1, "node": 0}.get(iptype, iptype)
        return sx.simplex_ldof(p, td)

    def number_of_global_ipoints(self, p):
        NN, NE, NC = self.number_of_nodes(), self.number_of_edges(), self.number_of_cells()
        n = NN + NE * (p - 1)
        if self.TD == 2:
            return n + NC * (p - 1) * (p - 2) // 2
        NF = self.number_of_faces()
        return n + NF * (p - 1) * (p - 2) // 2 + NC * (p - 1) * (p - 2) * (p - 3) // 6

    def ipoint_blocks(self, p):
        """Sizes of the contiguous ranges of the global interpolation-point
        numbering (vertices, edge interiors, face interiors, cell interiors;
        empty ranges left out), in the order number_of_global_ipoints counts
        them."""
        NN, NE, NC = self.number_of_nodes(), self.number_of_edges(), self.number_of_cells()
        sizes = [NN, NE * (p - 1)]
        if self.TD == 2:
            sizes.append(NC * (p - 1) * (p - 2) // 2)
        else:
            sizes += [self.number_of_faces() * (p - 1) * (p - 2) // 2, NC * (p - 1) * (p - 2) * (p - 3) // 6]
        return [int(v) for v in sizes if v > 0]

    def edge_to_ipoint(self, p, index=_S):
        NN = self.number_of_nodes()
        NE = self.number_of_edges()
        idx = torch.arange(NE, dtype=torch.int64, device=self.device)
        mid = idx[:, None] * (p - 1) + torch.arange(p - 1, device=self.device)[None, :] + NN
        e = self.edge.to(torch.int64)
        return torch.cat([e[:, :1], mid, e[:, 1:]], dim=1).to(torch.int32)[index]

    def cell_to_ipoint(self, p, index=_S):
        if p == 1:
            return self.cell[index]
        TD = self.TD
        if TD == 3 and p > 3:
            raise NotImplementedError("tetrahedron dofs are provided up to p = 3")
        if self.device.type == "cuda":
            from .kernels import cell_to_ipoint
            return cell_to_ipoint(self, p)[index]
        mi = sx.multi_index_matrix(p, TD)
        NC = self.number_of_cells()
        NN = self.number_of_nodes()
        NE = self.number_of_edges()
        cell = self.cell.to(torch.int64)
        c2e = self.cell2edge.to(torch.int64)
        edge = self.edge.to(torch.int64)
        c2p = torch.empty((NC, mi.shape[0]), dtype=torch.int64, device=self.device)
        local_edge = [(1, 2), (2, 0), (0, 1)] if TD == 2 else list(self.localEdge)
        edge_id = {tuple(sorted(e)): k for k, e in enumerate(local_edge)}
        nz = (mi > 0)
        interior_rank = 0
        face_base = NN + NE * (p - 1)
        for k in range(mi.shape[0]):
            support = np.nonzero(nz[k])[0]
            if len(support) == 1:
                c2p[:, k] = cell[:, support[0]]
            elif len(support) == 2:
                a, b = int(support[0]), int(support[1])
                le = edge_id[(a, b)]
                E = c2e[:, le]
                # position along the global edge = multi-index entry at the local
                # vertex that is the global edge's end vertex
                end_is_b = cell[:, b] == edge[E, 1]
                t = torch.where(end_is_b, torch.full_like(E, int(mi[k, b])), torch.full_like(E, int(mi[k, a])))
                c2p[:, k] = NN + E * (p - 1) + t - 1
            elif TD == 2:
                c2p[:, k] = face_base + torch.arange(NC, device=self.device) * ((p - 1) * (p - 2) // 2) + interior_rank
                interior_rank += 1
            else:
                # p == 3 tetrahedron: one interior point per face
                v_opp = int(np.nonzero(mi[k] == 0)[0][0])
                F = self.cell2face[:, v_opp].to(torch.int64)
                c2p[:, k] = face_base + F
        return c2p.to(torch.int32)[index]

    def interpolation_points(self, p, index=_S):
        if p == 1:
            return self.node[index]
        c2p = self.cell_to_ipoint(p).to(torch.int64)
        mi = torch.from_numpy(sx.multi_index_matrix(p, self.TD)).to(self.device, torch.float64) / p
        pts = torch.einsum("kv,cvd->ckd", mi, self.node[self.cell.long()])
        gdof = self.number_of_global_ipoints(p)
        ip = torch.empty((gdof, self.GD), dtype=torch.float64, device=self.device)
        ip[c2p.reshape(-1)] = pts.reshape(-1, self.GD)
        ip[: self.number_of_nodes()] = self.node
        return ip[index]

    def face_dof_mask(self, p):
        """(TD+1, ldof) bool: local dof k lies on the facet opposite local vertex v."""
        return torch.from_numpy(sx.local_face_of_multi_index(p, self.TD)).to(self.device)


class TriangleMesh(_SimplexMesh):
    TD = 2
    localEdge = [(1, 2), (2, 0), (0, 1)]
    localFace = [(1, 2), (2, 0), (0, 1)]

    @classmethod
    def from_box(cls, box=(0, 1, 0, 1), nx=10, ny=10, *, threshold=None, itype=None, ftype=None, device=None):
        """Structured triangulation of a box (``fealpy/mesh/triangle_mesh.py:1387-1435``)."""
        if threshold is not None:
            raise NotImplementedError("threshold-filtered boxes are not provided")
        x = _linspace(box[0], box[1], nx + 1, device)
        y = _linspace(box[2], box[3], ny + 1, device)
        X, Y = torch.meshgrid(x, y, indexing="ij")
        node = torch.stack([X.reshape(-1), Y.reshape(-1)], dim=1).contiguous()
        NN = (nx + 1) * (ny + 1)
        idx = torch.arange(NN, dtype=torch.int32, device=device).reshape(nx + 1, ny + 1)
        cell0 = torch.stack([idx[1:, :-1].T.reshape(-1), idx[1:, 1:].T.reshape(-1), idx[:-1, :-1].T.reshape(-1)], 1)
        cell1 = torch.stack([idx[:-1, 1:].T.reshape(-1), idx[:-1, :-1].T.reshape(-1), idx[1:, 1:].T.reshape(-1)], 1)
        cell = torch.cat([cell0, cell1], dim=0).contiguous()
        return cls(node, cell)


class TetrahedronMesh(_SimplexMesh):
    TD = 3
    localEdge = [(0, 1), (0, 2), (0, 3), (1, 2), (1, 3), (2, 3)]
    localFace = [(1, 2, 3), (0, 3, 2), (0, 1, 3), (0, 2, 1)]

    @classmethod
    def from_box(cls, box=(0, 1, 0, 1, 0, 1), nx=10, ny=10, nz=10, threshold=None, device=None):
        """Kuhn subdivision of a box into 6 tetrahedra per cube
        (``fealpy/mesh/tetrahedron_mesh.py:1017-1086``)."""
        if threshold is not None:
            raise NotImplementedError("threshold-filtered boxes are not provided")
        x = _linspace(box[0], box[1], nx + 1, device)
        y = _linspace(box[2], box[3], ny + 1, device)
        z = _linspace(box[4], box[5], nz + 1, device)
        X, Y, Z = torch.meshgrid(x, y, z, indexing="ij")
        node = torch.stack([X.reshape(-1), Y.reshape(-1), Z.reshape(-1)], dim=1).contiguous()
        NN = (nx + 1) * (ny + 1) * (nz + 1)
        idx = torch.arange(NN, dtype=torch.int32, device=device).reshape(nx + 1, ny + 1, nz + 1)
        nyz = (ny + 1) * (nz + 1)
        c0 = idx[:-1, :-1, :-1]
        c1 = c0 + nyz
        c2 = c1 + nz + 1
        c3 = c0 + nz + 1
        c4 = c0 + 1
        c5 = c4 + nyz
        c6 = c5 + nz + 1
        c7 = c4 + nz + 1
        cube = torch.stack([c.reshape(-1) for c in (c0, c1, c2, c3, c4, c5, c6, c7)], dim=1)
        local = torch.tensor([[0, 1, 2, 6], [0, 5, 1, 6], [0, 4, 5, 6], [0, 7, 4, 6], [0, 3, 7, 6], [0, 2, 3, 6]],
                             dtype=torch.int64, device=device)
        cell = cube[:, local].reshape(-1, 4).contiguous()
        mesh = cls(node, cell)
        mesh.box = list(box)
        return mesh
