// Mesh topology and interpolation-point (dof) numbering on the device.
//
// FEALPy's MeshDS.construct (fealpy/mesh/mesh_data_structure.py:428-464) lists
// every local sub-entity of every cell (edges, or faces), sorts the vertex
// tuples of each, lexsorts the sorted tuples and keeps the unique ones
// (flocc, fealpy/mesh/utils.py:81-110): entity e is the e-th distinct sorted
// tuple in lexicographic order, stored in the orientation of its first
// occurrence (cell order, then local index), and face2cell holds the first
// and last occurrence (cell, local index).
//
// Here the occurrences o = c * nfc + l are grouped by their smallest vertex s0
// (counting sort: count, scan, fill), every vertex's group is sorted by
// (rest of the sorted tuple, o) in shared memory by one warp, and the distinct
// tuples are ranked; the lexicographic order of (s0, s1, s2) is then vertex by
// vertex, tuple by tuple, so entity numbers are the scan of the per-vertex
// distinct counts plus the rank.  The occurrence order inside a group gives
// first and last occurrences exactly as the stable lexsort does.  Everything is
// integer work and deterministic.
//
// cell_to_ipoint (fealpy/mesh/triangle_mesh.py:218-270,
// fealpy/mesh/tetrahedron_mesh.py:388-441): vertices, then p-1 points per edge
// counted from the edge's first vertex, then face and cell interiors; one thread
// per (cell, local point) from a small per-point table built on the host.

#include "fgb_common.cuh"

#include <climits>

namespace fgb {

struct EntTable {
  int k;     // vertices per entity (2 edges, 3 faces)
  int nfc;   // entities per cell
  int nv;    // vertices per cell
  int le[6][3];
};

// sorted vertex tuple of occurrence o (s[0] < s[1] < s[2]); false on a bad index
__device__ __forceinline__ bool occ_sorted(const int32_t* __restrict__ cell, const EntTable& T, int64_t o,
                                           int64_t nn, int32_t s[3]) {
  const int64_t c = o / T.nfc;
  const int l = static_cast<int>(o - c * T.nfc);
  for (int a = 0; a < T.k; ++a) s[a] = __ldg(cell + c * T.nv + T.le[l][a]);
  if (T.k == 2) {
    if (s[0] > s[1]) { const int32_t t = s[0]; s[0] = s[1]; s[1] = t; }
    s[2] = 0;
  } else {
    if (s[0] > s[1]) { const int32_t t = s[0]; s[0] = s[1]; s[1] = t; }
    if (s[1] > s[2]) { const int32_t t = s[1]; s[1] = s[2]; s[2] = t; }
    if (s[0] > s[1]) { const int32_t t = s[0]; s[0] = s[1]; s[1] = t; }
  }
  for (int a = 0; a < T.k; ++a)
    if (s[a] < 0 || s[a] >= nn) return false;
  return true;
}

__global__ void topo_count(int64_t n_occ, const int32_t* __restrict__ cell, const __grid_constant__ EntTable T, int64_t nn,
                           int32_t* __restrict__ cnt, int32_t* status) {
  for (int64_t o = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; o < n_occ;
       o += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    int32_t s[3];
    if (!occ_sorted(cell, T, o, nn, s)) {
      set_status(status, FGB_ERR_INDEX);
      continue;
    }
    atomicAdd(cnt + s[0], 1);
  }
}

__global__ void topo_fill(int64_t n_occ, const int32_t* __restrict__ cell, const __grid_constant__ EntTable T, int64_t nn,
                          const int64_t* __restrict__ ptr, int32_t* __restrict__ cursor, int32_t* __restrict__ occ) {
  for (int64_t o = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; o < n_occ;
       o += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    int32_t s[3];
    if (!occ_sorted(cell, T, o, nn, s)) continue;
    const int32_t slot = atomicAdd(cursor + s[0], 1);
    occ[ptr[s[0]] + slot] = static_cast<int32_t>(o);
  }
}

// sort key of an occurrence inside its vertex group: the rest of the sorted
// tuple, then the occurrence itself (so equal tuples keep occurrence order)
struct OccKey {
  unsigned long long key;
  int32_t o;
};

__device__ __forceinline__ bool occ_less(const OccKey& a, const OccKey& b) {
  return a.key < b.key || (a.key == b.key && a.o < b.o);
}

constexpr int kTopoWarps = 8;
constexpr int kTopoCap = 128;      // occurrences per vertex group, first pass (warp, shared memory)
constexpr int kTopoBigCap = 4096;  // second pass (one warp per block)

// One vertex group: sort, rank distinct tuples.  mode 0: write the distinct
// count to ent_cnt[v]; mode 1: write entities, entity2cell and cell2entity.
// Returns false when the group exceeds `cap`.
__device__ bool topo_group(int64_t v, int mode, const int32_t* __restrict__ cell, const EntTable& T, int64_t nn,
                           const int64_t* __restrict__ ptr, const int32_t* __restrict__ occ,
                           int32_t* __restrict__ ent_cnt, const int64_t* __restrict__ eptr,
                           int32_t* __restrict__ entity, int32_t* __restrict__ ent2cell,
                           int32_t* __restrict__ cell2ent, OccKey* buf, int cap) {
  const int lane = threadIdx.x & 31;
  const int64_t s0 = ptr[v];
  const int m = static_cast<int>(ptr[v + 1] - s0);
  if (m > cap) return false;
  int np2 = 32;
  while (np2 < m) np2 <<= 1;
  if (np2 > cap) return false;
  for (int t = lane; t < np2; t += 32) {
    OccKey q;
    if (t < m) {
      const int32_t o = occ[s0 + t];
      int32_t s[3];
      occ_sorted(cell, T, o, nn, s);
      q.key = T.k == 2 ? static_cast<unsigned long long>(s[1])
                       : static_cast<unsigned long long>(s[1]) * static_cast<unsigned long long>(nn) + s[2];
      q.o = o;
    } else {
      q.key = ULLONG_MAX;
      q.o = INT_MAX;
    }
    buf[t] = q;
  }
  __syncwarp();
  for (int kk = 2; kk <= np2; kk <<= 1) {
    for (int j = kk >> 1; j > 0; j >>= 1) {
      for (int t = lane; t < np2; t += 32) {
        const int u = t ^ j;
        if (u > t) {
          const OccKey a = buf[t], b = buf[u];
          const bool up = (t & kk) == 0;
          if (occ_less(b, a) == up) {
            buf[t] = b;
            buf[u] = a;
          }
        }
      }
      __syncwarp();
    }
  }
  int running = 0;
  const int64_t base = mode == 1 ? eptr[v] : 0;
  for (int b0 = 0; b0 < m; b0 += 32) {
    const int t = b0 + lane;
    bool first = false;
    OccKey q{0ull, 0};
    if (t < m) {
      q = buf[t];
      first = t == 0 || buf[t - 1].key != q.key;
    }
    const unsigned ball = __ballot_sync(0xffffffffu, first);
    // entity of element t: distinct tuples up to and including t, minus one
    const int rank = running + __popc(ball & ((2u << lane) - 1u)) - 1;
    if (mode == 1 && t < m) {
      const int64_t e = base + rank;
      const int64_t c = q.o / T.nfc;
      const int l = static_cast<int>(q.o - c * T.nfc);
      cell2ent[q.o] = static_cast<int32_t>(e);
      const bool last = t == m - 1 || buf[t + 1].key != q.key;
      if (first) {
        for (int a = 0; a < T.k; ++a) entity[e * T.k + a] = __ldg(cell + c * T.nv + T.le[l][a]);
        if (ent2cell) {
          ent2cell[e * 4 + 0] = static_cast<int32_t>(c);
          ent2cell[e * 4 + 2] = l;
        }
      }
      if (last && ent2cell) {
        ent2cell[e * 4 + 1] = static_cast<int32_t>(c);
        ent2cell[e * 4 + 3] = l;
      }
    }
    running += __popc(ball);
  }
  if (mode == 0 && lane == 0) ent_cnt[v] = running;
  __syncwarp();
  return true;
}

__global__ void __launch_bounds__(kTopoWarps * 32) topo_rows(int64_t nn, int mode, const int32_t* __restrict__ cell,
                                                             const __grid_constant__ EntTable T, const int64_t* __restrict__ ptr,
                                                             const int32_t* __restrict__ occ,
                                                             int32_t* __restrict__ ent_cnt,
                                                             const int64_t* __restrict__ eptr,
                                                             int32_t* __restrict__ entity,
                                                             int32_t* __restrict__ ent2cell,
                                                             int32_t* __restrict__ cell2ent, int32_t* __restrict__ ovf,
                                                             int32_t* __restrict__ ovf_len) {
  __shared__ OccKey sbuf[kTopoWarps * kTopoCap];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  OccKey* buf = sbuf + wib * kTopoCap;
  const int64_t warp = (blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x) >> 5;
  const int64_t nwarps = (static_cast<int64_t>(gridDim.x) * blockDim.x) >> 5;
  for (int64_t v = warp; v < nn; v += nwarps) {
    const bool done = topo_group(v, mode, cell, T, nn, ptr, occ, ent_cnt, eptr, entity, ent2cell, cell2ent, buf,
                                 kTopoCap);
    if (!done && lane == 0) {
      const int slot = atomicAdd(ovf_len, 1);
      ovf[slot] = static_cast<int32_t>(v);
    }
  }
}

// Groups above the first-pass capacity: one warp per block, dynamic shared memory.
__global__ void topo_rows_big(int mode, const int32_t* __restrict__ cell, const __grid_constant__ EntTable T, int64_t nn,
                              const int64_t* __restrict__ ptr, const int32_t* __restrict__ occ,
                              int32_t* __restrict__ ent_cnt, const int64_t* __restrict__ eptr,
                              int32_t* __restrict__ entity, int32_t* __restrict__ ent2cell,
                              int32_t* __restrict__ cell2ent, const int32_t* __restrict__ ovf,
                              const int32_t* __restrict__ ovf_len, int32_t* status) {
  extern __shared__ __align__(16) unsigned char dsm[];
  OccKey* buf = reinterpret_cast<OccKey*>(dsm);
  const int n = *ovf_len;
  for (int r = blockIdx.x; r < n; r += gridDim.x) {
    const bool done = topo_group(ovf[r], mode, cell, T, nn, ptr, occ, ent_cnt, eptr, entity, ent2cell, cell2ent, buf,
                                 kTopoBigCap);
    if (!done && (threadIdx.x & 31) == 0) set_status(status, FGB_ERR_CAPACITY);
  }
}

// ------------------------------------------------------------ cell_to_ipoint
constexpr int kIpMax = 32;  // local interpolation points (P3 tetrahedra: 20)

struct IpTable {
  int ldof, td, p;
  int kind[kIpMax];  // 0 vertex, 1 edge, 2 cell interior (triangles), 3 face (P3 tetrahedra)
  int a[kIpMax], b[kIpMax];    // vertex: a; edge: local vertices a < b
  int le[kIpMax];              // edge: local edge index; face: local face index (= opposite vertex)
  int ma[kIpMax], mb[kIpMax];  // edge: multi-index entries at a and b
  int rank[kIpMax];            // cell interior: rank among the cell's interior points
};

__global__ void cell_to_ipoint_kernel(int64_t n_cell, const int32_t* __restrict__ cell,
                                      const int32_t* __restrict__ cell2edge, const int32_t* __restrict__ edge,
                                      const int32_t* __restrict__ cell2face, int64_t nn, int64_t ne,
                                      int64_t n_face_pts, const __grid_constant__ IpTable P,
                                      int32_t* __restrict__ c2p) {
  const int64_t total = n_cell * P.ldof;
  const int nv = P.td + 1;
  const int ne_loc = P.td == 2 ? 3 : 6;
  const int64_t n_int = P.td == 2 ? static_cast<int64_t>(P.p - 1) * (P.p - 2) / 2 : 0;
  for (int64_t t = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; t < total;
       t += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int64_t c = t / P.ldof;
    const int k = static_cast<int>(t - c * P.ldof);
    int64_t out;
    switch (P.kind[k]) {
      case 0:
        out = __ldg(cell + c * nv + P.a[k]);
        break;
      case 1: {
        const int64_t E = __ldg(cell2edge + c * ne_loc + P.le[k]);
        // position along the global edge: the multi-index entry at the local
        // vertex that is the global edge's end vertex
        const bool end_is_b = __ldg(cell + c * nv + P.b[k]) == __ldg(edge + 2 * E + 1);
        out = nn + E * (P.p - 1) + (end_is_b ? P.mb[k] : P.ma[k]) - 1;
        break;
      }
      case 2:
        out = nn + ne * (P.p - 1) + c * n_int + P.rank[k];
        break;
      default:
        out = nn + ne * (P.p - 1) + __ldg(cell2face + c * 4 + P.le[k]);
        break;
    }
    (void)n_face_pts;
    c2p[t] = static_cast<int32_t>(out);
  }
}

}  // namespace fgb

using namespace fgb;

extern "C" {

size_t fgb_topology_workspace_bytes(int64_t n_node, int64_t n_occ) {
  return align_up(static_cast<size_t>(n_node + 1) * sizeof(int64_t)) * 2 +
         align_up(static_cast<size_t>(n_node + 1) * sizeof(int32_t)) * 2 +
         align_up(static_cast<size_t>(n_occ) * sizeof(int32_t)) + align_up(static_cast<size_t>(n_node) * 4) +
         align_up(sizeof(int32_t)) + scan_workspace_bytes(n_node + 1);
}

int32_t fgb_topology_count(int64_t n_cell, int32_t nv, const int32_t* cell, int64_t n_node, int32_t k, int32_t nfc,
                           const int32_t* local_host, int64_t* n_entity_host, int32_t* status, void* workspace,
                           size_t workspace_bytes, void* stream) {
  if (n_cell <= 0 || nv < 3 || nv > 4 || !cell || n_node <= 0 || (k != 2 && k != 3) || nfc <= 0 || nfc > 6 ||
      !local_host || !n_entity_host || !status)
    return FGB_ERR_ARG;
  const int64_t n_occ = n_cell * nfc;
  if (n_occ >= (int64_t(1) << 31) || n_node >= (int64_t(1) << 31)) return FGB_ERR_CAPACITY;
  if (!workspace || workspace_bytes < fgb_topology_workspace_bytes(n_node, n_occ)) return FGB_ERR_WORKSPACE;
  EntTable T{};
  T.k = k;
  T.nfc = nfc;
  T.nv = nv;
  for (int l = 0; l < nfc; ++l)
    for (int a = 0; a < k; ++a) {
      const int v = local_host[l * k + a];
      if (v < 0 || v >= nv) return FGB_ERR_ARG;
      T.le[l][a] = v;
    }
  cudaStream_t st = as_stream(stream);
  Carver cv(workspace, workspace_bytes);
  int64_t* ptr = cv.take<int64_t>(n_node + 1);
  int64_t* eptr = cv.take<int64_t>(n_node + 1);
  int32_t* cnt = cv.take<int32_t>(n_node + 1);
  int32_t* ecnt = cv.take<int32_t>(n_node + 1);
  int32_t* occ = cv.take<int32_t>(n_occ);
  int32_t* ovf = cv.take<int32_t>(n_node);
  int32_t* ovf_len = cv.take<int32_t>(1);
  void* scan_ws = cv.base + cv.off;
  const size_t scan_bytes = workspace_bytes - cv.off;
  if (!cv.ok) return FGB_ERR_WORKSPACE;
  const int grid = grid_for(n_occ, 256, kNumSMs * 16);
  if (cudaMemsetAsync(cnt, 0, (n_node + 1) * sizeof(int32_t), st) != cudaSuccess) return FGB_ERR_CUDA;
  topo_count<<<grid, 256, 0, st>>>(n_occ, cell, T, n_node, cnt, status);
  int rc = exclusive_scan_i32_to_i64(cnt, n_node, ptr, scan_ws, scan_bytes, st);
  if (rc) return rc;
  if (cudaMemsetAsync(cnt, 0, (n_node + 1) * sizeof(int32_t), st) != cudaSuccess) return FGB_ERR_CUDA;
  topo_fill<<<grid, 256, 0, st>>>(n_occ, cell, T, n_node, ptr, cnt, occ);
  if (cudaMemsetAsync(ovf_len, 0, sizeof(int32_t), st) != cudaSuccess) return FGB_ERR_CUDA;
  if (cudaMemsetAsync(ecnt, 0, (n_node + 1) * sizeof(int32_t), st) != cudaSuccess) return FGB_ERR_CUDA;
  const int rgrid = grid_for(n_node, kTopoWarps, kNumSMs * 16);
  topo_rows<<<rgrid, kTopoWarps * 32, 0, st>>>(n_node, 0, cell, T, ptr, occ, ecnt, nullptr, nullptr, nullptr, nullptr,
                                               ovf, ovf_len);
  const size_t big = static_cast<size_t>(kTopoBigCap) * sizeof(OccKey);
  cudaFuncSetAttribute(topo_rows_big, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(big));
  topo_rows_big<<<kNumSMs, 32, big, st>>>(0, cell, T, n_node, ptr, occ, ecnt, nullptr, nullptr, nullptr, nullptr, ovf,
                                          ovf_len, status);
  rc = exclusive_scan_i32_to_i64(ecnt, n_node, eptr, scan_ws, scan_bytes, st);
  if (rc) return rc;
  if (cudaMemcpyAsync(n_entity_host, eptr + n_node, sizeof(int64_t), cudaMemcpyDeviceToHost, st) != cudaSuccess)
    return FGB_ERR_CUDA;
  if (cudaStreamSynchronize(st) != cudaSuccess) return FGB_ERR_CUDA;
  return launch_status();
}

int32_t fgb_topology_fill(int64_t n_cell, int32_t nv, const int32_t* cell, int64_t n_node, int32_t k, int32_t nfc,
                          const int32_t* local_host, int32_t* entity, int32_t* entity2cell, int32_t* cell2entity,
                          int32_t* status, void* workspace, size_t workspace_bytes, void* stream) {
  if (n_cell <= 0 || nv < 3 || nv > 4 || !cell || n_node <= 0 || (k != 2 && k != 3) || nfc <= 0 || nfc > 6 ||
      !local_host || !entity || !cell2entity || !status)
    return FGB_ERR_ARG;
  const int64_t n_occ = n_cell * nfc;
  if (!workspace || workspace_bytes < fgb_topology_workspace_bytes(n_node, n_occ)) return FGB_ERR_WORKSPACE;
  EntTable T{};
  T.k = k;
  T.nfc = nfc;
  T.nv = nv;
  for (int l = 0; l < nfc; ++l)
    for (int a = 0; a < k; ++a) T.le[l][a] = local_host[l * k + a];
  cudaStream_t st = as_stream(stream);
  Carver cv(workspace, workspace_bytes);
  int64_t* ptr = cv.take<int64_t>(n_node + 1);
  int64_t* eptr = cv.take<int64_t>(n_node + 1);
  int32_t* cnt = cv.take<int32_t>(n_node + 1);
  int32_t* ecnt = cv.take<int32_t>(n_node + 1);
  int32_t* occ = cv.take<int32_t>(n_occ);
  int32_t* ovf = cv.take<int32_t>(n_node);
  int32_t* ovf_len = cv.take<int32_t>(1);
  if (!cv.ok) return FGB_ERR_WORKSPACE;
  (void)cnt;
  // the grouping (ptr, occ) and the entity offsets (eptr) of fgb_topology_count
  // are still in the workspace; the overflow list is rebuilt by this pass
  if (cudaMemsetAsync(ovf_len, 0, sizeof(int32_t), st) != cudaSuccess) return FGB_ERR_CUDA;
  const int rgrid = grid_for(n_node, kTopoWarps, kNumSMs * 16);
  topo_rows<<<rgrid, kTopoWarps * 32, 0, st>>>(n_node, 1, cell, T, ptr, occ, ecnt, eptr, entity, entity2cell,
                                               cell2entity, ovf, ovf_len);
  const size_t big = static_cast<size_t>(kTopoBigCap) * sizeof(OccKey);
  cudaFuncSetAttribute(topo_rows_big, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(big));
  topo_rows_big<<<kNumSMs, 32, big, st>>>(1, cell, T, n_node, ptr, occ, ecnt, eptr, entity, entity2cell, cell2entity,
                                          ovf, ovf_len, status);
  return launch_status();
}

int32_t fgb_cell_to_ipoint(int64_t n_cell, int32_t td, int32_t p, int32_t ldof, const int32_t* cell,
                           const int32_t* cell2edge, const int32_t* edge, const int32_t* cell2face, int64_t n_node,
                           int64_t n_edge, const int32_t* kind_host, const int32_t* a_host, const int32_t* b_host,
                           const int32_t* le_host, const int32_t* ma_host, const int32_t* mb_host,
                           const int32_t* rank_host, int32_t* cell2ipoint, void* stream) {
  if (n_cell <= 0 || (td != 2 && td != 3) || p < 1 || ldof <= 0 || ldof > kIpMax || !cell || !cell2ipoint ||
      !kind_host)
    return FGB_ERR_ARG;
  IpTable P{};
  P.ldof = ldof;
  P.td = td;
  P.p = p;
  bool need_edges = false, need_faces = false;
  for (int k = 0; k < ldof; ++k) {
    P.kind[k] = kind_host[k];
    P.a[k] = a_host[k];
    P.b[k] = b_host[k];
    P.le[k] = le_host[k];
    P.ma[k] = ma_host[k];
    P.mb[k] = mb_host[k];
    P.rank[k] = rank_host[k];
    if (P.kind[k] < 0 || P.kind[k] > 3 || P.a[k] < 0 || P.a[k] > td || P.b[k] < 0 || P.b[k] > td) return FGB_ERR_ARG;
    if (P.kind[k] == 1) need_edges = true;
    if (P.kind[k] == 3) need_faces = true;
    if (P.kind[k] == 1 && (P.le[k] < 0 || P.le[k] >= (td == 2 ? 3 : 6))) return FGB_ERR_ARG;
    if (P.kind[k] == 3 && (td != 3 || P.le[k] < 0 || P.le[k] > 3)) return FGB_ERR_ARG;
  }
  if ((need_edges && (!cell2edge || !edge)) || (need_faces && !cell2face)) return FGB_ERR_ARG;
  const int64_t total = n_cell * ldof;
  cell_to_ipoint_kernel<<<grid_for(total, 256, kNumSMs * 16), 256, 0, as_stream(stream)>>>(
      n_cell, cell, cell2edge, edge, cell2face, n_node, n_edge, 0, P, cell2ipoint);
  return launch_status();
}

}  // extern "C"
