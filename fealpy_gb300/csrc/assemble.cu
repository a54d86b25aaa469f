// Numeric assembly: per-cell geometric factors and the row-gather scatter of
// cell contributions straight into CSR values.
//
// FEALPy evaluates gphi (NC, NQ, ldof, GD) at every quadrature point, contracts
// it with einsum into dense local matrices (NC, ldof, ldof), lays them out as COO
// triplets and sums duplicates with np.add.at after a lexsort
// (fealpy/functional.py:68-106, fealpy/fem/bilinear_form.py:46-75,
// fealpy/sparse/coo_tensor.py:184-213).  For affine simplices and coefficients
// that are constant per cell the quadrature sum factors exactly:
//
//   K_c[i][j] = sum_q w_q |T_c| k_c grad(phi_i).grad(phi_j)
//             = sum_{k<=l} (|T_c| k_c grad(l_k).grad(l_l)) * S_kl[i][j]
//
// with S_kl = sum_q w_q dphi_i/dl_k dphi_j/dl_l (symmetrised) a mesh-independent
// table built once on the host from the same quadrature rule.  The device work
// is therefore split in two:
//   1. cell_factors: one thread per cell computes the FP64 Jacobian, its
//      determinant and inverse and writes a handful of factor channels;
//   2. assemble_*: one warp per CSR row gathers the cells around the row's dof
//      (adjacency sorted by cell), rebuilds that row of each local matrix from
//      the factors and the tables held in shared memory, and accumulates into a
//      shared-memory copy of the row.  Contributions are summed in cell order
//      and every CSR value is written exactly once: no atomics, deterministic.

#include "fgb_common.cuh"

namespace fgb {

struct ChanParams {
  int n;
  int kind[FGB_MAX_CHANNELS];
  int coef[FGB_MAX_CHANNELS];
  double scale[FGB_MAX_CHANNELS];
};

template <typename TOut, int TD>
__global__ void cell_factors_kernel(int64_t n_cell, const double* __restrict__ node, const int32_t* __restrict__ cell,
                                    ChanParams ch, const double* __restrict__ coef, TOut* __restrict__ out,
                                    int32_t* status) {
  constexpr int NV = TD + 1;
  for (int64_t c = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; c < n_cell;
       c += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    int v[NV];
    if (NV == 4) {
      int4 q = __ldg(reinterpret_cast<const int4*>(cell) + c);
      v[0] = q.x; v[1] = q.y; v[2] = q.z; v[3] = q.w;
    } else {
#pragma unroll
      for (int k = 0; k < NV; ++k) v[k] = __ldg(cell + c * NV + k);
    }
    double x0[TD], J[TD][TD];
#pragma unroll
    for (int a = 0; a < TD; ++a) x0[a] = __ldg(node + static_cast<int64_t>(v[0]) * TD + a);
#pragma unroll
    for (int k = 0; k < TD; ++k)
#pragma unroll
      for (int a = 0; a < TD; ++a) J[a][k] = __ldg(node + static_cast<int64_t>(v[k + 1]) * TD + a) - x0[a];
    double inv[TD][TD];  // inv[k][a] = d lambda_{k+1} / d x_a
    double det, measure;
    if (TD == 2) {
      det = J[0][0] * J[1][1] - J[0][1] * J[1][0];
      double r = 1.0 / det;
      inv[0][0] = J[1][1] * r;  inv[0][1] = -J[0][1] * r;
      inv[1][0] = -J[1][0] * r; inv[1][1] = J[0][0] * r;
      measure = 0.5 * det;
    } else {
      double c00 = J[1][1] * J[2][2] - J[1][2] * J[2][1];
      double c01 = J[1][2] * J[2][0] - J[1][0] * J[2][2];
      double c02 = J[1][0] * J[2][1] - J[1][1] * J[2][0];
      det = J[0][0] * c00 + J[0][1] * c01 + J[0][2] * c02;
      double r = 1.0 / det;
      // inverse of J: inv[k][a] = cofactor(a, k) / det
      inv[0][0] = c00 * r;
      inv[0][1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) * r;
      inv[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) * r;
      inv[1][0] = c01 * r;
      inv[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) * r;
      inv[1][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) * r;
      inv[2][0] = c02 * r;
      inv[2][1] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) * r;
      inv[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) * r;
      measure = det * (1.0 / 6.0);
    }
    if (!isfinite(det) || det == 0.0) set_status(status, FGB_ERR_NONFINITE);
    for (int j = 0; j < ch.n; ++j) {
      const int kind = ch.kind[j];
      double val;
      if (kind == FGB_CH_MEASURE) {
        val = measure;
      } else if (kind < FGB_CH_GRAD) {
        const int k = (kind - FGB_CH_METRIC) / 3, l = (kind - FGB_CH_METRIC) % 3;
        double s = 0.0;
#pragma unroll
        for (int a = 0; a < TD; ++a) s += inv[k][a] * inv[l][a];
        val = measure * s;
      } else {
        const int k = (kind - FGB_CH_GRAD) / 3, a = (kind - FGB_CH_GRAD) % 3;
        val = inv[k][a];
      }
      val *= ch.scale[j];
      if (ch.coef[j] >= 0) val *= __ldg(coef + static_cast<int64_t>(ch.coef[j]) * n_cell + c);
      out[c * ch.n + j] = static_cast<TOut>(val);
    }
  }
}

// ---------------------------------------------------------------------------
// scalar assembly
// ---------------------------------------------------------------------------
struct RowSmem {
  int cap;     // row capacity (entries)
  int ncopy;   // independent accumulator copies per warp
};

// LDOF > 0: the local dof count as a compile-time constant (divisions by it
// become multiply-shifts); LDOF == 0: taken from `ldof_rt`.  MAP: the
// contribution of adjacency entry k and local dof j lands at the row slot
// pos[k * ldof + j] recorded by the pattern pass (rows of at most kRowMapMax
// entries); otherwise the slot is found by a binary search of the row's
// columns.
template <typename T, int LDOF, bool MAP>
__device__ bool assemble_scalar_row(int64_t i, const int64_t* __restrict__ adj_ptr, const int32_t* __restrict__ adj,
                                    const int32_t* __restrict__ c2d, int ldof_rt, int nt, const T* __restrict__ tab,
                                    const T* __restrict__ factors, const int64_t* __restrict__ indptr,
                                    const int32_t* __restrict__ indices, const uint8_t* __restrict__ pos,
                                    T* __restrict__ values, float* __restrict__ values32, int32_t* cols, T* acc,
                                    int cap, int ncopy, int accumulate, int32_t* status) {
  const int ldof = LDOF > 0 ? LDOF : ldof_rt;
  const int lane = threadIdx.x & 31;
  const int64_t base = indptr[i];
  const int L = static_cast<int>(indptr[i + 1] - base);
  if (L > cap) return false;
  if constexpr (!MAP)
    for (int t = lane; t < L; t += 32) cols[t] = __ldg(indices + base + t);
  for (int g = 0; g < ncopy; ++g)
    for (int t = lane; t < L; t += 32) acc[g * cap + t] = T(0);
  __syncwarp();
  const int64_t s = adj_ptr[i], e = adj_ptr[i + 1];
  const int g = lane / ldof, lj = lane - g * ldof;
  const int ld2 = ldof * ldof;
  for (int64_t k0 = s; k0 < e; k0 += ncopy) {
    const int64_t k = k0 + g;
    if (g < ncopy && k < e) {
      const int32_t en = __ldg(adj + k);
      const int32_t c = en / ldof;
      const int li = en - c * ldof;
      int slot;
      if constexpr (MAP) {
        slot = __ldg(pos + k * ldof + lj);
      } else {
        const int32_t col = __ldg(c2d + static_cast<int64_t>(c) * ldof + lj);
        slot = lower_bound_i32(cols, L, col);
        if (slot < L && cols[slot] != col) slot = L;
      }
      const T* f = factors + static_cast<int64_t>(c) * nt;
      const T* tb = tab + li * ldof + lj;
      T v = T(0);
      for (int t = 0; t < nt; ++t) v += __ldg(f + t) * tb[t * ld2];
      if (slot < L) acc[g * cap + slot] += v;
      else set_status(status, FGB_ERR_PATTERN);
    }
    __syncwarp();
  }
  for (int t = lane; t < L; t += 32) {
    T v = acc[t];
    for (int gg = 1; gg < ncopy; ++gg) v += acc[gg * cap + t];
    if (accumulate) v = values[base + t] + v;  // a later pass of split factor channels
    values[base + t] = v;
    if (values32) values32[base + t] = static_cast<float>(v);
  }
  __syncwarp();
  return true;
}

// Dynamic shared memory layout: tables (nt*ldof*ldof T) | per warp: acc (ncopy*cap T) | cols (cap int32)
template <typename T, int LDOF, bool MAP>
__global__ void assemble_scalar_kernel(int64_t n_rows, const int32_t* __restrict__ row_list,
                                       const int32_t* __restrict__ row_list_len, const int64_t* __restrict__ adj_ptr,
                                       const int32_t* __restrict__ adj, const int32_t* __restrict__ c2d, int ldof,
                                       int nt, const T* __restrict__ tables, const T* __restrict__ factors,
                                       const int64_t* __restrict__ indptr, const int32_t* __restrict__ indices,
                                       const uint8_t* __restrict__ pos, T* __restrict__ values,
                                       float* __restrict__ values32, int cap, int ncopy,
                                       int accumulate, int32_t* __restrict__ ovf, int32_t* __restrict__ ovf_len,
                                       int32_t* status) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* tab = reinterpret_cast<T*>(smem_raw);
  const int ntab = nt * ldof * ldof;
  for (int t = threadIdx.x; t < ntab; t += blockDim.x) tab[t] = tables[t];
  __syncthreads();
  const int wpb = blockDim.x >> 5, wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
  size_t off = align_up(static_cast<size_t>(ntab) * sizeof(T), 16);
  const size_t per_warp = align_up(static_cast<size_t>(ncopy) * cap * sizeof(T) + static_cast<size_t>(cap) * 4, 16);
  T* acc = reinterpret_cast<T*>(smem_raw + off + per_warp * wib);
  int32_t* cols = reinterpret_cast<int32_t*>(smem_raw + off + per_warp * wib + static_cast<size_t>(ncopy) * cap * sizeof(T));
  const int64_t n = row_list ? static_cast<int64_t>(*row_list_len) : n_rows;
  const int64_t warp = static_cast<int64_t>(blockIdx.x) * wpb + wib;
  const int64_t nwarps = static_cast<int64_t>(gridDim.x) * wpb;
  for (int64_t r = warp; r < n; r += nwarps) {
    const int64_t i = row_list ? row_list[r] : r;
    bool done = assemble_scalar_row<T, LDOF, MAP>(i, adj_ptr, adj, c2d, ldof, nt, tab, factors, indptr, indices, pos,
                                                  values, values32, cols, acc, cap, ncopy, accumulate, status);
    if (!done && lane == 0) {
      if (ovf) { int slot = atomicAdd(ovf_len, 1); ovf[slot] = static_cast<int32_t>(i); }
      else set_status(status, FGB_ERR_CAPACITY);
    }
  }
}

// ---------------------------------------------------------------------------
// P1 linear elasticity, interleaved components
// ---------------------------------------------------------------------------
template <typename T, int GD>
__device__ __forceinline__ void grad_p1(const T* f, int li, T* g) {
  // f[k*GD + a] = d lambda_{k+1} / d x_a ; grad lambda_0 = -sum_k grad lambda_{k+1}
  if (li == 0) {
#pragma unroll
    for (int a = 0; a < GD; ++a) {
      T s = T(0);
#pragma unroll
      for (int k = 0; k < GD; ++k) s += f[k * GD + a];
      g[a] = -s;
    }
  } else {
#pragma unroll
    for (int a = 0; a < GD; ++a) g[a] = f[(li - 1) * GD + a];
  }
}

template <typename T, int GD>
__device__ bool assemble_elasticity_row(int64_t i, const int64_t* __restrict__ adj_ptr, const int32_t* __restrict__ adj,
                                        const int32_t* __restrict__ cell, const T* __restrict__ factors,
                                        const int64_t* __restrict__ node_indptr, const int32_t* __restrict__ node_indices,
                                        const int64_t* __restrict__ indptr, T* __restrict__ values,
                                        float* __restrict__ values32, int32_t* cols, T* acc, int cap, int ncopy,
                                        int32_t* status) {
  constexpr int NV = GD + 1;
  constexpr int LPC = NV * GD;  // lanes per cell
  constexpr int NF = GD * GD + 3;
  const int lane = threadIdx.x & 31;
  const int64_t nbase = node_indptr[i];
  const int L = static_cast<int>(node_indptr[i + 1] - nbase);
  if (L > cap) return false;
  const int rowlen = L * GD;               // entries per vector row
  const int stride = GD * rowlen;          // per-copy accumulator size
  for (int t = lane; t < L; t += 32) cols[t] = __ldg(node_indices + nbase + t);
  for (int t = lane; t < ncopy * stride; t += 32) acc[t] = T(0);
  __syncwarp();
  const int64_t s = adj_ptr[i], e = adj_ptr[i + 1];
  const int g = lane / LPC, r = lane - g * LPC, lj = r / GD, b = r - lj * GD;
  for (int64_t k0 = s; k0 < e; k0 += ncopy) {
    const int64_t k = k0 + g;
    if (g < ncopy && k < e) {
      const int32_t en = __ldg(adj + k);
      const int32_t c = en / NV;
      const int li = en - c * NV;
      const int32_t j = __ldg(cell + static_cast<int64_t>(c) * NV + lj);
      T f[NF];
#pragma unroll
      for (int t = 0; t < NF; ++t) f[t] = __ldg(factors + static_cast<int64_t>(c) * NF + t);
      T gi[GD], gj[GD];
      grad_p1<T, GD>(f, li, gi);
      grad_p1<T, GD>(f, lj, gj);
      const T d00 = f[GD * GD], dl = f[GD * GD + 1], dm = f[GD * GD + 2];
      T dot = T(0);
#pragma unroll
      for (int a = 0; a < GD; ++a) dot += gi[a] * gj[a];
      const int pos = lower_bound_i32(cols, L, j);
      if (pos < L && cols[pos] == j) {
        T* ac = acc + g * stride + pos * GD + b;
#pragma unroll
        for (int a = 0; a < GD; ++a) {
          T val;
          if (a == b) val = d00 * gi[a] * gj[a] + dm * (dot - gi[a] * gj[a]);
          else val = dl * gi[a] * gj[b] + dm * gi[b] * gj[a];
          ac[a * rowlen] += val;
        }
      } else {
        set_status(status, FGB_ERR_PATTERN);
      }
    }
    __syncwarp();
  }
  for (int a = 0; a < GD; ++a) {
    const int64_t o = indptr[i * GD + a];
    for (int t = lane; t < rowlen; t += 32) {
      T v = acc[a * rowlen + t];
      for (int gg = 1; gg < ncopy; ++gg) v += acc[gg * stride + a * rowlen + t];
      values[o + t] = v;
      if (values32) values32[o + t] = static_cast<float>(v);
    }
  }
  __syncwarp();
  return true;
}

template <typename T, int GD>
__global__ void assemble_elasticity_kernel(int64_t n_node, const int32_t* __restrict__ row_list,
                                           const int32_t* __restrict__ row_list_len, const int64_t* __restrict__ adj_ptr,
                                           const int32_t* __restrict__ adj, const int32_t* __restrict__ cell,
                                           const T* __restrict__ factors, const int64_t* __restrict__ node_indptr,
                                           const int32_t* __restrict__ node_indices, const int64_t* __restrict__ indptr,
                                           T* __restrict__ values, float* __restrict__ values32, int cap, int ncopy,
                                           int32_t* __restrict__ ovf, int32_t* __restrict__ ovf_len, int32_t* status) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int wpb = blockDim.x >> 5, wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const size_t per_warp =
      align_up(static_cast<size_t>(ncopy) * GD * GD * cap * sizeof(T) + static_cast<size_t>(cap) * 4, 16);
  T* acc = reinterpret_cast<T*>(smem_raw + per_warp * wib);
  int32_t* cols = reinterpret_cast<int32_t*>(smem_raw + per_warp * wib + static_cast<size_t>(ncopy) * GD * GD * cap * sizeof(T));
  const int64_t n = row_list ? static_cast<int64_t>(*row_list_len) : n_node;
  const int64_t warp = static_cast<int64_t>(blockIdx.x) * wpb + wib;
  const int64_t nwarps = static_cast<int64_t>(gridDim.x) * wpb;
  for (int64_t r = warp; r < n; r += nwarps) {
    const int64_t i = row_list ? row_list[r] : r;
    bool done = assemble_elasticity_row<T, GD>(i, adj_ptr, adj, cell, factors, node_indptr, node_indices, indptr,
                                               values, values32, cols, acc, cap, ncopy, status);
    if (!done && lane == 0) {
      if (ovf) { int slot = atomicAdd(ovf_len, 1); ovf[slot] = static_cast<int32_t>(i); }
      else set_status(status, FGB_ERR_CAPACITY);
    }
  }
}

// out[i] = sum over i's adjacency of local[c*ldof + li], in cell order: the
// deterministic replacement of the index_add scatter of cell vectors.
template <typename T>
__global__ void gather_sum_kernel(int64_t n, const int64_t* __restrict__ adj_ptr, const int32_t* __restrict__ adj,
                                  const T* __restrict__ local, T* __restrict__ out) {
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    T s = T(0);
    for (int64_t k = adj_ptr[i]; k < adj_ptr[i + 1]; ++k) s += local[adj[k]];
    out[i] = s;
  }
}

constexpr int kAsmWarps = 8;
constexpr int kAsmCap = 128;      // first pass: row entries per warp
constexpr int kAsmBigCap = 4096;  // second pass: one warp per block, one accumulator copy
constexpr size_t kMaxDynSmem = 200 * 1024;

template <typename T, bool MAP>
auto scalar_kernel_for(int ldof) {
  switch (ldof) {
    case 3: return assemble_scalar_kernel<T, 3, MAP>;
    case 4: return assemble_scalar_kernel<T, 4, MAP>;
    case 6: return assemble_scalar_kernel<T, 6, MAP>;
    case 10: return assemble_scalar_kernel<T, 10, MAP>;
    default: return assemble_scalar_kernel<T, 0, MAP>;
  }
}

// First launch: rows of at most kAsmCap entries, one warp each (direct slots
// when the pattern's positions are given); rows that do not fit are listed
// and done by a second launch with one warp per block and a larger row
// buffer (column search).  Measured on the P2 tetrahedral 64^3 matrix (60.9 M
// entries): FP64 values 3.15 ms with slots against 3.56 ms searching, FP32
// 1.39 against 1.94 ms; recording the slots adds 0.64 ms to the pattern, so
// they pay off once a pattern is assembled into more than once.
template <typename T>
int launch_scalar(int64_t n_dof, const int64_t* adj_ptr, const int32_t* adj, const int32_t* c2d, int ldof, int nt,
                  const T* tables, const T* factors, const int64_t* indptr, const int32_t* indices,
                  const uint8_t* pos, T* values, float* values32, int accumulate, int32_t* status, int32_t* ovf,
                  int32_t* ovf_len, cudaStream_t st) {
  static_assert(kAsmCap <= kRowMapMax, "direct slots exist for rows up to kRowMapMax entries");
  const size_t tab_bytes = align_up(static_cast<size_t>(nt) * ldof * ldof * sizeof(T), 16);
  const int ncopy = 32 / ldof;
  const size_t per_warp1 = align_up(static_cast<size_t>(ncopy) * kAsmCap * sizeof(T) + kAsmCap * 4, 16);
  const size_t smem1 = tab_bytes + per_warp1 * kAsmWarps;
  const size_t per_warp2 = align_up(static_cast<size_t>(kAsmBigCap) * sizeof(T) + kAsmBigCap * 4, 16);
  const size_t smem2 = tab_bytes + per_warp2;
  if (smem1 > kMaxDynSmem || smem2 > kMaxDynSmem) return FGB_ERR_CAPACITY;
  auto kern = scalar_kernel_for<T, false>(ldof);
  auto kmap = scalar_kernel_for<T, true>(ldof);
  auto k1 = pos ? kmap : kern;
  cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem2 > smem1 ? smem2 : smem1));
  cudaFuncSetAttribute(kmap, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem1));
  cudaMemsetAsync(ovf_len, 0, sizeof(int32_t), st);
  const int grid1 = grid_for(n_dof, kAsmWarps, kNumSMs * 16);
  k1<<<grid1, kAsmWarps * 32, smem1, st>>>(n_dof, nullptr, nullptr, adj_ptr, adj, c2d, ldof, nt, tables, factors,
                                           indptr, indices, pos, values, values32, kAsmCap, ncopy, accumulate, ovf,
                                           ovf_len, status);
  kern<<<kNumSMs, 32, smem2, st>>>(n_dof, ovf, ovf_len, adj_ptr, adj, c2d, ldof, nt, tables, factors, indptr, indices,
                                   nullptr, values, values32, kAsmBigCap, 1, accumulate, nullptr, nullptr, status);
  return launch_status();
}

template <typename T, int GD>
int launch_elasticity(int64_t n_node, const int64_t* adj_ptr, const int32_t* adj, const int32_t* cell,
                      const T* factors, const int64_t* node_indptr, const int32_t* node_indices,
                      const int64_t* indptr, T* values, float* values32, int32_t* status, int32_t* ovf,
                      int32_t* ovf_len, cudaStream_t st) {
  constexpr int LPC = (GD + 1) * GD;
  const int ncopy = 32 / LPC;
  constexpr int cap1 = 64, cap2 = 1024;
  const size_t per_warp1 = align_up(static_cast<size_t>(ncopy) * GD * GD * cap1 * sizeof(T) + cap1 * 4, 16);
  const size_t smem1 = per_warp1 * kAsmWarps;
  const size_t smem2 = align_up(static_cast<size_t>(GD) * GD * cap2 * sizeof(T) + cap2 * 4, 16);
  cudaFuncSetAttribute(assemble_elasticity_kernel<T, GD>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       static_cast<int>(smem2 > smem1 ? smem2 : smem1));
  cudaMemsetAsync(ovf_len, 0, sizeof(int32_t), st);
  assemble_elasticity_kernel<T, GD><<<grid_for(n_node, kAsmWarps, kNumSMs * 16), kAsmWarps * 32, smem1, st>>>(
      n_node, nullptr, nullptr, adj_ptr, adj, cell, factors, node_indptr, node_indices, indptr, values, values32, cap1,
      ncopy, ovf, ovf_len, status);
  assemble_elasticity_kernel<T, GD><<<kNumSMs, 32, smem2, st>>>(n_node, ovf, ovf_len, adj_ptr, adj, cell, factors,
                                                                node_indptr, node_indices, indptr, values, values32,
                                                                cap2, 1, nullptr, nullptr, status);
  return launch_status();
}

}  // namespace fgb

using namespace fgb;

extern "C" {

int32_t fgb_cell_factors(int32_t td, int64_t n_cell, const double* node, const int32_t* cell, int32_t n_channel,
                         const int32_t* chan_kind_host, const int32_t* chan_coef_host,
                         const double* chan_scale_host, const double* coef, int32_t out_dtype, void* factors,
                         int32_t* status, void* stream) {
  if ((td != 2 && td != 3) || n_cell < 0 || n_channel <= 0 || n_channel > FGB_MAX_CHANNELS) return FGB_ERR_ARG;
  if (n_cell == 0) return FGB_OK;
  if (node == nullptr || cell == nullptr || factors == nullptr || chan_kind_host == nullptr) return FGB_ERR_ARG;
  if (out_dtype != FGB_F32 && out_dtype != FGB_F64) return FGB_ERR_ARG;
  if (td == 3 && (reinterpret_cast<uintptr_t>(cell) % 16) != 0) return FGB_ERR_ARG;
  ChanParams ch{};
  ch.n = n_channel;
  for (int j = 0; j < n_channel; ++j) {
    int kind = chan_kind_host[j];
    bool ok = kind == FGB_CH_MEASURE ||
              (kind >= FGB_CH_METRIC && kind < FGB_CH_METRIC + 9 && (kind - FGB_CH_METRIC) / 3 < td &&
               (kind - FGB_CH_METRIC) % 3 < td) ||
              (kind >= FGB_CH_GRAD && kind < FGB_CH_GRAD + 9 && (kind - FGB_CH_GRAD) / 3 < td &&
               (kind - FGB_CH_GRAD) % 3 < td);
    if (!ok) return FGB_ERR_ARG;
    ch.kind[j] = kind;
    ch.coef[j] = chan_coef_host ? chan_coef_host[j] : -1;
    if (ch.coef[j] >= 0 && coef == nullptr) return FGB_ERR_ARG;
    ch.scale[j] = chan_scale_host ? chan_scale_host[j] : 1.0;
  }
  cudaStream_t st = as_stream(stream);
  const int grid = grid_for(n_cell, 256, kNumSMs * 32);
  if (td == 2) {
    if (out_dtype == FGB_F64)
      cell_factors_kernel<double, 2><<<grid, 256, 0, st>>>(n_cell, node, cell, ch, coef, static_cast<double*>(factors), status);
    else
      cell_factors_kernel<float, 2><<<grid, 256, 0, st>>>(n_cell, node, cell, ch, coef, static_cast<float*>(factors), status);
  } else {
    if (out_dtype == FGB_F64)
      cell_factors_kernel<double, 3><<<grid, 256, 0, st>>>(n_cell, node, cell, ch, coef, static_cast<double*>(factors), status);
    else
      cell_factors_kernel<float, 3><<<grid, 256, 0, st>>>(n_cell, node, cell, ch, coef, static_cast<float*>(factors), status);
  }
  return launch_status();
}

int32_t fgb_gather_sum(int32_t dtype, int64_t n, const int64_t* adj_ptr, const int32_t* adj, const void* local,
                       void* out, void* stream) {
  if (n <= 0 || !adj_ptr || !adj || !local || !out) return FGB_ERR_ARG;
  cudaStream_t st = as_stream(stream);
  const int grid = grid_for(n, 256, kNumSMs * 16);
  if (dtype == FGB_F64)
    gather_sum_kernel<double><<<grid, 256, 0, st>>>(n, adj_ptr, adj, static_cast<const double*>(local),
                                                    static_cast<double*>(out));
  else if (dtype == FGB_F32)
    gather_sum_kernel<float><<<grid, 256, 0, st>>>(n, adj_ptr, adj, static_cast<const float*>(local),
                                                   static_cast<float*>(out));
  else
    return FGB_ERR_ARG;
  return launch_status();
}

size_t fgb_assemble_workspace_bytes(int64_t n_rows) {
  return align_up(static_cast<size_t>(n_rows) * sizeof(int32_t)) + align_up(sizeof(int32_t));
}

int32_t fgb_assemble_scalar(int32_t dtype, int64_t n_dof, const int64_t* adj_ptr, const int32_t* adj,
                            const int32_t* cell2dof, int32_t ldof, int32_t n_table, const void* tables,
                            const void* factors, const int64_t* indptr, const int32_t* indices, void* values,
                            float* values_f32, int32_t* status, void* workspace, size_t workspace_bytes,
                            void* stream) {
  return fgb_assemble_scalar_acc(dtype, n_dof, adj_ptr, adj, cell2dof, ldof, n_table, tables, factors, indptr, indices,
                                 nullptr, values, values_f32, 0, status, workspace, workspace_bytes, stream);
}

int32_t fgb_assemble_scalar_acc(int32_t dtype, int64_t n_dof, const int64_t* adj_ptr, const int32_t* adj,
                                const int32_t* cell2dof, int32_t ldof, int32_t n_table, const void* tables,
                                const void* factors, const int64_t* indptr, const int32_t* indices,
                                const uint8_t* positions, void* values, float* values_f32, int32_t accumulate,
                                int32_t* status, void* workspace, size_t workspace_bytes, void* stream) {
  if (n_dof <= 0 || ldof <= 0 || ldof > 32 || n_table <= 0 || !adj_ptr || !adj || !cell2dof || !tables ||
      !factors || !indptr || !indices || !values)
    return FGB_ERR_ARG;
  if (workspace == nullptr || workspace_bytes < fgb_assemble_workspace_bytes(n_dof)) return FGB_ERR_WORKSPACE;
  Carver cv(workspace, workspace_bytes);
  int32_t* ovf = cv.take<int32_t>(n_dof);
  int32_t* ovf_len = cv.take<int32_t>(1);
  cudaStream_t st = as_stream(stream);
  if (dtype == FGB_F64)
    return launch_scalar<double>(n_dof, adj_ptr, adj, cell2dof, ldof, n_table, static_cast<const double*>(tables),
                                 static_cast<const double*>(factors), indptr, indices, positions,
                                 static_cast<double*>(values), values_f32, accumulate ? 1 : 0, status, ovf, ovf_len, st);
  if (dtype == FGB_F32)
    return launch_scalar<float>(n_dof, adj_ptr, adj, cell2dof, ldof, n_table, static_cast<const float*>(tables),
                                static_cast<const float*>(factors), indptr, indices, positions,
                                static_cast<float*>(values), values_f32, accumulate ? 1 : 0, status, ovf, ovf_len, st);
  return FGB_ERR_ARG;
}

int32_t fgb_assemble_elasticity_p1(int32_t dtype, int32_t gd, int64_t n_node, const int64_t* adj_ptr,
                                   const int32_t* adj, const int32_t* cell, const void* factors,
                                   const int64_t* node_indptr, const int32_t* node_indices, const int64_t* indptr,
                                   void* values, float* values_f32, int32_t* status, void* workspace,
                                   size_t workspace_bytes, void* stream) {
  if ((gd != 2 && gd != 3) || n_node <= 0 || !adj_ptr || !adj || !cell || !factors || !node_indptr ||
      !node_indices || !indptr || !values)
    return FGB_ERR_ARG;
  if (workspace == nullptr || workspace_bytes < fgb_assemble_workspace_bytes(n_node)) return FGB_ERR_WORKSPACE;
  Carver cv(workspace, workspace_bytes);
  int32_t* ovf = cv.take<int32_t>(n_node);
  int32_t* ovf_len = cv.take<int32_t>(1);
  cudaStream_t st = as_stream(stream);
  if (dtype == FGB_F64) {
    if (gd == 3)
      return launch_elasticity<double, 3>(n_node, adj_ptr, adj, cell, static_cast<const double*>(factors), node_indptr,
                                          node_indices, indptr, static_cast<double*>(values), values_f32, status, ovf,
                                          ovf_len, st);
    return launch_elasticity<double, 2>(n_node, adj_ptr, adj, cell, static_cast<const double*>(factors), node_indptr,
                                        node_indices, indptr, static_cast<double*>(values), values_f32, status, ovf,
                                        ovf_len, st);
  }
  if (dtype == FGB_F32) {
    if (gd == 3)
      return launch_elasticity<float, 3>(n_node, adj_ptr, adj, cell, static_cast<const float*>(factors), node_indptr,
                                         node_indices, indptr, static_cast<float*>(values), values_f32, status, ovf,
                                         ovf_len, st);
    return launch_elasticity<float, 2>(n_node, adj_ptr, adj, cell, static_cast<const float*>(factors), node_indptr,
                                       node_indices, indptr, static_cast<float*>(values), values_f32, status, ovf,
                                       ovf_len, st);
  }
  return FGB_ERR_ARG;
}

}  // extern "C"
