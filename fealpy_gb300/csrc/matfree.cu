// Matrix-free operator apply: y = A x for a bilinear form that has not been
// assembled, as FEALPy's BilinearForm.__matmul__ does when no global matrix
// exists (fealpy/fem/bilinear_form.py:126-158: gather u at each cell's dofs,
// einsum with the cell-local matrices, index_add into the output).
//
// Two kernels, no atomics:
//   cell_apply  one thread per cell: gathers x at the cell's dofs, forms
//               K_c x_c = sum_t f_t(c) (S_t x_c) from the per-cell factor
//               channels and the mesh-independent tables S_t (the same
//               factorisation as the CSR assembly), and writes the cell's
//               ldof results;
//   gather_sum  one thread per dof: adds the results of the cells around it
//               in cell order (the adjacency of the symbolic phase).
// The tables travel in the kernel's parameter space: the fully unrolled
// contraction reads them as constant-bank operands of its multiply-adds, so
// the cell kernel is limited by its gathers and the factor/dof-map stream,
// not by shared-memory loads.  Tables of more than 10 local dofs (P3
// tetrahedra) are read from shared memory by a generic kernel.

#include "fgb_common.cuh"

namespace fgb {

constexpr int kMfMaxNt = 16;     // table channels (FGB_MAX_CHANNELS)
constexpr int kMfMaxLdof = 10;   // local dofs of the unrolled kernels
constexpr int kMfThreads = 256;

template <typename T>
struct CellTables {
  T s[kMfMaxNt * kMfMaxLdof * kMfMaxLdof];
};

template <typename T, int LDOF>
__global__ void __launch_bounds__(kMfThreads) cell_apply_kernel(int64_t n_cell, const int32_t* __restrict__ c2d,
                                                                  int nt, const T* __restrict__ factors,
                                                                  const T* __restrict__ x, T* __restrict__ ycell,
                                                                  const __grid_constant__ CellTables<T> tab) {
  for (int64_t c = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; c < n_cell;
       c += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    T xl[LDOF];
#pragma unroll
    for (int j = 0; j < LDOF; ++j) xl[j] = __ldg(x + __ldg(c2d + c * LDOF + j));
    T y[LDOF];
#pragma unroll
    for (int i = 0; i < LDOF; ++i) y[i] = T(0);
#pragma unroll
    for (int t = 0; t < kMfMaxNt; ++t) {
      if (t < nt) {
        const T f = __ldg(factors + c * nt + t);
#pragma unroll
        for (int i = 0; i < LDOF; ++i) {
          T w = T(0);
#pragma unroll
          for (int j = 0; j < LDOF; ++j) w += tab.s[(t * LDOF + i) * LDOF + j] * xl[j];
          y[i] += f * w;
        }
      }
    }
#pragma unroll
    for (int i = 0; i < LDOF; ++i) ycell[c * LDOF + i] = y[i];
  }
}

// Any ldof up to 32: tables in shared memory, runtime loops.
template <typename T>
__global__ void __launch_bounds__(kMfThreads) cell_apply_generic(int64_t n_cell, const int32_t* __restrict__ c2d,
                                                                   int ldof, int nt, const T* __restrict__ tables,
                                                                   const T* __restrict__ factors,
                                                                   const T* __restrict__ x, T* __restrict__ ycell) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* tab = reinterpret_cast<T*>(smem_raw);
  const int ntab = nt * ldof * ldof;
  for (int k = threadIdx.x; k < ntab; k += blockDim.x) tab[k] = tables[k];
  __syncthreads();
  for (int64_t c = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; c < n_cell;
       c += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    T xl[32];
    for (int j = 0; j < ldof; ++j) xl[j] = __ldg(x + __ldg(c2d + c * ldof + j));
    for (int i = 0; i < ldof; ++i) {
      T yi = T(0);
      for (int t = 0; t < nt; ++t) {
        T w = T(0);
        const T* s = tab + (t * ldof + i) * ldof;
        for (int j = 0; j < ldof; ++j) w += s[j] * xl[j];
        yi += __ldg(factors + c * nt + t) * w;
      }
      ycell[c * ldof + i] = yi;
    }
  }
}

template <typename T>
int launch_cell_apply(int64_t n_cell, int ldof, const int32_t* c2d, int nt, const double* tables_host,
                      const T* tables_dev, const T* factors, const T* x, T* ycell, cudaStream_t st) {
  const int grid = grid_for(n_cell, kMfThreads, kNumSMs * 16);
  if (ldof <= kMfMaxLdof && (ldof == 3 || ldof == 4 || ldof == 6 || ldof == 10) && tables_host) {
    CellTables<T> tab;
    for (int t = 0; t < nt; ++t)
      for (int k = 0; k < ldof * ldof; ++k) tab.s[t * ldof * ldof + k] = static_cast<T>(tables_host[t * ldof * ldof + k]);
    switch (ldof) {
      case 3: cell_apply_kernel<T, 3><<<grid, kMfThreads, 0, st>>>(n_cell, c2d, nt, factors, x, ycell, tab); break;
      case 4: cell_apply_kernel<T, 4><<<grid, kMfThreads, 0, st>>>(n_cell, c2d, nt, factors, x, ycell, tab); break;
      case 6: cell_apply_kernel<T, 6><<<grid, kMfThreads, 0, st>>>(n_cell, c2d, nt, factors, x, ycell, tab); break;
      default: cell_apply_kernel<T, 10><<<grid, kMfThreads, 0, st>>>(n_cell, c2d, nt, factors, x, ycell, tab); break;
    }
    return launch_status();
  }
  if (!tables_dev) return FGB_ERR_ARG;
  const size_t smem = static_cast<size_t>(nt) * ldof * ldof * sizeof(T);
  if (smem > 200 * 1024) return FGB_ERR_CAPACITY;
  cudaFuncSetAttribute(cell_apply_generic<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
  cell_apply_generic<T><<<grid, kMfThreads, smem, st>>>(n_cell, c2d, ldof, nt, tables_dev, factors, x, ycell);
  return launch_status();
}

}  // namespace fgb

using namespace fgb;

extern "C" {

int32_t fgb_cell_apply(int32_t dtype, int64_t n_cell, int32_t ldof, const int32_t* cell2dof, int32_t n_table,
                       const double* tables_host, const void* tables, const void* factors, const void* x,
                       void* ycell, void* stream) {
  if (n_cell < 0 || ldof <= 0 || ldof > 32 || n_table <= 0 || n_table > kMfMaxNt) return FGB_ERR_ARG;
  if (n_cell == 0) return FGB_OK;
  if (!cell2dof || !factors || !x || !ycell || (!tables_host && !tables)) return FGB_ERR_ARG;
  cudaStream_t st = as_stream(stream);
  if (dtype == FGB_F64)
    return launch_cell_apply<double>(n_cell, ldof, cell2dof, n_table, tables_host, static_cast<const double*>(tables),
                                     static_cast<const double*>(factors), static_cast<const double*>(x),
                                     static_cast<double*>(ycell), st);
  if (dtype == FGB_F32)
    return launch_cell_apply<float>(n_cell, ldof, cell2dof, n_table, tables_host, static_cast<const float*>(tables),
                                    static_cast<const float*>(factors), static_cast<const float*>(x),
                                    static_cast<float*>(ycell), st);
  return FGB_ERR_ARG;
}

}  // extern "C"
