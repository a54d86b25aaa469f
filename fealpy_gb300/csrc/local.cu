// Cell-local matrices on request: Integrator.assembly(space) of FEALPy
// (fealpy/fem/scalar_diffusion_integrator.py, scalar_mass_integrator.py,
// linear_elasticity_integrator.py:61-181 return the (NC, ldof, ldof) local
// matrices).  The CSR path never forms them (the row-gather assembly
// contracts factors and tables per contribution); these kernels serve callers
// that want the local matrices themselves, from the same factor channels.

#include "fgb_common.cuh"

namespace fgb {

// out[c][i][j] (+)= sum_t factors[c][t] * tables[t][i][j]: one thread per
// entry, consecutive threads on consecutive (i, j) of a cell (coalesced
// writes; the cell's factors are the same address for its entries).
template <typename T>
__global__ void local_matrices_kernel(int64_t n_cell, int ldof, int nt, const T* __restrict__ factors,
                                      const T* __restrict__ tables, T* __restrict__ out, int accumulate) {
  const int64_t l2 = static_cast<int64_t>(ldof) * ldof;
  const int64_t total = n_cell * l2;
  for (int64_t e = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; e < total;
       e += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int64_t c = e / l2;
    const int64_t ij = e - c * l2;
    const T* f = factors + c * nt;
    T v = T(0);
    for (int t = 0; t < nt; ++t) v += f[t] * __ldg(tables + t * l2 + ij);
    out[e] = accumulate ? out[e] + v : v;
  }
}

// P1 elasticity: K[(li, a), (lj, b)] from the factor channels of the CSR
// kernel (grad lambda_{1..GD}, then |T| D00, |T| D_lambda, |T| D_mu):
//   a == b: D00 g_i[a] g_j[a] + D_mu (g_i . g_j - g_i[a] g_j[a])
//   a != b: D_lambda g_i[a] g_j[b] + D_mu g_i[b] g_j[a]
// Local index li * GD + a (interleaved components, priority 0) or
// a * (GD + 1) + li (component-major, priority 1).
template <typename T, int GD>
__global__ void local_elasticity_kernel(int64_t n_cell, const T* __restrict__ factors, int priority,
                                        T* __restrict__ out) {
  constexpr int NV = GD + 1;
  constexpr int LD = NV * GD;
  constexpr int NF = GD * GD + 3;
  const int64_t total = n_cell * LD * LD;
  for (int64_t e = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; e < total;
       e += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int64_t c = e / (LD * LD);
    const int r = static_cast<int>(e - c * LD * LD);
    const int I = r / LD, J = r - (r / LD) * LD;
    int li, a, lj, b;
    if (priority) {
      a = I / NV; li = I - a * NV; b = J / NV; lj = J - b * NV;
    } else {
      li = I / GD; a = I - li * GD; lj = J / GD; b = J - lj * GD;
    }
    const T* f = factors + c * NF;
    T gi[GD], gj[GD];
#pragma unroll
    for (int x = 0; x < GD; ++x) {
      T si = T(0);
#pragma unroll
      for (int k = 0; k < GD; ++k) si += f[k * GD + x];
      gi[x] = li == 0 ? -si : f[(li - 1) * GD + x];
      gj[x] = lj == 0 ? -si : f[(lj - 1) * GD + x];
    }
    const T d00 = f[GD * GD], dl = f[GD * GD + 1], dm = f[GD * GD + 2];
    T dot = T(0);
#pragma unroll
    for (int x = 0; x < GD; ++x) dot += gi[x] * gj[x];
    out[e] = a == b ? d00 * gi[a] * gj[a] + dm * (dot - gi[a] * gj[a]) : dl * gi[a] * gj[b] + dm * gi[b] * gj[a];
  }
}

}  // namespace fgb

using namespace fgb;

extern "C" {

int32_t fgb_local_matrices(int32_t dtype, int64_t n_cell, int32_t ldof, int32_t n_table, const void* tables,
                           const void* factors, void* out, int32_t accumulate, void* stream) {
  if (n_cell < 0 || ldof <= 0 || ldof > 64 || n_table <= 0 || !tables || !factors || !out) return FGB_ERR_ARG;
  if (n_cell == 0) return FGB_OK;
  cudaStream_t st = as_stream(stream);
  const int g = grid_for(n_cell * ldof * ldof, 256, kNumSMs * 16);
  if (dtype == FGB_F64)
    local_matrices_kernel<double><<<g, 256, 0, st>>>(n_cell, ldof, n_table, static_cast<const double*>(factors),
                                                    static_cast<const double*>(tables), static_cast<double*>(out),
                                                    accumulate ? 1 : 0);
  else if (dtype == FGB_F32)
    local_matrices_kernel<float><<<g, 256, 0, st>>>(n_cell, ldof, n_table, static_cast<const float*>(factors),
                                                   static_cast<const float*>(tables), static_cast<float*>(out),
                                                   accumulate ? 1 : 0);
  else
    return FGB_ERR_ARG;
  return launch_status();
}

int32_t fgb_local_elasticity_p1(int32_t dtype, int32_t gd, int64_t n_cell, const void* factors, int32_t priority,
                                void* out, void* stream) {
  if ((gd != 2 && gd != 3) || n_cell < 0 || !factors || !out) return FGB_ERR_ARG;
  if (n_cell == 0) return FGB_OK;
  cudaStream_t st = as_stream(stream);
  const int ld = (gd + 1) * gd;
  const int g = grid_for(n_cell * ld * ld, 256, kNumSMs * 16);
  const int pr = priority ? 1 : 0;
  if (dtype == FGB_F64) {
    if (gd == 3)
      local_elasticity_kernel<double, 3><<<g, 256, 0, st>>>(n_cell, static_cast<const double*>(factors), pr,
                                                          static_cast<double*>(out));
    else
      local_elasticity_kernel<double, 2><<<g, 256, 0, st>>>(n_cell, static_cast<const double*>(factors), pr,
                                                          static_cast<double*>(out));
  } else if (dtype == FGB_F32) {
    if (gd == 3)
      local_elasticity_kernel<float, 3><<<g, 256, 0, st>>>(n_cell, static_cast<const float*>(factors), pr,
                                                         static_cast<float*>(out));
    else
      local_elasticity_kernel<float, 2><<<g, 256, 0, st>>>(n_cell, static_cast<const float*>(factors), pr,
                                                         static_cast<float*>(out));
  } else {
    return FGB_ERR_ARG;
  }
  return launch_status();
}

}  // extern "C"
