// Right-hand sides of scalar sources: ScalarSourceIntegrator.assembly
// (fealpy/fem/scalar_source_integrator.py:51-58, linear_integral of
// fealpy/functional.py) and LinearForm.assembly's scatter
// (fealpy/fem/linear_form.py:36-86).
//
// The cell vector of cell c is  b_c[i] = |T_c| sum_q w_q phi_i(q) f(c, q)
// with the source f given as one number (mode 0), one value per cell (mode 1)
// or one value per quadrature point (mode 2, f (NC, NQ) row-major).
// wphi (NQ x ldof) holds w_q phi_i(q) and sv (ldof) its column sums.
// fgb_source_local writes the cell vectors; fgb_source_gather forms them on
// the fly per dof over the dof -> (cell, local) adjacency, in adjacency order
// (deterministic), so the global vector needs no cell-vector array.

#include "fgb_common.cuh"

namespace fgb {

__device__ __forceinline__ double source_term(int mode, int64_t c, int li, int ldof, int nq, double f_scalar,
                                              const double* __restrict__ f, const double* __restrict__ wphi,
                                              const double* __restrict__ sv) {
  if (mode == 0) return sv[li] * f_scalar;
  if (mode == 1) return sv[li] * f[c];
  double s = 0.0;
  for (int q = 0; q < nq; ++q) s += wphi[q * ldof + li] * f[c * nq + q];
  return s;
}

__global__ void source_local_kernel(int64_t n_cell, int ldof, int nq, const double* __restrict__ cm, int mode,
                                    double f_scalar, const double* __restrict__ f, const double* __restrict__ wphi,
                                    const double* __restrict__ sv, double* __restrict__ out) {
  const int64_t total = n_cell * ldof;
  for (int64_t e = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; e < total;
       e += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int64_t c = e / ldof;
    const int li = static_cast<int>(e - c * ldof);
    out[e] = cm[c] * source_term(mode, c, li, ldof, nq, f_scalar, f, wphi, sv);
  }
}

__global__ void source_gather_kernel(int64_t n_dof, const int64_t* __restrict__ adj_ptr,
                                     const int32_t* __restrict__ adj, int ldof, int nq,
                                     const double* __restrict__ cm, int mode, double f_scalar,
                                     const double* __restrict__ f, const double* __restrict__ wphi,
                                     const double* __restrict__ sv, double* __restrict__ out, int accumulate) {
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n_dof;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    double s = 0.0;
    for (int64_t k = adj_ptr[i]; k < adj_ptr[i + 1]; ++k) {
      const int32_t en = adj[k];
      const int64_t c = en / ldof;
      const int li = en - static_cast<int>(c) * ldof;
      s += cm[c] * source_term(mode, c, li, ldof, nq, f_scalar, f, wphi, sv);
    }
    out[i] = accumulate ? out[i] + s : s;
  }
}

}  // namespace fgb

using namespace fgb;

extern "C" {

int32_t fgb_source_local(int64_t n_cell, int32_t ldof, int32_t nq, const double* cm, int32_t mode, double f_scalar,
                         const double* f, const double* wphi, const double* sv, double* out, void* stream) {
  if (n_cell < 0 || ldof <= 0 || nq <= 0 || mode < 0 || mode > 2 || !cm || !wphi || !sv || !out ||
      (mode > 0 && !f))
    return FGB_ERR_ARG;
  if (n_cell == 0) return FGB_OK;
  source_local_kernel<<<grid_for(n_cell * ldof, 256, kNumSMs * 16), 256, 0, as_stream(stream)>>>(
      n_cell, ldof, nq, cm, mode, f_scalar, f, wphi, sv, out);
  return launch_status();
}

int32_t fgb_source_gather(int64_t n_dof, const int64_t* adj_ptr, const int32_t* adj, int32_t ldof, int32_t nq,
                          const double* cm, int32_t mode, double f_scalar, const double* f, const double* wphi,
                          const double* sv, double* out, int32_t accumulate, void* stream) {
  if (n_dof < 0 || ldof <= 0 || nq <= 0 || mode < 0 || mode > 2 || !adj_ptr || !adj || !cm || !wphi || !sv ||
      !out || (mode > 0 && !f))
    return FGB_ERR_ARG;
  if (n_dof == 0) return FGB_OK;
  source_gather_kernel<<<grid_for(n_dof, 256, kNumSMs * 16), 256, 0, as_stream(stream)>>>(
      n_dof, adj_ptr, adj, ldof, nq, cm, mode, f_scalar, f, wphi, sv, out, accumulate ? 1 : 0);
  return launch_status();
}

}  // extern "C"
