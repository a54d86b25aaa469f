// Jacobi-preconditioned CG for several right-hand sides of one matrix, the
// (n, batch) path of fealpy/solver/cg.py:60-123: every column runs its own CG
// recurrence (alpha and beta per column), all columns take the same number of
// iterations, and the stopping test is on sqrt(sum over columns of r.z)
// against atol and rtol * ||B|| (Frobenius norm of all right-hand sides).
//
// B, X, R, Z, P and AP are row-major (n, k): entry (i, c) at i * k + c, so
// a nonzero a_ij meets the k contiguous values of row j.  Threads are laid
// out as (row, column) pairs, k consecutive threads per row; blocks hold a
// whole number of rows, so a thread keeps its column over its grid-stride
// loop and the per-column block sums take a fixed order.  The iterations run
// as a CUDA-graph while node (alpha, beta and the stopping test on the
// device).

#include "fgb_common.cuh"

#include <cmath>
#include <cstring>

namespace fgb {

constexpr int kMrMaxCols = 64;
constexpr int kMrThreads = 256;
constexpr int kMrMaxBlocks = kNumSMs * 8;

struct MrState {
  double rz[kMrMaxCols], rz_new[kMrMaxCols], pap[kMrMaxCols], beta[kMrMaxCols];
  double tol, atol, resid, b_norm;
  long long niter, maxit, trips, trip_cap;
  int done, k;
};

// per-column partial of v over the block's threads (thread t holds column
// t % k): written to part[blockIdx.x * k + c] in row order
__device__ void mr_block_partials(double v, int k, double* sbuf, double* part) {
  sbuf[threadIdx.x] = v;
  __syncthreads();
  const int rows = blockDim.x / k;
  if (threadIdx.x < static_cast<unsigned>(k)) {
    double s = 0.0;
    for (int m = 0; m < rows; ++m) s += sbuf[m * k + threadIdx.x];
    part[static_cast<int64_t>(blockIdx.x) * k + threadIdx.x] = s;
  }
}

#define MR_LOOP(n, k)                                                                                 \
  const int rows_per_block = blockDim.x / (k);                                                        \
  const int c = threadIdx.x % (k);                                                                    \
  const bool lane_ok = threadIdx.x < static_cast<unsigned>(rows_per_block * (k));                     \
  for (int64_t i = static_cast<int64_t>(blockIdx.x) * rows_per_block + threadIdx.x / (k);             \
       lane_ok && i < (n); i += static_cast<int64_t>(gridDim.x) * rows_per_block)

// mode 0: Y = B - A X ; mode 1: Y = A X with per-column partials of X.Y ;
// mode 2: Y = A X (A of any width: X holds k values per column of A)
__global__ void mr_spmm(int64_t n, int k, const int64_t* __restrict__ indptr, const int32_t* __restrict__ indices,
                        const double* __restrict__ values, const double* __restrict__ X,
                        const double* __restrict__ B, double* __restrict__ Y, int mode, double* part) {
  __shared__ double sbuf[kMrThreads];
  double acc_dot = 0.0;
  MR_LOOP(n, k) {
    double s = 0.0;
    for (int64_t e = indptr[i]; e < indptr[i + 1]; ++e) s += values[e] * X[static_cast<int64_t>(indices[e]) * k + c];
    const int64_t o = i * k + c;
    if (mode == 0) {
      Y[o] = B[o] - s;
    } else {
      Y[o] = s;
      if (mode == 1) acc_dot += X[o] * s;
    }
  }
  if (mode == 1) mr_block_partials(acc_dot, k, sbuf, part);
  (void)acc_dot;
}

// Z = D^-1 R (or R), P = Z, per-column partials of R.Z and of B.B
__global__ void mr_init(int64_t n, int k, const double* __restrict__ dinv, const double* __restrict__ R,
                        const double* __restrict__ B, double* __restrict__ Z, double* __restrict__ P, double* part,
                        double* part_b) {
  __shared__ double sbuf[kMrThreads];
  double rz = 0.0, bb = 0.0;
  MR_LOOP(n, k) {
    const int64_t o = i * k + c;
    const double z = dinv ? dinv[i] * R[o] : R[o];
    Z[o] = z;
    P[o] = z;
    rz += R[o] * z;
    bb += B[o] * B[o];
  }
  mr_block_partials(rz, k, sbuf, part);
  __syncthreads();
  mr_block_partials(bb, k, sbuf, part_b);
}

// out[c] = sum over blocks of part[b * k + c] (one block per column, fixed order)
__global__ void mr_column_sums(const double* __restrict__ part, int nb, int k, double* __restrict__ out) {
  __shared__ double ws[32];
  const int c = blockIdx.x;
  double t = 0.0;
  for (int b = threadIdx.x; b < nb; b += blockDim.x) t += part[static_cast<int64_t>(b) * k + c];
  t = warp_sum(t);
  if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = t;
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0.0;
    for (int w = 0; w < static_cast<int>(blockDim.x >> 5); ++w) a += ws[w];
    out[c] = a;
  }
}

// X += alpha P, R -= alpha AP, Z = D^-1 R with alpha_c = rz_c / pap_c (a
// column with rz_c = 0 is exact and stays put; pap_c <= 0 otherwise ends the
// solve as a breakdown); per-column partials of R.Z
__global__ void mr_update(int64_t n, MrState* s, const double* __restrict__ dinv, const double* __restrict__ P,
                          const double* __restrict__ AP, double* __restrict__ X, double* __restrict__ R,
                          double* __restrict__ Z, double* part) {
  __shared__ double sbuf[kMrThreads];
  const int k = s->k;
  double rz = 0.0;
  {
    MR_LOOP(n, k) {
      const double pap = s->pap[c], rzc = s->rz[c];
      const double alpha = (rzc == 0.0 || !(pap > 0.0)) ? 0.0 : rzc / pap;
      const int64_t o = i * k + c;
      X[o] += alpha * P[o];
      const double r = R[o] - alpha * AP[o];
      R[o] = r;
      const double z = dinv ? dinv[i] * r : r;
      Z[o] = z;
      rz += r * z;
    }
  }
  mr_block_partials(rz, k, sbuf, part);
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    for (int c = 0; c < k; ++c) {
      const double pap = s->pap[c];
      if (s->rz[c] != 0.0 && !(pap > 0.0)) s->done = isfinite(pap) ? FGB_PCG_BREAKDOWN : FGB_PCG_NONFINITE;
    }
  }
}

// stopping test and beta (one thread), then the while condition
__global__ void mr_ctl(MrState* s, cudaGraphConditionalHandle handle) {
  if (!s->done) {
    double sum = 0.0;
    for (int c = 0; c < s->k; ++c) sum += s->rz_new[c];
    const double res = sqrt(sum);
    s->niter += 1;
    s->resid = res;
    if (!isfinite(res)) s->done = FGB_PCG_NONFINITE;
    else if (res < s->atol) s->done = FGB_PCG_ATOL;
    else if (res < s->tol) s->done = FGB_PCG_RTOL;
    else if (s->niter >= s->maxit) s->done = FGB_PCG_MAXIT;
    else
      for (int c = 0; c < s->k; ++c) {
        s->beta[c] = s->rz[c] != 0.0 ? s->rz_new[c] / s->rz[c] : 0.0;
        s->rz[c] = s->rz_new[c];
      }
  }
  s->trips += 1;
  if (!s->done && s->trips >= s->trip_cap) s->done = FGB_PCG_MAXIT;
  if (s->done) cudaGraphSetConditional(handle, 0);
}

// P = Z + beta P (nothing once the solve has ended)
__global__ void mr_pupdate(int64_t n, const MrState* s, const double* __restrict__ Z, double* __restrict__ P) {
  if (s->done) return;
  const int k = s->k;
  MR_LOOP(n, k) {
    const int64_t o = i * k + c;
    P[o] = Z[o] + s->beta[c] * P[o];
  }
}

inline int mr_blocks(int64_t n, int k) {
  const int rows = kMrThreads / k;
  return grid_for(n, rows, kMrMaxBlocks);
}

}  // namespace fgb

using namespace fgb;

extern "C" {

size_t fgb_pcg_multi_workspace_bytes(int64_t n, int32_t k) {
  if (n <= 0 || k <= 0 || k > kMrMaxCols) return 0;
  const size_t nk = static_cast<size_t>(n) * k;
  return 4 * align_up(nk * sizeof(double)) + 2 * align_up(static_cast<size_t>(kMrMaxBlocks) * k * sizeof(double)) +
         align_up(sizeof(MrState));
}

int32_t fgb_pcg_multi_f64(int64_t n, int32_t k, const int64_t* indptr, const int32_t* indices, const double* values,
                          const double* dinv, const double* B, double* X, double atol, double rtol, int64_t maxit,
                          fgb_pcg_info* info, void* workspace, size_t workspace_bytes, void* stream) {
  if (n <= 0 || k <= 0 || k > kMrMaxCols || !indptr || !indices || !values || !B || !X || maxit <= 0)
    return FGB_ERR_ARG;
  if (!workspace || workspace_bytes < fgb_pcg_multi_workspace_bytes(n, k)) return FGB_ERR_WORKSPACE;
  cudaStream_t st = as_stream(stream);
  Carver cv(workspace, workspace_bytes);
  const int64_t nk = n * k;
  double* R = cv.take<double>(nk);
  double* Z = cv.take<double>(nk);
  double* P = cv.take<double>(nk);
  double* AP = cv.take<double>(nk);
  double* part = cv.take<double>(static_cast<int64_t>(kMrMaxBlocks) * k);
  double* part_b = cv.take<double>(static_cast<int64_t>(kMrMaxBlocks) * k);
  MrState* s = cv.take<MrState>(1);
  if (!cv.ok) return FGB_ERR_WORKSPACE;
  const int nb = mr_blocks(n, k);
  // R = B - A X, Z = M R, P = Z, rz_c, ||B||
  mr_spmm<<<nb, kMrThreads, 0, st>>>(n, k, indptr, indices, values, X, B, R, 0, nullptr);
  mr_init<<<nb, kMrThreads, 0, st>>>(n, k, dinv, R, B, Z, P, part, part_b);
  mr_column_sums<<<k, 256, 0, st>>>(part, nb, k, s->rz);
  mr_column_sums<<<k, 256, 0, st>>>(part_b, nb, k, s->rz_new);  // B.B per column, read once below
  MrState h;
  if (cudaMemcpyAsync(&h, s, sizeof(h), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return FGB_ERR_CUDA;
  double bb = 0.0;
  for (int c = 0; c < k; ++c) bb += h.rz_new[c];
  const double b_norm = sqrt(bb);
  int reason = FGB_PCG_RUNNING;
  int64_t launches = 4;
  if (b_norm < 1e-15) {
    // FEALPy returns zeros for a zero right-hand side
    if (cudaMemsetAsync(X, 0, nk * sizeof(double), st) != cudaSuccess) return FGB_ERR_CUDA;
    reason = FGB_PCG_ZERO_RHS;
    h.niter = 0;
    h.resid = 0.0;
  } else {
    h.tol = rtol * b_norm;
    h.atol = atol;
    h.b_norm = b_norm;
    h.resid = 0.0;
    h.niter = 0;
    h.maxit = maxit;
    h.trips = 0;
    h.trip_cap = maxit + 1;
    h.done = 0;
    h.k = k;
    if (cudaMemcpyAsync(s, &h, sizeof(h), cudaMemcpyHostToDevice, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
      return FGB_ERR_CUDA;
    cudaGraph_t g = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaStream_t cs = nullptr;
    int rc = FGB_OK;
    do {
      if (cudaGraphCreate(&g, 0) != cudaSuccess) { g = nullptr; rc = FGB_ERR_CUDA; break; }
      cudaGraphConditionalHandle hw;
      if (cudaGraphConditionalHandleCreate(&hw, g, 1, cudaGraphCondAssignDefault) != cudaSuccess) { rc = FGB_ERR_CUDA; break; }
      cudaGraphNodeParams wp = {};
      wp.type = cudaGraphNodeTypeConditional;
      wp.conditional.handle = hw;
      wp.conditional.type = cudaGraphCondTypeWhile;
      wp.conditional.size = 1;
      cudaGraphNode_t wnode;
      if (cudaGraphAddNode(&wnode, g, nullptr, nullptr, 0, &wp) != cudaSuccess) { rc = FGB_ERR_CUDA; break; }
      if (cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking) != cudaSuccess) { cs = nullptr; rc = FGB_ERR_CUDA; break; }
      if (cudaStreamBeginCaptureToGraph(cs, wp.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                        cudaStreamCaptureModeRelaxed) != cudaSuccess) {
        rc = FGB_ERR_CUDA;
        break;
      }
      mr_spmm<<<nb, kMrThreads, 0, cs>>>(n, k, indptr, indices, values, P, nullptr, AP, 1, part);
      mr_column_sums<<<k, 256, 0, cs>>>(part, nb, k, s->pap);
      mr_update<<<nb, kMrThreads, 0, cs>>>(n, s, dinv, P, AP, X, R, Z, part);
      mr_column_sums<<<k, 256, 0, cs>>>(part, nb, k, s->rz_new);
      mr_ctl<<<1, 1, 0, cs>>>(s, hw);
      mr_pupdate<<<nb, kMrThreads, 0, cs>>>(n, s, Z, P);
      cudaGraph_t captured = nullptr;
      if (cudaStreamEndCapture(cs, &captured) != cudaSuccess) { rc = FGB_ERR_CUDA; break; }
      if (cudaGraphInstantiate(&exec, g, 0) != cudaSuccess) { exec = nullptr; rc = FGB_ERR_CUDA; break; }
      if (cudaGraphLaunch(exec, st) != cudaSuccess) { rc = FGB_ERR_CUDA; break; }
      if (cudaMemcpyAsync(&h, s, sizeof(h), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
          cudaStreamSynchronize(st) != cudaSuccess)
        rc = FGB_ERR_CUDA;
    } while (false);
    if (exec) cudaGraphExecDestroy(exec);
    if (g) cudaGraphDestroy(g);
    if (cs) cudaStreamDestroy(cs);
    if (rc) {
      cudaGetLastError();
      return rc;
    }
    reason = h.done;
    launches += 6 * h.trips;
  }
  if (cudaStreamSynchronize(st) != cudaSuccess) return FGB_ERR_CUDA;
  if (info) {
    memset(info, 0, sizeof(*info));
    info->niter = h.niter;
    info->residual = h.resid;
    info->b_norm = b_norm;
    info->true_relres = -1.0;
    info->reason = reason;
    info->launches = launches;
    info->graph = reason == FGB_PCG_ZERO_RHS ? 0 : 1;
  }
  if (reason == FGB_PCG_BREAKDOWN) return FGB_ERR_BREAKDOWN;
  if (reason == FGB_PCG_NONFINITE) return FGB_ERR_NONFINITE;
  return launch_status();
}

int32_t fgb_csr_spmm_f64(int64_t n_row, int32_t k, const int64_t* indptr, const int32_t* indices,
                         const double* values, const double* X, double* Y, void* stream) {
  if (n_row <= 0 || k <= 0 || k > kMrMaxCols || !indptr || !indices || !values || !X || !Y) return FGB_ERR_ARG;
  cudaStream_t st = as_stream(stream);
  mr_spmm<<<mr_blocks(n_row, k), kMrThreads, 0, st>>>(n_row, k, indptr, indices, values, X, nullptr, Y, 2, nullptr);
  return launch_status();
}

}  // extern "C"
