// CSR SpMV, Jacobi diagonal and the Jacobi-preconditioned CG solvers.
//
// The reference CG (fealpy/solver/cg.py:76-123) issues, per iteration, two
// SpMVs (A p and the diagonal-CSR M r), two dots and three axpys, each a
// separate array operation, and reads two scalars back to the host for its
// stopping test.  Here one iteration is two kernels with every scalar kept on
// the device:
//
//   A: p_new = z + beta p_old (formed on the fly for every gathered column),
//      Ap = A p_new, partial p_new.Ap;   last block: alpha = rz / pAp
//   B: x += alpha p_new, r -= alpha Ap, z = D^-1 r, partial r.z (and r.r);
//      last block: convergence test, beta, rz
//
// p is double-buffered (A reads p_old of neighbour rows while writing p_new of
// its own rows).  Dots are reduced deterministically: per-block partials in
// FP64, combined in index order by the last block (threadfence + counter).
// After convergence every further launch returns at once, so the host only
// polls the `done` word every `check_every` iterations.

#include "fgb_common.cuh"

#include <cmath>
#include <cstring>

namespace fgb {

// ---------------------------------------------------------------------------
// SpMV: G lanes per row
// ---------------------------------------------------------------------------
template <typename T, int G>
__global__ void spmv_kernel(int64_t n, const int64_t* __restrict__ indptr, const int32_t* __restrict__ indices,
                            const T* __restrict__ values, const T* __restrict__ x, T* __restrict__ y) {
  const int sub = threadIdx.x & (G - 1);
  const int64_t grp = (blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x) / G;
  const int64_t ngrp = (static_cast<int64_t>(gridDim.x) * blockDim.x) / G;
  // every thread runs the same number of trips so the group shuffles stay converged
  const int64_t nround = ((n + ngrp - 1) / ngrp) * ngrp;
  for (int64_t i = grp; i < nround; i += ngrp) {
    T acc = T(0);
    if (i < n) {
      const int64_t s = indptr[i], e = indptr[i + 1];
      for (int64_t k = s + sub; k < e; k += G) acc += ld_stream(values + k) * __ldg(x + ld_stream(indices + k));
    }
    acc = group_sum(acc, G);
    if (i < n && sub == 0) y[i] = acc;
  }
}

template <typename T>
int spmv_dispatch(int64_t n, const int64_t* indptr, const int32_t* indices, const T* values, const T* x, T* y,
                  int lanes, cudaStream_t st) {
  const int threads = 256;
  auto grid = [&](int g) { return grid_for(n * g, threads, kNumSMs * 32); };
  switch (lanes) {
    case 1: spmv_kernel<T, 1><<<grid(1), threads, 0, st>>>(n, indptr, indices, values, x, y); break;
    case 2: spmv_kernel<T, 2><<<grid(2), threads, 0, st>>>(n, indptr, indices, values, x, y); break;
    case 4: spmv_kernel<T, 4><<<grid(4), threads, 0, st>>>(n, indptr, indices, values, x, y); break;
    case 8: spmv_kernel<T, 8><<<grid(8), threads, 0, st>>>(n, indptr, indices, values, x, y); break;
    case 16: spmv_kernel<T, 16><<<grid(16), threads, 0, st>>>(n, indptr, indices, values, x, y); break;
    case 32: spmv_kernel<T, 32><<<grid(32), threads, 0, st>>>(n, indptr, indices, values, x, y); break;
    default: return FGB_ERR_ARG;
  }
  return launch_status();
}

// Lanes per row from the mean row length (an initial choice; the Python side
// keeps a measured per-shape table, see fealpy_gb300/tuning.py).
inline int auto_lanes(int64_t n, int64_t nnz) {
  double avg = n > 0 ? static_cast<double>(nnz) / n : 1.0;
  if (avg <= 3) return 2;
  if (avg <= 12) return 4;
  if (avg <= 24) return 8;
  if (avg <= 48) return 16;
  return 32;
}

template <typename T>
__global__ void diagonal_kernel(int64_t n, const int64_t* __restrict__ indptr, const int32_t* __restrict__ indices,
                                const T* __restrict__ values, T* __restrict__ diag, T* __restrict__ diag_inv) {
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int64_t s = indptr[i], e = indptr[i + 1];
    int64_t lo = s, hi = e;
    while (lo < hi) {
      int64_t mid = (lo + hi) >> 1;
      if (indices[mid] < i) lo = mid + 1; else hi = mid;
    }
    T d = (lo < e && indices[lo] == i) ? values[lo] : T(0);
    if (diag) diag[i] = d;
    if (diag_inv) diag_inv[i] = T(1) / d;
  }
}

// ---------------------------------------------------------------------------
// PCG state kept on the device
// ---------------------------------------------------------------------------
struct PcgState {
  double rz;        // r.z of the current iterate
  double rz_prev;   // r.z of the previous iterate (mixed: beta after a replacement)
  double rr;        // r.r (FP32-iterated residual, mixed solver)
  double alpha, beta;
  double b_norm;
  double tol;       // stopping threshold on the monitored norm
  double atol;
  double resid;     // monitored norm at the last test
  double r_upd;     // mixed: ||r|| right after the last reliable update
  double true_rel;  // mixed: last true relative residual
  long long niter;
  long long maxit;
  int done;         // 0 running, else an fgb_pcg_reason
  int need_update;  // mixed: a reliable update is due this iteration
  int n_updates;
  int norm_rr;      // monitor sqrt(r.r) instead of sqrt(r.z)
  unsigned int counter[4];
};

constexpr int kPcgThreads = 256;
constexpr int kPcgMaxBlocks = kNumSMs * 8;

// Last-block-done reduction of up to two FP64 partials per block.  Returns true
// in the (single) block that arrives last; that block finds the totals in
// out0/out1 (valid in thread 0).
__device__ bool last_block_reduce(double v0, double v1, double* partials, unsigned int* counter, double* out0,
                                  double* out1) {
  __shared__ double red[kPcgThreads / 32];
  __shared__ bool am_last;
  double s0 = block_sum(v0, red);
  __syncthreads();
  double s1 = block_sum(v1, red);
  if (threadIdx.x == 0) {
    partials[blockIdx.x] = s0;
    partials[kPcgMaxBlocks + blockIdx.x] = s1;
    __threadfence();
    unsigned int t = atomicAdd(counter, 1u);
    am_last = (t == gridDim.x - 1);
  }
  __syncthreads();
  if (!am_last) return false;
  __threadfence();
  double a = 0.0, b = 0.0;
  for (int k = threadIdx.x; k < static_cast<int>(gridDim.x); k += blockDim.x) {
    a += __ldcg(partials + k);
    b += __ldcg(partials + kPcgMaxBlocks + k);
  }
  __syncthreads();
  a = block_sum(a, red);
  __syncthreads();
  b = block_sum(b, red);
  if (threadIdx.x == 0) {
    *out0 = a;
    *out1 = b;
    *counter = 0u;
  }
  return true;
}

// r = b - A x, z = Dinv r, p = z ; rz, b.b (and r.r)
template <typename T, int G>
__global__ void __launch_bounds__(kPcgThreads) pcg_init_kernel(int64_t n, const int64_t* __restrict__ indptr,
                                                               const int32_t* __restrict__ indices,
                                                               const T* __restrict__ values, const T* __restrict__ dinv,
                                                               const T* __restrict__ b, const T* __restrict__ x,
                                                               T* __restrict__ r, T* __restrict__ z, T* __restrict__ p,
                                                               double* partials, PcgState* st) {
  const int sub = threadIdx.x & (G - 1);
  const int64_t grp = (blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x) / G;
  const int64_t ngrp = (static_cast<int64_t>(gridDim.x) * blockDim.x) / G;
  double rz = 0.0, bb = 0.0;
  const int64_t nround = ((n + ngrp - 1) / ngrp) * ngrp;
  for (int64_t i = grp; i < nround; i += ngrp) {
    T acc = T(0);
    if (i < n) {
      const int64_t s = indptr[i], e = indptr[i + 1];
      for (int64_t k = s + sub; k < e; k += G) acc += values[k] * x[indices[k]];
    }
    acc = group_sum(acc, G);
    if (i < n && sub == 0) {
      const T bi = b[i];
      const T ri = bi - acc;
      const T zi = dinv ? dinv[i] * ri : ri;
      r[i] = ri; z[i] = zi; p[i] = zi;
      rz += static_cast<double>(ri) * static_cast<double>(zi);
      bb += static_cast<double>(bi) * static_cast<double>(bi);
    }
  }
  double trz, tbb;
  if (last_block_reduce(rz, bb, partials, &st->counter[0], &trz, &tbb) && threadIdx.x == 0) {
    st->rz = trz;
    st->b_norm = sqrt(tbb);
    st->beta = 0.0;
    st->niter = 0;
    st->n_updates = 0;
    st->need_update = 0;
    if (st->b_norm < 1e-15) st->done = FGB_PCG_ZERO_RHS;
  }
}

// Kernel A: p_new = z + beta p_old ; Ap = A p_new ; alpha = rz / (p_new . Ap)
template <typename T, int G>
__global__ void __launch_bounds__(kPcgThreads) pcg_spmv_kernel(int64_t n, const int64_t* __restrict__ indptr,
                                                               const int32_t* __restrict__ indices,
                                                               const T* __restrict__ values, const T* __restrict__ z,
                                                               const T* __restrict__ p_old, T* __restrict__ p_new,
                                                               T* __restrict__ Ap, double* partials, PcgState* st) {
  if (st->done) return;
  const T beta = static_cast<T>(st->beta);
  const int sub = threadIdx.x & (G - 1);
  const int64_t grp = (blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x) / G;
  const int64_t ngrp = (static_cast<int64_t>(gridDim.x) * blockDim.x) / G;
  double pap = 0.0;
  const int64_t nround = ((n + ngrp - 1) / ngrp) * ngrp;
  for (int64_t i = grp; i < nround; i += ngrp) {
    T acc = T(0);
    if (i < n) {
      const int64_t s = indptr[i], e = indptr[i + 1];
      for (int64_t k = s + sub; k < e; k += G) {
        const int32_t j = ld_stream(indices + k);
        acc += ld_stream(values + k) * (z[j] + beta * p_old[j]);
      }
    }
    acc = group_sum(acc, G);
    if (i < n && sub == 0) {
      const T pi = z[i] + beta * p_old[i];
      p_new[i] = pi;
      Ap[i] = acc;
      pap += static_cast<double>(pi) * static_cast<double>(acc);
    }
  }
  double tpap, unused;
  if (last_block_reduce(pap, 0.0, partials, &st->counter[1], &tpap, &unused) && threadIdx.x == 0) {
    if (!(tpap > 0.0) || !isfinite(tpap)) {
      st->done = isfinite(tpap) ? FGB_PCG_BREAKDOWN : FGB_PCG_NONFINITE;
      st->alpha = 0.0;
    } else {
      st->alpha = st->rz / tpap;
    }
  }
}

// Kernel B (FP64 solver): x += alpha p ; r -= alpha Ap ; z = Dinv r ; stopping test ; beta
template <typename T>
__global__ void __launch_bounds__(kPcgThreads) pcg_update_kernel(int64_t n, const T* __restrict__ dinv,
                                                                 const T* __restrict__ p, const T* __restrict__ Ap,
                                                                 T* __restrict__ x, T* __restrict__ r,
                                                                 T* __restrict__ z, double* partials, PcgState* st) {
  if (st->done) return;
  const T alpha = static_cast<T>(st->alpha);
  double rz = 0.0, rr = 0.0;
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const T pi = p[i];
    x[i] += alpha * pi;
    const T ri = r[i] - alpha * Ap[i];
    const T zi = dinv ? dinv[i] * ri : ri;
    r[i] = ri;
    z[i] = zi;
    rz += static_cast<double>(ri) * static_cast<double>(zi);
    rr += static_cast<double>(ri) * static_cast<double>(ri);
  }
  double trz, trr;
  if (last_block_reduce(rz, rr, partials, &st->counter[2], &trz, &trr) && threadIdx.x == 0) {
    st->niter += 1;
    const double res = st->norm_rr ? sqrt(trr) : sqrt(trz);
    st->resid = res;
    st->rr = trr;
    if (!isfinite(res)) st->done = FGB_PCG_NONFINITE;
    else if (res < st->atol) st->done = FGB_PCG_ATOL;
    else if (res < st->tol) st->done = FGB_PCG_RTOL;
    else if (st->niter >= st->maxit) st->done = FGB_PCG_MAXIT;
    st->beta = trz / st->rz;
    st->rz = trz;
  }
}

// ---------------------------------------------------------------------------
// mixed precision (FP32 iterations, FP64 reliable updates)
// ---------------------------------------------------------------------------
// Kernel B (mixed): y += alpha p ; r -= alpha Ap ; z = Dinv r (all FP32) ;
// decides whether a reliable update is due.
__global__ void __launch_bounds__(kPcgThreads) mixed_update_kernel(int64_t n, const float* __restrict__ dinv,
                                                                   const float* __restrict__ p,
                                                                   const float* __restrict__ Ap, float* __restrict__ y,
                                                                   float* __restrict__ r, float* __restrict__ z,
                                                                   double* partials, PcgState* st, double delta) {
  if (st->done) return;
  const float alpha = static_cast<float>(st->alpha);
  double rz = 0.0, rr = 0.0;
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const float pi = p[i];
    y[i] += alpha * pi;
    const float ri = r[i] - alpha * Ap[i];
    const float zi = dinv[i] * ri;
    r[i] = ri;
    z[i] = zi;
    rz += static_cast<double>(ri) * static_cast<double>(zi);
    rr += static_cast<double>(ri) * static_cast<double>(ri);
  }
  double trz, trr;
  if (last_block_reduce(rz, rr, partials, &st->counter[2], &trz, &trr) && threadIdx.x == 0) {
    st->niter += 1;
    const double res = sqrt(trr);
    st->resid = res;
    st->rr = trr;
    if (!isfinite(res)) {
      st->done = FGB_PCG_NONFINITE;
    } else {
      st->need_update = (res < delta * st->r_upd) || (res < st->tol) || (st->niter >= st->maxit);
    }
    st->rz_prev = st->rz;
    st->beta = trz / st->rz;
    st->rz = trz;
  }
}

// Reliable update, part 1: x += y (FP64), y = 0, r64 = b - A64 x ; ||r64||^2
template <int G>
__global__ void __launch_bounds__(kPcgThreads) mixed_residual_kernel(int64_t n, const int64_t* __restrict__ indptr,
                                                                     const int32_t* __restrict__ indices,
                                                                     const double* __restrict__ values,
                                                                     const double* __restrict__ b, double* __restrict__ x,
                                                                     float* __restrict__ y, double* __restrict__ r64,
                                                                     double* partials, PcgState* st, int first) {
  if (!first && (st->done || !st->need_update)) return;
  // fold the FP32 correction into the FP64 iterate (own rows), then a grid-wide
  // dependency: the SpMV below reads x of neighbour rows.  That dependency is
  // honoured by running the fold in a separate launch (mixed_fold_kernel); this
  // kernel only computes the residual.
  const int sub = threadIdx.x & (G - 1);
  const int64_t grp = (blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x) / G;
  const int64_t ngrp = (static_cast<int64_t>(gridDim.x) * blockDim.x) / G;
  double rr = 0.0;
  const int64_t nround = ((n + ngrp - 1) / ngrp) * ngrp;
  for (int64_t i = grp; i < nround; i += ngrp) {
    double acc = 0.0;
    if (i < n) {
      const int64_t s = indptr[i], e = indptr[i + 1];
      for (int64_t k = s + sub; k < e; k += G) acc += ld_stream(values + k) * x[ld_stream(indices + k)];
    }
    acc = group_sum(acc, G);
    if (i < n && sub == 0) {
      const double ri = b[i] - acc;
      r64[i] = ri;
      rr += ri * ri;
    }
  }
  double trr, unused;
  if (last_block_reduce(rr, 0.0, partials, &st->counter[3], &trr, &unused) && threadIdx.x == 0) {
    const double rel = st->b_norm > 0.0 ? sqrt(trr) / st->b_norm : 0.0;
    st->true_rel = rel;
    st->resid = sqrt(trr);
    if (!first) st->n_updates += 1;
    if (!isfinite(rel)) st->done = FGB_PCG_NONFINITE;
    else if (st->b_norm < 1e-15) st->done = FGB_PCG_ZERO_RHS;
    else if (sqrt(trr) <= st->tol) st->done = FGB_PCG_RTOL;
    else if (st->niter >= st->maxit) st->done = FGB_PCG_MAXIT;
  }
}

__global__ void mixed_fold_kernel(int64_t n, double* __restrict__ x, float* __restrict__ y, const PcgState* st,
                                  int first) {
  if (!first && (st->done || !st->need_update)) return;
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    x[i] += static_cast<double>(y[i]);
    y[i] = 0.0f;
  }
}

// Reliable update, part 2: r = float(r64), z = Dinv r, rz ; restart p on the
// first call, otherwise keep the direction and recompute beta from the new rz.
__global__ void __launch_bounds__(kPcgThreads) mixed_replace_kernel(int64_t n, const double* __restrict__ dinv64,
                                                                    const double* __restrict__ r64,
                                                                    float* __restrict__ r, float* __restrict__ z,
                                                                    float* __restrict__ p, float* __restrict__ dinv32,
                                                                    double* partials, PcgState* st, double rz_prev_in,
                                                                    int first) {
  if (!first && !st->need_update) return;
  if (!first && st->done) return;
  double rz = 0.0, rr = 0.0;
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const float ri = static_cast<float>(r64[i]);
    const float di = first ? static_cast<float>(dinv64[i]) : dinv32[i];
    if (first) dinv32[i] = di;
    const float zi = di * ri;
    r[i] = ri;
    z[i] = zi;
    if (first) p[i] = zi;
    rz += static_cast<double>(ri) * static_cast<double>(zi);
    rr += static_cast<double>(ri) * static_cast<double>(ri);
  }
  double trz, trr;
  if (last_block_reduce(rz, rr, partials, &st->counter[0], &trz, &trr) && threadIdx.x == 0) {
    if (first) {
      st->beta = 0.0;
    } else {
      // the update kernel already advanced rz to the iterated value; the CG
      // direction update must use the replaced residual instead
      st->beta = trz / st->rz_prev;
    }
    st->rz = trz;
    st->rr = trr;
    st->r_upd = sqrt(trr);
    st->need_update = 0;
  }
}

template <int G>
void mixed_launch_iteration(int64_t n, const int64_t* indptr, const int32_t* indices, const double* values64,
                            const float* values32, const double* dinv64, const double* b, double* x, float* y,
                            float* r, float* z, float* p0, float* p1, float* Ap, double* r64, float* dinv32,
                            double* partials, PcgState* st, double delta, int64_t it, int grid_rows, int grid_vec,
                            cudaEvent_t ev0, cudaEvent_t ev1, cudaStream_t s) {
  float* p_old = (it & 1) ? p1 : p0;
  float* p_new = (it & 1) ? p0 : p1;
  if (ev0) cudaEventRecord(ev0, s);
  pcg_spmv_kernel<float, G><<<grid_rows, kPcgThreads, 0, s>>>(n, indptr, indices, values32, z, p_old, p_new, Ap,
                                                              partials, st);
  if (ev1) cudaEventRecord(ev1, s);
  mixed_update_kernel<<<grid_vec, kPcgThreads, 0, s>>>(n, dinv32, p_new, Ap, y, r, z, partials, st, delta);
  mixed_fold_kernel<<<grid_vec, kPcgThreads, 0, s>>>(n, x, y, st, 0);
  mixed_residual_kernel<G><<<grid_rows, kPcgThreads, 0, s>>>(n, indptr, indices, values64, b, x, y, r64, partials,
                                                             st, 0);
  mixed_replace_kernel<<<grid_vec, kPcgThreads, 0, s>>>(n, dinv64, r64, r, z, p_new, dinv32, partials, st, 0.0, 0);
}

}  // namespace fgb

using namespace fgb;

namespace {

// CUDA-event timing of the SpMV launch of each iteration of a chunk.  Only the
// iterations that did work (counted by the device iteration counter) are summed,
// so the no-op launches after convergence do not dilute the average.
struct SpmvProfiler {
  bool on = false;
  int cap = 0;
  cudaEvent_t* ev = nullptr;
  double ms = 0.0;
  int64_t launches = 0;
  SpmvProfiler(bool enable, int chunk) : on(enable), cap(chunk) {
    if (!on) return;
    ev = new cudaEvent_t[2 * cap];
    for (int k = 0; k < 2 * cap; ++k) cudaEventCreate(&ev[k]);
  }
  ~SpmvProfiler() {
    if (!ev) return;
    for (int k = 0; k < 2 * cap; ++k) cudaEventDestroy(ev[k]);
    delete[] ev;
  }
  cudaEvent_t before(int k) const { return on ? ev[2 * k] : nullptr; }
  cudaEvent_t after(int k) const { return on ? ev[2 * k + 1] : nullptr; }
  void collect(int64_t executed) {
    if (!on) return;
    for (int64_t k = 0; k < executed && k < cap; ++k) {
      float t = 0.0f;
      if (cudaEventElapsedTime(&t, ev[2 * k], ev[2 * k + 1]) == cudaSuccess) {
        ms += t;
        ++launches;
      }
    }
  }
};

struct PcgBuffers {
  PcgState* st = nullptr;
  double* partials = nullptr;
};

template <typename T>
struct Vecs {
  T *r, *z, *p0, *p1, *Ap;
};

int grid_rows_for(int64_t n, int G) { return grid_for(n * G, kPcgThreads, kPcgMaxBlocks); }
int grid_vec_for(int64_t n) { return grid_for(n, kPcgThreads, kPcgMaxBlocks); }

template <typename T, int G>
void f64_iteration(int64_t n, const int64_t* indptr, const int32_t* indices, const T* values, const T* dinv, T* x,
                   Vecs<T>& v, PcgBuffers& pb, int64_t it, cudaEvent_t ev0, cudaEvent_t ev1, cudaStream_t s) {
  T* p_old = (it & 1) ? v.p1 : v.p0;
  T* p_new = (it & 1) ? v.p0 : v.p1;
  if (ev0) cudaEventRecord(ev0, s);
  pcg_spmv_kernel<T, G><<<grid_rows_for(n, G), kPcgThreads, 0, s>>>(n, indptr, indices, values, v.z, p_old, p_new,
                                                                    v.Ap, pb.partials, pb.st);
  if (ev1) cudaEventRecord(ev1, s);
  pcg_update_kernel<T><<<grid_vec_for(n), kPcgThreads, 0, s>>>(n, dinv, p_new, v.Ap, x, v.r, v.z, pb.partials, pb.st);
}

int finish_status(int done) {
  return done == FGB_PCG_BREAKDOWN ? FGB_ERR_BREAKDOWN : (done == FGB_PCG_NONFINITE ? FGB_ERR_NONFINITE : FGB_OK);
}

template <int G>
int run_pcg_f64(int64_t n, const int64_t* indptr, const int32_t* indices, const double* values, const double* dinv,
                const double* b, double* x, double atol, double rtol, int64_t maxit, int check_every, int norm_rr,
                int profile, Carver& cv, fgb_pcg_info* info, cudaStream_t s) {
  PcgBuffers pb;
  pb.st = cv.take<PcgState>(1);
  pb.partials = cv.take<double>(2 * kPcgMaxBlocks);
  Vecs<double> v;
  v.r = cv.take<double>(n); v.z = cv.take<double>(n); v.p0 = cv.take<double>(n); v.p1 = cv.take<double>(n);
  v.Ap = cv.take<double>(n);
  if (!cv.ok) return FGB_ERR_WORKSPACE;
  SpmvProfiler prof(profile != 0, check_every);
  int64_t launches = 0;
  PcgState h{};
  h.atol = atol;
  h.maxit = maxit;
  h.norm_rr = norm_rr;
  if (cudaMemcpyAsync(pb.st, &h, sizeof(PcgState), cudaMemcpyHostToDevice, s) != cudaSuccess) return FGB_ERR_CUDA;
  pcg_init_kernel<double, G><<<grid_rows_for(n, G), kPcgThreads, 0, s>>>(n, indptr, indices, values, dinv, b, x, v.r,
                                                                          v.z, v.p0, pb.partials, pb.st);
  ++launches;
  // tol = rtol * ||b|| needs ||b||: one read-back before iterating
  if (cudaMemcpyAsync(&h, pb.st, sizeof(PcgState), cudaMemcpyDeviceToHost, s) != cudaSuccess) return FGB_ERR_CUDA;
  if (cudaStreamSynchronize(s) != cudaSuccess) return FGB_ERR_CUDA;
  if (h.done == FGB_PCG_ZERO_RHS) {
    cudaMemsetAsync(x, 0, n * sizeof(double), s);
  } else {
    const double tol = rtol * h.b_norm;
    if (cudaMemcpyAsync(reinterpret_cast<char*>(pb.st) + offsetof(PcgState, tol), &tol, sizeof(double),
                        cudaMemcpyHostToDevice, s) != cudaSuccess)
      return FGB_ERR_CUDA;
    int64_t it = 0;
    while (true) {
      const int64_t before = h.niter;
      for (int k = 0; k < check_every; ++k, ++it)
        f64_iteration<double, G>(n, indptr, indices, values, dinv, x, v, pb, it, prof.before(k), prof.after(k), s);
      launches += 2 * check_every;
      if (cudaGetLastError() != cudaSuccess) return FGB_ERR_CUDA;
      if (cudaMemcpyAsync(&h, pb.st, sizeof(PcgState), cudaMemcpyDeviceToHost, s) != cudaSuccess) return FGB_ERR_CUDA;
      if (cudaStreamSynchronize(s) != cudaSuccess) return FGB_ERR_CUDA;
      prof.collect(h.niter - before);
      if (h.done) break;
    }
  }
  if (info) {
    info->niter = h.niter;
    info->residual = h.resid;
    info->b_norm = h.b_norm;
    info->true_relres = -1.0;
    info->reason = h.done;
    info->n_updates = 0;
    info->launches = launches;
    info->kernel_ms = prof.ms;
    info->kernel_launches = prof.launches;
    info->other_ms = 0.0;
    info->extra_ms = 0.0;
    info->graph = 0;
    info->reserved = 0;
  }
  return finish_status(h.done);
}

template <int G>
int run_pcg_mixed(int64_t n, const int64_t* indptr, const int32_t* indices, const double* values64,
                  const float* values32, const double* dinv64, const double* b, double* x, double rtol, double delta,
                  int64_t maxit, int check_every, int profile, Carver& cv, fgb_pcg_info* info, cudaStream_t s) {
  PcgState* st = cv.take<PcgState>(1);
  double* partials = cv.take<double>(2 * kPcgMaxBlocks);
  float* r = cv.take<float>(n);
  float* z = cv.take<float>(n);
  float* p0 = cv.take<float>(n);
  float* p1 = cv.take<float>(n);
  float* Ap = cv.take<float>(n);
  float* y = cv.take<float>(n);
  float* dinv32 = cv.take<float>(n);
  double* r64 = cv.take<double>(n);
  if (!cv.ok) return FGB_ERR_WORKSPACE;
  SpmvProfiler prof(profile != 0, check_every);
  int64_t launches = 0;
  const int grid_rows = grid_rows_for(n, G), grid_vec = grid_vec_for(n);
  PcgState h{};
  h.maxit = maxit;
  h.atol = 0.0;
  h.tol = 0.0;
  h.norm_rr = 1;
  if (cudaMemcpyAsync(st, &h, sizeof(PcgState), cudaMemcpyHostToDevice, s) != cudaSuccess) return FGB_ERR_CUDA;
  cudaMemsetAsync(y, 0, n * sizeof(float), s);
  // ||b|| (for tol = rtol ||b||) from the FP64 init kernel, run on the r64 buffer
  // only (r, z and p all alias r64 there, which the kernel tolerates: it writes
  // the same value to all three)
  pcg_init_kernel<double, G><<<grid_rows, kPcgThreads, 0, s>>>(n, indptr, indices, values64, nullptr, b, x, r64, r64,
                                                               r64, partials, st);
  ++launches;
  if (cudaMemcpyAsync(&h, st, sizeof(PcgState), cudaMemcpyDeviceToHost, s) != cudaSuccess) return FGB_ERR_CUDA;
  if (cudaStreamSynchronize(s) != cudaSuccess) return FGB_ERR_CUDA;
  if (h.done == FGB_PCG_ZERO_RHS) {
    cudaMemsetAsync(x, 0, n * sizeof(double), s);
  } else {
    const double tol = rtol * h.b_norm;
    if (cudaMemcpyAsync(reinterpret_cast<char*>(st) + offsetof(PcgState, tol), &tol, sizeof(double),
                        cudaMemcpyHostToDevice, s) != cudaSuccess)
      return FGB_ERR_CUDA;
    // initial residual in FP64, converted to FP32; p = z
    mixed_residual_kernel<G><<<grid_rows, kPcgThreads, 0, s>>>(n, indptr, indices, values64, b, x, y, r64, partials, st, 1);
    mixed_replace_kernel<<<grid_vec, kPcgThreads, 0, s>>>(n, dinv64, r64, r, z, p0, dinv32, partials, st, 0.0, 1);
    launches += 2;
    int64_t it = 0;
    while (true) {
      const int64_t before = h.niter;
      for (int k = 0; k < check_every; ++k, ++it)
        mixed_launch_iteration<G>(n, indptr, indices, values64, values32, dinv64, b, x, y, r, z, p0, p1, Ap, r64,
                                  dinv32, partials, st, delta, it, grid_rows, grid_vec, prof.before(k), prof.after(k),
                                  s);
      launches += 5 * check_every;
      if (cudaGetLastError() != cudaSuccess) return FGB_ERR_CUDA;
      if (cudaMemcpyAsync(&h, st, sizeof(PcgState), cudaMemcpyDeviceToHost, s) != cudaSuccess) return FGB_ERR_CUDA;
      if (cudaStreamSynchronize(s) != cudaSuccess) return FGB_ERR_CUDA;
      prof.collect(h.niter - before);
      if (h.done) break;
    }
  }
  if (info) {
    info->niter = h.niter;
    info->residual = h.resid;
    info->b_norm = h.b_norm;
    info->true_relres = h.true_rel;
    info->reason = h.done;
    info->n_updates = h.n_updates;
    info->launches = launches;
    info->kernel_ms = prof.ms;
    info->kernel_launches = prof.launches;
    info->other_ms = 0.0;
    info->extra_ms = 0.0;
    info->graph = 0;
    info->reserved = 0;
  }
  return finish_status(h.done);
}

}  // namespace

namespace fgb {

constexpr int kResBlocks = 2 * kNumSMs;
constexpr int kResThreads = 512;

// per block: sum of r_i^2 over its rows (a warp per row, rows strided over
// the grid's warps) and of b_i^2, in double2 partials [2 * block]
__global__ void __launch_bounds__(kResThreads) residual_partials(int64_t n, const int64_t* __restrict__ indptr,
                                                               const int32_t* __restrict__ indices,
                                                               const double* __restrict__ values,
                                                               const double* __restrict__ b,
                                                               const double* __restrict__ x, double* part) {
  __shared__ double2 ws[kResThreads / 32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int64_t warp = (blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x) >> 5;
  const int64_t nwarps = (static_cast<int64_t>(gridDim.x) * blockDim.x) >> 5;
  double rr = 0.0, bb = 0.0;
  for (int64_t i = warp; i < n; i += nwarps) {
    double acc = 0.0;
    for (int64_t k = indptr[i] + lane; k < indptr[i + 1]; k += 32) acc += values[k] * x[indices[k]];
    acc = warp_sum(acc);
    if (lane == 0) {
      const double ri = b[i] - acc;
      rr += ri * ri;
      bb += b[i] * b[i];
    }
  }
  if (lane == 0) ws[wid] = make_double2(rr, bb);
  __syncthreads();
  if (wid == 0) {
    double2 t = lane < kResThreads / 32 ? ws[lane] : make_double2(0.0, 0.0);
    t.x = warp_sum(t.x);
    t.y = warp_sum(t.y);
    if (lane == 0) {
      part[2 * blockIdx.x] = t.x;
      part[2 * blockIdx.x + 1] = t.y;
    }
  }
}

// one warp: the partials in block order -> out2[0] = ||r||^2, out2[1] = ||b||^2
__global__ void residual_total(const double* __restrict__ part, double* out2) {
  const int lane = threadIdx.x;
  double a = 0.0, c = 0.0;
  for (int k = lane; k < kResBlocks; k += 32) {
    a += part[2 * k];
    c += part[2 * k + 1];
  }
  a = warp_sum(a);
  c = warp_sum(c);
  if (lane == 0) {
    out2[0] = a;
    out2[1] = c;
  }
}

}  // namespace fgb

extern "C" {

const char* fgb_status_string(int32_t status) {
  switch (status) {
    case FGB_OK: return "ok";
    case FGB_ERR_ARG: return "invalid argument";
    case FGB_ERR_WORKSPACE: return "workspace missing or too small";
    case FGB_ERR_INDEX: return "index out of range";
    case FGB_ERR_PATTERN: return "contribution outside the CSR pattern";
    case FGB_ERR_NONFINITE: return "non-finite value (degenerate cell or NaN input)";
    case FGB_ERR_BREAKDOWN: return "CG breakdown (p.Ap <= 0: matrix not SPD)";
    case FGB_ERR_CUDA: return "CUDA error";
    case FGB_ERR_CAPACITY: return "size exceeds a fixed kernel limit";
    default: return "unknown status";
  }
}

int32_t fgb_abi_version(void) { return 2; }

int32_t fgb_csr_spmv(int32_t dtype, int64_t n_row, const int64_t* indptr, const int32_t* indices, const void* values,
                     const void* x, void* y, int32_t lanes_per_row, void* stream) {
  if (n_row <= 0 || !indptr || !indices || !values || !x || !y) return FGB_ERR_ARG;
  int lanes = lanes_per_row;
  if (lanes == 0) {
    int64_t nnz = 0;
    cudaStream_t st = as_stream(stream);
    // the mean row length needs nnz: read indptr[n] (a small synchronous copy)
    if (cudaMemcpyAsync(&nnz, indptr + n_row, sizeof(int64_t), cudaMemcpyDeviceToHost, st) != cudaSuccess)
      return FGB_ERR_CUDA;
    if (cudaStreamSynchronize(st) != cudaSuccess) return FGB_ERR_CUDA;
    lanes = auto_lanes(n_row, nnz);
  }
  if (dtype == FGB_F64)
    return spmv_dispatch<double>(n_row, indptr, indices, static_cast<const double*>(values),
                                 static_cast<const double*>(x), static_cast<double*>(y), lanes, as_stream(stream));
  if (dtype == FGB_F32)
    return spmv_dispatch<float>(n_row, indptr, indices, static_cast<const float*>(values),
                                static_cast<const float*>(x), static_cast<float*>(y), lanes, as_stream(stream));
  return FGB_ERR_ARG;
}

// two partial sums (r.r, b.b) per block of residual_partials
size_t fgb_residual_norm_workspace_bytes(void) { return align_up(2 * kResBlocks * sizeof(double)); }

// ||b - A x||^2 and ||b||^2 (FP64 values, vectors and sums): a warp per row
// forms r_i = b_i - (A x)_i, every block writes its partial sums, one block
// adds the partials in block order (deterministic).  The true residual of
// the restart loops of cg_mixed's FP64 continuation and of multigrid_solve.
int32_t fgb_residual_norm(int64_t n, const int64_t* indptr, const int32_t* indices, const double* values,
                          const double* b, const double* x, double* out2, void* workspace, size_t workspace_bytes,
                          void* stream) {
  if (n <= 0 || !indptr || !indices || !values || !b || !x || !out2) return FGB_ERR_ARG;
  if (!workspace || workspace_bytes < fgb_residual_norm_workspace_bytes()) return FGB_ERR_WORKSPACE;
  cudaStream_t st = as_stream(stream);
  double* part = static_cast<double*>(workspace);
  residual_partials<<<kResBlocks, kResThreads, 0, st>>>(n, indptr, indices, values, b, x, part);
  residual_total<<<1, 32, 0, st>>>(part, out2);
  return launch_status();
}

int32_t fgb_csr_diagonal(int32_t dtype, int64_t n, const int64_t* indptr, const int32_t* indices, const void* values,
                         void* diag, void* diag_inv, void* stream) {
  if (n <= 0 || !indptr || !indices || !values || (!diag && !diag_inv)) return FGB_ERR_ARG;
  cudaStream_t st = as_stream(stream);
  const int grid = grid_for(n, 256, kNumSMs * 16);
  if (dtype == FGB_F64)
    diagonal_kernel<double><<<grid, 256, 0, st>>>(n, indptr, indices, static_cast<const double*>(values),
                                                  static_cast<double*>(diag), static_cast<double*>(diag_inv));
  else if (dtype == FGB_F32)
    diagonal_kernel<float><<<grid, 256, 0, st>>>(n, indptr, indices, static_cast<const float*>(values),
                                                 static_cast<float*>(diag), static_cast<float*>(diag_inv));
  else
    return FGB_ERR_ARG;
  return launch_status();
}

size_t fgb_pcg_workspace_bytes(int64_t n) {
  return align_up(sizeof(PcgState)) + align_up(2 * kPcgMaxBlocks * sizeof(double)) +
         5 * align_up(static_cast<size_t>(n) * sizeof(double));
}

int32_t fgb_pcg_f64(int64_t n, const int64_t* indptr, const int32_t* indices, const double* values,
                    const double* diag_inv, const double* b, double* x, double atol, double rtol, int64_t maxit,
                    int32_t check_every, int32_t lanes_per_row, int32_t norm, int32_t profile, void* workspace,
                    size_t workspace_bytes, fgb_pcg_info* info_host, void* stream) {
  if (n <= 0 || !indptr || !indices || !values || !b || !x || maxit <= 0) return FGB_ERR_ARG;
  if (!workspace || workspace_bytes < fgb_pcg_workspace_bytes(n)) return FGB_ERR_WORKSPACE;
  if (check_every <= 0) check_every = 16;
  Carver cv(workspace, workspace_bytes);
  cudaStream_t s = as_stream(stream);
  int G = lanes_per_row;
  if (G == 0) {
    int64_t nnz = 0;
    if (cudaMemcpyAsync(&nnz, indptr + n, sizeof(int64_t), cudaMemcpyDeviceToHost, s) != cudaSuccess) return FGB_ERR_CUDA;
    if (cudaStreamSynchronize(s) != cudaSuccess) return FGB_ERR_CUDA;
    G = auto_lanes(n, nnz);
  }
  switch (G) {
    case 2: return run_pcg_f64<2>(n, indptr, indices, values, diag_inv, b, x, atol, rtol, maxit, check_every, norm, profile, cv, info_host, s);
    case 4: return run_pcg_f64<4>(n, indptr, indices, values, diag_inv, b, x, atol, rtol, maxit, check_every, norm, profile, cv, info_host, s);
    case 8: return run_pcg_f64<8>(n, indptr, indices, values, diag_inv, b, x, atol, rtol, maxit, check_every, norm, profile, cv, info_host, s);
    case 16: return run_pcg_f64<16>(n, indptr, indices, values, diag_inv, b, x, atol, rtol, maxit, check_every, norm, profile, cv, info_host, s);
    case 32: return run_pcg_f64<32>(n, indptr, indices, values, diag_inv, b, x, atol, rtol, maxit, check_every, norm, profile, cv, info_host, s);
    default: return FGB_ERR_ARG;
  }
}

}  // extern "C"

// ---------------------------------------------------------------------------
// FP64 Jacobi-PCG without any allocation: the solver's scratch (state block,
// reduction partials and the r, z, p, p', Ap vectors) lives in one static
// device array of this library instead of a caller workspace.
namespace {

constexpr size_t cx_align(size_t b) { return (b + 255) / 256 * 256; }

// Same layout and size as fgb_pcg_workspace_bytes(FGB_PCG_NOALLOC_MAX_ROWS):
// 5 FP64 vectors of 65,536 rows + state + partials, about 2.6 MB.
constexpr size_t kNoAllocScratchBytes = cx_align(sizeof(PcgState)) + cx_align(2 * kPcgMaxBlocks * sizeof(double)) +
                                        5 * cx_align(static_cast<size_t>(FGB_PCG_NOALLOC_MAX_ROWS) * sizeof(double));

__device__ __align__(256) unsigned char g_pcg_noalloc_scratch[kNoAllocScratchBytes];

// Device address of the static scratch in the context current on the calling
// thread.  It is looked up on every call, never cached: the address belongs
// to the CUDA context that holds this library's module, and a context can be
// replaced while the process runs (cudaDeviceReset, another context made
// current on the same device), after which a cached address would point at
// freed memory.  The first lookup in a context may load this library's device
// code into it; later ones are a table lookup.
int noalloc_scratch(void** out) {
  void* p = nullptr;
  if (cudaGetSymbolAddress(&p, g_pcg_noalloc_scratch) != cudaSuccess || !p) return FGB_ERR_CUDA;
  *out = p;
  return FGB_OK;
}

}  // namespace

extern "C" {

int32_t fgb_pcg_f64_noalloc(int64_t n, const int64_t* indptr, const int32_t* indices, const double* values,
                            const double* diag_inv, const double* b, double* x, double atol, double rtol,
                            int64_t maxit, int32_t check_every, int32_t lanes_per_row, int32_t norm,
                            fgb_pcg_info* info_host, void* stream) {
  if (n <= 0 || !indptr || !indices || !values || !b || !x || maxit <= 0) return FGB_ERR_ARG;
  if (n > FGB_PCG_NOALLOC_MAX_ROWS) return FGB_ERR_CAPACITY;
  if (fgb_pcg_workspace_bytes(n) > kNoAllocScratchBytes) return FGB_ERR_CAPACITY;
  void* scratch = nullptr;
  const int rc = noalloc_scratch(&scratch);
  if (rc != FGB_OK) return rc;
  // profile = 0: the event-timing option creates CUDA events, so it is not offered here
  return fgb_pcg_f64(n, indptr, indices, values, diag_inv, b, x, atol, rtol, maxit, check_every, lanes_per_row, norm,
                     0, scratch, kNoAllocScratchBytes, info_host, stream);
}

size_t fgb_pcg_mixed_workspace_bytes(int64_t n) {
  return align_up(sizeof(PcgState)) + align_up(2 * kPcgMaxBlocks * sizeof(double)) +
         7 * align_up(static_cast<size_t>(n) * sizeof(float)) + align_up(static_cast<size_t>(n) * sizeof(double));
}

int32_t fgb_pcg_mixed(int64_t n, const int64_t* indptr, const int32_t* indices, const double* values64,
                      const float* values32, const double* diag_inv64, const double* b, double* x, double rtol,
                      double delta, int64_t maxit, int32_t check_every, int32_t lanes_per_row, int32_t profile,
                      void* workspace, size_t workspace_bytes, fgb_pcg_info* info_host, void* stream) {
  if (n <= 0 || !indptr || !indices || !values64 || !values32 || !diag_inv64 || !b || !x || maxit <= 0)
    return FGB_ERR_ARG;
  if (!(delta > 0.0 && delta < 1.0)) return FGB_ERR_ARG;
  if (!workspace || workspace_bytes < fgb_pcg_mixed_workspace_bytes(n)) return FGB_ERR_WORKSPACE;
  if (check_every <= 0) check_every = 16;
  Carver cv(workspace, workspace_bytes);
  cudaStream_t s = as_stream(stream);
  int G = lanes_per_row;
  if (G == 0) {
    int64_t nnz = 0;
    if (cudaMemcpyAsync(&nnz, indptr + n, sizeof(int64_t), cudaMemcpyDeviceToHost, s) != cudaSuccess) return FGB_ERR_CUDA;
    if (cudaStreamSynchronize(s) != cudaSuccess) return FGB_ERR_CUDA;
    G = auto_lanes(n, nnz);
  }
  switch (G) {
    case 2: return run_pcg_mixed<2>(n, indptr, indices, values64, values32, diag_inv64, b, x, rtol, delta, maxit, check_every, profile, cv, info_host, s);
    case 4: return run_pcg_mixed<4>(n, indptr, indices, values64, values32, diag_inv64, b, x, rtol, delta, maxit, check_every, profile, cv, info_host, s);
    case 8: return run_pcg_mixed<8>(n, indptr, indices, values64, values32, diag_inv64, b, x, rtol, delta, maxit, check_every, profile, cv, info_host, s);
    case 16: return run_pcg_mixed<16>(n, indptr, indices, values64, values32, diag_inv64, b, x, rtol, delta, maxit, check_every, profile, cv, info_host, s);
    case 32: return run_pcg_mixed<32>(n, indptr, indices, values64, values32, diag_inv64, b, x, rtol, delta, maxit, check_every, profile, cv, info_host, s);
    default: return FGB_ERR_ARG;
  }
}

}  // extern "C"
