// Batched FP32-refined Jacobi-PCG: many independent systems (each with its own
// SELL-32x4 copy and Krylov vectors) iterate together.  One iteration is four
// kernels over tile lists plus a reliable-update branch.  A tile (a few slices
// or ~1000 rows of one system) is processed by one warp, which takes the next
// tile with an atomic ticket: no block barriers in the tile loops, and the
// load balances itself however uneven the systems are.
//
//   slice tiles: Ap = A p_new with p_new = z + beta p_old formed per gathered
//                column; per-tile partials of p.Ap
//   systems    : alpha = rz / p.Ap per system (sum of its tiles, in order)
//   row tiles  : y += alpha p, r -= alpha Ap, z = Dinv r; per-tile r.z, r.r
//   control    : per system rz, rr, beta, stopping test, reliable update due?;
//                any update due -> IF branch; nothing running -> end of loop
//   IF branch  : x += y (row tiles), r64 = b - A x in FP64 arithmetic and the
//                replaced r, z (slice tiles), true residual test (systems)
//
// Every reduction of a system adds its own tiles in tile order, and a
// system's tiles depend only on its own sizes, so its iterates are the same
// whatever else is in the batch.  Systems join (fgb_batch_admit) and leave
// (fgb_batch_retire) between runs; the graph reads the tables from fixed
// device addresses, so it is captured once per handle.

#include "fgb_common.cuh"
#include "sell_rows.cuh"

#include <cmath>
#include <cstdint>
#include <cstring>
#include <new>

namespace fgb {

constexpr int kBatchRowThreads = 512;
constexpr int kBatchRowBlocks = 2 * kNumSMs;

struct BatchCtl {
  long long trips, trip_limit, if_trips;
  int any_update, running;
  int any_acc, running_acc;  // accumulated over the blocks of batch_control
  unsigned int arrived;
  // tile tickets of the tile kernels (SpMV, update, fold, reliable, p update):
  // each warp takes the next tile with one atomic; a kernel that follows in
  // stream order puts the ticket back to 0
  unsigned int ticket[5];
};

enum { kTicketSpmv = 0, kTicketUpdate = 1, kTicketFold = 2, kTicketReliable = 3, kTicketP = 4 };

// The next tile for the calling warp (all lanes get the same index).
__device__ __forceinline__ int next_tile(unsigned int* ticket) {
  unsigned int t = 0;
  if ((threadIdx.x & 31) == 0) t = atomicAdd(ticket, 1u);
  return static_cast<int>(__shfl_sync(0xffffffffu, t, 0));
}

// Per-system sums of tile partials: a block per system; thread k adds tiles
// k, k + blockDim, ... and the block adds the threads in a fixed tree, so the
// result does not depend on timing.  Valid in thread 0.  `stride` partials per
// tile, component `c`.
__device__ __forceinline__ double tile_sum(const double* __restrict__ part, int t0, int t1, int stride, int c,
                                           double* red) {
  double v = 0.0;
  for (int t = t0 + threadIdx.x; t < t1; t += blockDim.x) v += part[stride * t + c];
  return block_sum(v, red);
}

// ---------------------------------------------------------------- kernels
// Vector type of a system: float (FP32 iterations) or double (fp64 systems).
template <typename T> struct Vec;
template <> struct Vec<float> {
  __device__ static const float* val(const fgb_batch_system& A) { return A.val32; }
  __device__ static const float* dinv(const fgb_batch_system& A) { return static_cast<const float*>(A.dinv32); }
};
template <> struct Vec<double> {
  __device__ static const double* val(const fgb_batch_system& A) { return A.val64; }
  __device__ static const double* dinv(const fgb_batch_system& A) { return A.dinv64; }
};
template <typename T> __device__ __forceinline__ T* vp(void* p) { return static_cast<T*>(p); }

// One row tile, one warp: p = z + beta p in place (a single
// gather per entry in the SpMV that follows is cheaper than forming p on the
// fly from two gathers).
template <typename T>
__device__ void p_tile(const fgb_batch_system& A, const fgb_batch_state& S, const fgb_batch_tile& tile) {
  const T beta = static_cast<T>(S.beta);
  const T* __restrict__ z = vp<T>(A.z);
  T* __restrict__ p = vp<T>(A.p);
  for (int i = tile.begin + (threadIdx.x & 31); i < tile.end; i += 32) p[i] = z[i] + beta * p[i];
}

// Row tiles (a warp each, by ticket): the p update of every running system.
__global__ void __launch_bounds__(1024, 1) batch_p_update(const fgb_batch_system* __restrict__ sys,
                                                          const fgb_batch_state* __restrict__ st,
                                                          const fgb_batch_tile* __restrict__ tiles,
                                                          const int32_t* __restrict__ n_tiles, BatchCtl* ctl) {
  const int nt = *n_tiles;
  while (true) {
    const int t = next_tile(&ctl->ticket[kTicketP]);
    if (t >= nt) break;
    const fgb_batch_tile tile = tiles[t];
    const fgb_batch_state& S = st[tile.sys];
    if (!S.active || S.done || S.need_update) continue;
    const fgb_batch_system& A = sys[tile.sys];
    if (A.fp64) p_tile<double>(A, S, tile);
    else p_tile<float>(A, S, tile);
  }
}

// One slice tile, one warp: Ap and the lane's p.Ap (in the vector type, FP64
// from the warp sum on).
template <typename T>
__device__ double spmv_tile(const fgb_batch_system& A, const fgb_batch_state& S, const fgb_batch_tile& tile) {
  const int lane = threadIdx.x & 31;
  const T* p = vp<T>(A.p);
  T* Ap = vp<T>(A.Ap);
  const GatherX<T> g{p};
  T pap = T(0);
  for (int64_t s = tile.begin; s < tile.end; ++s) {
    const int64_t sbase = A.slice_ptr[s];
    const int w = static_cast<int>((A.slice_ptr[s + 1] - sbase) >> 5);
    const T acc = sell_row(A.col, Vec<T>::val(A), sbase, w, lane, g);
    const int32_t row = A.perm[s * kSellC + lane];
    if (row >= 0) {
      Ap[row] = acc;
      pap += p[row] * acc;
    }
  }
  return static_cast<double>(warp_sum(pap));
}

// Slice tiles (a warp each, taken by ticket): Ap and the tile's p.Ap.
__global__ void __launch_bounds__(1024, 1) batch_spmv_step(const fgb_batch_system* __restrict__ sys,
                                                           const fgb_batch_state* __restrict__ st,
                                                           const fgb_batch_tile* __restrict__ tiles,
                                                           const int32_t* __restrict__ n_tiles, double* spart,
                                                           BatchCtl* ctl) {
  const int nt = *n_tiles;
  while (true) {
    const int t = next_tile(&ctl->ticket[kTicketSpmv]);
    if (t >= nt) break;
    const fgb_batch_tile tile = tiles[t];
    const fgb_batch_state& S = st[tile.sys];
    double pap = 0.0;
    if (S.active && !S.done && !S.need_update) {  // need_update: admission pending
      const fgb_batch_system& A = sys[tile.sys];
      pap = A.fp64 ? spmv_tile<double>(A, S, tile) : spmv_tile<float>(A, S, tile);
    }
    if ((threadIdx.x & 31) == 0) spart[t] = pap;
  }
}

// Systems (a block each): alpha = rz / p.Ap.  Also returns the p-update and
// SpMV tickets.
__global__ void batch_alpha(int32_t n_sys, fgb_batch_state* st, const int32_t* __restrict__ tile_ptr,
                            const double* __restrict__ spart, BatchCtl* ctl) {
  __shared__ double red[32];
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    ctl->ticket[kTicketSpmv] = 0u;
    ctl->ticket[kTicketP] = 0u;
  }
  const int s = blockIdx.x;
  if (s >= n_sys) return;
  fgb_batch_state& S = st[s];
  if (!S.active || S.done || S.need_update) return;
  const double pap = tile_sum(spart, tile_ptr[s], tile_ptr[s + 1], 1, 0, red);
  if (threadIdx.x != 0) return;
  if (!(pap > 0.0) || !isfinite(pap)) {
    S.done = isfinite(pap) ? FGB_PCG_BREAKDOWN : FGB_PCG_NONFINITE;
    S.alpha = 0.0;
  } else {
    S.alpha = S.rz / pap;
  }
}

// One row tile, one warp: y += alpha p, r -= alpha Ap, z = Dinv r; the lane's
// r.z, r.r (accumulated in the vector type).
template <typename T>
__device__ void update_tile(const fgb_batch_system& A, const fgb_batch_state& S, const fgb_batch_tile& tile,
                            double* rz_out, double* rr_out) {
  const T alpha = static_cast<T>(S.alpha);
  const T* __restrict__ p = vp<T>(A.p);
  const T* __restrict__ Ap = vp<T>(A.Ap);
  const T* __restrict__ dinv = Vec<T>::dinv(A);
  T* __restrict__ y = vp<T>(A.y);
  T* __restrict__ r = vp<T>(A.r);
  T* __restrict__ z = vp<T>(A.z);
  T rz = T(0), rr = T(0);
  for (int i = tile.begin + (threadIdx.x & 31); i < tile.end; i += 32) {
    y[i] += alpha * p[i];
    const T ri = r[i] - alpha * Ap[i];
    const T zi = dinv[i] * ri;
    r[i] = ri;
    z[i] = zi;
    rz += ri * zi;
    rr += ri * ri;
  }
  *rz_out = static_cast<double>(rz);
  *rr_out = static_cast<double>(rr);
}

// Row tiles (a warp each, by ticket): the updates and the tile's r.z, r.r.
__global__ void __launch_bounds__(1024, 1) batch_update(const fgb_batch_system* __restrict__ sys,
                                                        const fgb_batch_state* __restrict__ st,
                                                        const fgb_batch_tile* __restrict__ tiles,
                                                        const int32_t* __restrict__ n_tiles, double* vpart,
                                                        BatchCtl* ctl) {
  const int nt = *n_tiles;
  while (true) {
    const int t = next_tile(&ctl->ticket[kTicketUpdate]);
    if (t >= nt) break;
    const fgb_batch_tile tile = tiles[t];
    const fgb_batch_state& S = st[tile.sys];
    double rz = 0.0, rr = 0.0;
    if (S.active && !S.done && !S.need_update) {
      const fgb_batch_system& A = sys[tile.sys];
      if (A.fp64) update_tile<double>(A, S, tile, &rz, &rr);
      else update_tile<float>(A, S, tile, &rz, &rr);
    }
    rz = warp_sum(rz);
    rr = warp_sum(rr);
    if ((threadIdx.x & 31) == 0) { vpart[2 * t] = rz; vpart[2 * t + 1] = rr; }
  }
}

// Systems (a block each): rz, rr, beta, stopping test and whether a reliable
// update (or a check of the true residual) is due; the last block to finish
// sets the graph conditions.  Also returns the update ticket.
__global__ void batch_control(int32_t n_sys, fgb_batch_state* st, const int32_t* __restrict__ tile_ptr,
                              const double* __restrict__ vpart, const fgb_batch_system* __restrict__ sys,
                              BatchCtl* ctl, cudaGraphConditionalHandle h_if, cudaGraphConditionalHandle h_while,
                              int graph) {
  __shared__ double red[32];
  __shared__ bool last;
  if (blockIdx.x == 0 && threadIdx.x == 0) ctl->ticket[kTicketUpdate] = 0u;
  int any = 0, running = 0;
  const int s = blockIdx.x;
  if (s < n_sys) {
    fgb_batch_state& S = st[s];
    if (S.active && !S.done) {
      if (S.need_update) {
        running = 1;
      } else {
        const double rz = tile_sum(vpart, tile_ptr[s], tile_ptr[s + 1], 2, 0, red);
        __syncthreads();
        const double rr = tile_sum(vpart, tile_ptr[s], tile_ptr[s + 1], 2, 1, red);
        if (threadIdx.x == 0) {
          S.niter += 1;
          const double res = sqrt(rr);
          S.resid = res;
          S.rr = rr;
          if (!isfinite(res)) {
            S.done = FGB_PCG_NONFINITE;
          } else {
            const long long gap = S.niter - S.last_upd;
            const long long slack = S.max_gap / 2 > 100 ? S.max_gap / 2 : 100;
            // before any residual-triggered update: a first check after 1000
            // iterations; FP64 systems (no residual-triggered updates) are checked
            // every 5000 iterations, so a residual that stalls above rtol ends
            // after three checks instead of at the iteration limit
            const bool plateau = sys[s].fp64 ? gap > 5000
                                             : (S.max_gap > 0 ? gap > S.max_gap + slack : gap > 1000);
            // FP64 systems run plain FP64 PCG: the true residual is formed only
            // to confirm convergence (or at the iteration limit)
            const bool due = (!sys[s].fp64 && res < S.delta * S.r_upd) || (res < S.tol) || (S.niter >= S.maxit);
            S.need_update = due ? 1 : (plateau ? 3 : 0);  // 3: a check of the true residual
            S.rz_prev = S.rz;
            S.beta = rz / S.rz;
            S.rz = rz;
          }
          any = S.need_update && !S.done;
          running = !S.done;
        }
      }
    }
  }
  if (threadIdx.x == 0) {
    if (any) atomicOr(&ctl->any_acc, 1);
    if (running) atomicOr(&ctl->running_acc, 1);
    __threadfence();
    last = atomicAdd(&ctl->arrived, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!last || threadIdx.x != 0) return;
  __threadfence();
  const int a = atomicOr(&ctl->any_acc, 0), r = atomicOr(&ctl->running_acc, 0);
  ctl->any_acc = 0;
  ctl->running_acc = 0;
  ctl->arrived = 0u;
  ctl->trips += 1;
  ctl->if_trips += a ? 1 : 0;
  ctl->any_update = a;
  ctl->running = r;
  if (graph) {
    cudaGraphSetConditional(h_if, a ? 1u : 0u);
    if (!r || ctl->trips >= ctl->trip_limit) cudaGraphSetConditional(h_while, 0u);
  }
}

template <typename T>
__device__ void fold_tile(const fgb_batch_system& A, const fgb_batch_tile& tile) {
  T* y = vp<T>(A.y);
  for (int i = tile.begin + (threadIdx.x & 31); i < tile.end; i += 32) {
    A.x[i] += static_cast<double>(y[i]);
    y[i] = T(0);
  }
}

template <typename T>
__device__ double admit_tile(const fgb_batch_system& A, const fgb_batch_tile& tile) {
  T* y = vp<T>(A.y);
  double bb = 0.0;
  for (int i = tile.begin + (threadIdx.x & 31); i < tile.end; i += 32) {
    y[i] = T(0);
    bb += A.b[i] * A.b[i];
  }
  return bb;
}

// Row tiles (a warp each, by ticket) of systems with an update due (or all
// given slots when force): x += y, y = 0.  Admission (need_update == 2)
// instead zeroes y and forms the per-tile partials of b.b.
__global__ void __launch_bounds__(1024, 1) batch_fold(const fgb_batch_system* __restrict__ sys,
                                                      const fgb_batch_state* __restrict__ st,
                                                      const fgb_batch_tile* __restrict__ tiles,
                                                      const int32_t* __restrict__ n_tiles,
                                                      const int32_t* __restrict__ force, double* vpart,
                                                      BatchCtl* ctl) {
  const int nt = *n_tiles;
  while (true) {
    const int t = next_tile(&ctl->ticket[kTicketFold]);
    if (t >= nt) break;
    const fgb_batch_tile tile = tiles[t];
    const fgb_batch_state& S = st[tile.sys];
    const bool forced = force && force[tile.sys];
    const int mode = S.active ? S.need_update : 0;
    const fgb_batch_system& A = sys[tile.sys];
    if (forced || ((mode == 1 || mode == 3) && !S.done)) {
      if (A.fp64) fold_tile<double>(A, tile);
      else fold_tile<float>(A, tile);
    } else if (mode == 2 && !S.done) {
      double bb = A.fp64 ? admit_tile<double>(A, tile) : admit_tile<float>(A, tile);
      bb = warp_sum(bb);
      if ((threadIdx.x & 31) == 0) vpart[2 * t] = bb;
    }
  }
}

// Admission: ||b||, tol = rtol * ||b|| (rtol was stored in tol), zero rhs.
// Also returns the fold ticket.
__global__ void batch_bnorm(int32_t n_sys, fgb_batch_state* st, const int32_t* __restrict__ tile_ptr,
                            const double* __restrict__ vpart, BatchCtl* ctl) {
  __shared__ double red[32];
  if (blockIdx.x == 0 && threadIdx.x == 0) ctl->ticket[kTicketFold] = 0u;
  const int s = blockIdx.x;
  if (s >= n_sys) return;
  fgb_batch_state& S = st[s];
  if (!S.active || S.done || S.need_update != 2) return;
  const double bb = tile_sum(vpart, tile_ptr[s], tile_ptr[s + 1], 2, 0, red);
  if (threadIdx.x != 0) return;
  S.b_norm = sqrt(bb);
  S.tol = S.tol * S.b_norm;
  if (S.b_norm < 1e-15) S.done = FGB_PCG_ZERO_RHS;
}

// One slice tile, one warp, of a system with an update due (1, 3) or admitted
// (2): r64 = b - A x in FP64 arithmetic (V: the stored values), r = T(r64),
// z = Dinv r; the lane's r64.r64 and r.z.  Admission of an FP32 system also
// builds its FP32 inverse diagonal; admission starts p = z (with beta = 0 the
// first p update keeps it).
template <typename V, typename T>
__device__ void reliable_tile(const fgb_batch_system& A, const fgb_batch_state& S, const V* __restrict__ val,
                              const fgb_batch_tile& tile, int mode, double* rr_out, double* rz_out) {
  const int lane = threadIdx.x & 31;
  double rr64 = 0.0, rz = 0.0;
  T* p = vp<T>(A.p);
  T* r = vp<T>(A.r);
  T* z = vp<T>(A.z);
  for (int64_t s = tile.begin; s < tile.end; ++s) {
    const int64_t sbase = A.slice_ptr[s];
    const int w = static_cast<int>((A.slice_ptr[s + 1] - sbase) >> 5);
    const double acc = sell_row_acc<V, double>(A.col, val, sbase, w, lane, GatherX<double>{A.x});
    const int32_t row = A.perm[s * kSellC + lane];
    if (row >= 0) {
      const double r64 = A.b[row] - acc;
      rr64 += r64 * r64;
      T di;
      if (sizeof(T) == 8) {
        di = static_cast<T>(A.dinv64[row]);
      } else if (mode == 2) {
        di = static_cast<T>(A.dinv64[row]);
        vp<T>(A.dinv32)[row] = di;
      } else {
        di = vp<T>(A.dinv32)[row];
      }
      const T ri = static_cast<T>(r64);
      const T zi = di * ri;
      r[row] = ri;
      z[row] = zi;
      if (mode == 2) p[row] = zi;
      rz += static_cast<double>(ri) * static_cast<double>(zi);
    }
  }
  *rr_out = rr64;
  *rz_out = rz;
}

__global__ void __launch_bounds__(1024, 1) batch_reliable(const fgb_batch_system* __restrict__ sys,
                                                          const fgb_batch_state* __restrict__ st,
                                                          const fgb_batch_tile* __restrict__ tiles,
                                                          const int32_t* __restrict__ n_tiles, double* rpart,
                                                          BatchCtl* ctl) {
  const int nt = *n_tiles;
  while (true) {
    const int t = next_tile(&ctl->ticket[kTicketReliable]);
    if (t >= nt) break;
    const fgb_batch_tile tile = tiles[t];
    const fgb_batch_state& S = st[tile.sys];
    const int mode = S.active && !S.done ? S.need_update : 0;
    if (!mode) continue;
    const fgb_batch_system& A = sys[tile.sys];
    double rr, rz;
    if (A.fp64) reliable_tile<double, double>(A, S, A.val64, tile, mode, &rr, &rz);
    else if (A.val64) reliable_tile<double, float>(A, S, A.val64, tile, mode, &rr, &rz);
    else reliable_tile<float, float>(A, S, A.val32, tile, mode, &rr, &rz);
    rr = warp_sum(rr);
    rz = warp_sum(rz);
    if ((threadIdx.x & 31) == 0) { rpart[2 * t] = rr; rpart[2 * t + 1] = rz; }
  }
}

// Systems (a block each) with an update due or admitted: true residual test,
// beta from the replaced residual.  An FP32 system whose true residual has not
// halved since the previous check stops as FGB_PCG_STAGNATED (its condition
// number is beyond what FP32 iterations resolve); the caller continues it in
// FP64.  Also returns the fold and reliable tickets.
__global__ void batch_reliable_fin(int32_t n_sys, fgb_batch_state* st, const int32_t* __restrict__ tile_ptr,
                                   const double* __restrict__ rpart, const fgb_batch_system* __restrict__ sys,
                                   BatchCtl* ctl) {
  __shared__ double red[32];
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    ctl->ticket[kTicketFold] = 0u;
    ctl->ticket[kTicketReliable] = 0u;
  }
  const int s = blockIdx.x;
  if (s >= n_sys) return;
  fgb_batch_state& S = st[s];
  const int mode = S.active && !S.done ? S.need_update : 0;
  if (!mode) return;
  const double rr = tile_sum(rpart, tile_ptr[s], tile_ptr[s + 1], 2, 0, red);
  __syncthreads();
  const double rz = tile_sum(rpart, tile_ptr[s], tile_ptr[s + 1], 2, 1, red);
  if (threadIdx.x != 0) return;
  const double nrm = sqrt(rr);
  S.true_rel = S.b_norm > 0.0 ? nrm / S.b_norm : 0.0;
  S.resid = nrm;
  if (mode != 2) {
    S.n_updates += 1;
    // the longest gap between updates triggered by the residual estimate
    // (not by a check) sets when the next check is due
    const long long gap = S.niter - S.last_upd;
    if (mode == 1 && gap > S.max_gap) S.max_gap = gap;
    S.last_upd = S.niter;
    if (nrm < 0.5 * S.r_best) {
      S.r_best = nrm;
      S.stall = 0;
    } else {
      S.stall += 1;
    }
  } else {
    S.r_best = nrm;
    S.last_upd = S.niter;
  }
  if (!isfinite(nrm)) S.done = FGB_PCG_NONFINITE;
  else if (nrm <= S.tol) S.done = FGB_PCG_RTOL;
  else if (S.niter >= S.maxit) S.done = FGB_PCG_MAXIT;
  else if (S.stall >= (sys[s].fp64 ? 3 : 1)) S.done = FGB_PCG_STAGNATED;  // FP64: attainable accuracy
  S.beta = mode == 2 ? 0.0 : rz / S.rz_prev;
  S.rz = rz;
  S.rr = rr;
  S.r_upd = nrm;
  S.need_update = 0;
}

// Retirement: slots flagged in `force` become inactive; flags cleared.  Also
// returns the fold ticket (retirement runs batch_fold first).
__global__ void batch_deactivate(int32_t n_sys, fgb_batch_state* st, int32_t* force, BatchCtl* ctl) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s == 0) ctl->ticket[kTicketFold] = 0u;
  if (s >= n_sys || !force[s]) return;
  st[s].active = 0;
  force[s] = 0;
}

// y_s = A_s x_s (FP32) over slice tiles, a warp per tile (tiles dealt out
// round-robin); the autotuner's timing kernel.
__global__ void __launch_bounds__(1024, 1) batch_spmv_plain(const fgb_batch_system* __restrict__ sys,
                                                            const fgb_batch_tile* __restrict__ tiles,
                                                            const int32_t* __restrict__ n_tiles,
                                                            const float* const* __restrict__ xs,
                                                            float* const* __restrict__ ys) {
  const int nt = *n_tiles;
  const int lane = threadIdx.x & 31;
  const int w0 = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nw = (gridDim.x * blockDim.x) >> 5;
  for (int t = w0; t < nt; t += nw) {
    const fgb_batch_tile tile = tiles[t];
    const fgb_batch_system& A = sys[tile.sys];
    if (A.fp64) continue;
    const GatherX<float> g{xs[tile.sys]};
    float* y = ys[tile.sys];
    for (int64_t s = tile.begin; s < tile.end; ++s) {
      const int64_t sbase = A.slice_ptr[s];
      const int w = static_cast<int>((A.slice_ptr[s + 1] - sbase) >> 5);
      const float acc = sell_row(A.col, A.val32, sbase, w, lane, g);
      const int32_t row = A.perm[s * kSellC + lane];
      if (row >= 0) y[row] = acc;
    }
  }
}

}  // namespace fgb

using namespace fgb;

// ------------------------------------------------------------------ host side
struct fgb_batch {
  int32_t max_sys, max_st, max_vt, slice_threads;
  int32_t n_sys = 0, n_st = 0, n_vt = 0;
  fgb_batch_system* sys;
  fgb_batch_state* st;
  fgb_batch_tile *stiles, *vtiles;
  int32_t *stile_ptr, *vtile_ptr, *n_stiles, *n_vtiles, *force;
  double *spart, *vpart, *rpart;
  BatchCtl* ctl;
  const float** xs;
  float** ys;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  bool graph_failed = false;
};

namespace {

size_t batch_layout(int32_t ms, int32_t mst, int32_t mvt, fgb_batch* b, void* base, size_t bytes) {
  Carver cv(base, bytes);
  auto sys = cv.take<fgb_batch_system>(ms);
  auto st = cv.take<fgb_batch_state>(ms);
  auto stiles = cv.take<fgb_batch_tile>(mst);
  auto vtiles = cv.take<fgb_batch_tile>(mvt);
  auto sptr = cv.take<int32_t>(ms + 1);
  auto vptr = cv.take<int32_t>(ms + 1);
  auto counts = cv.take<int32_t>(2);
  auto force = cv.take<int32_t>(ms);
  auto spart = cv.take<double>(mst);
  auto vpart = cv.take<double>(2 * static_cast<size_t>(mvt));
  auto rpart = cv.take<double>(2 * static_cast<size_t>(mst));
  auto ctl = cv.take<BatchCtl>(1);
  auto xs = cv.take<const float*>(ms);
  auto ys = cv.take<float*>(ms);
  if (b) {
    b->sys = sys; b->st = st; b->stiles = stiles; b->vtiles = vtiles; b->stile_ptr = sptr; b->vtile_ptr = vptr;
    b->n_stiles = counts; b->n_vtiles = counts + 1; b->force = force; b->spart = spart; b->vpart = vpart;
    b->rpart = rpart; b->ctl = ctl; b->xs = xs; b->ys = ys;
  }
  return cv.ok ? cv.off : 0;
}

int sys_blocks(int32_t n) { return (n + 255) / 256; }
constexpr int kSysThreads = 256;  // a block per system for the per-system sums
// The tile loops are persistent: as many blocks as stay resident at once (the
// slice kernels use up to 64 registers a thread, so 1024 threads per SM), so
// that no block of a later wave holds a tile back.
int slice_grid(const fgb_batch* b) {
  const int resident = kNumSMs * (1024 / b->slice_threads > 0 ? 1024 / b->slice_threads : 1);
  return b->max_st < resident ? b->max_st : resident;
}
int row_grid(const fgb_batch* b) { return b->max_vt < kBatchRowBlocks ? b->max_vt : kBatchRowBlocks; }

void launch_iteration(fgb_batch* b, cudaStream_t s, int graph, cudaGraphConditionalHandle h_if,
                      cudaGraphConditionalHandle h_while) {
  batch_p_update<<<row_grid(b), kBatchRowThreads, 0, s>>>(b->sys, b->st, b->vtiles, b->n_vtiles, b->ctl);
  batch_spmv_step<<<slice_grid(b), b->slice_threads, 0, s>>>(b->sys, b->st, b->stiles, b->n_stiles, b->spart,
                                                              b->ctl);
  batch_alpha<<<b->max_sys, kSysThreads, 0, s>>>(b->max_sys, b->st, b->stile_ptr, b->spart, b->ctl);
  batch_update<<<row_grid(b), kBatchRowThreads, 0, s>>>(b->sys, b->st, b->vtiles, b->n_vtiles, b->vpart, b->ctl);
  batch_control<<<b->max_sys, kSysThreads, 0, s>>>(b->max_sys, b->st, b->vtile_ptr, b->vpart, b->sys, b->ctl, h_if, h_while,
                                               graph);
}

void launch_reliable(fgb_batch* b, cudaStream_t s) {
  batch_fold<<<row_grid(b), kBatchRowThreads, 0, s>>>(b->sys, b->st, b->vtiles, b->n_vtiles, nullptr, b->vpart,
                                                      b->ctl);
  batch_reliable<<<slice_grid(b), b->slice_threads, 0, s>>>(b->sys, b->st, b->stiles, b->n_stiles, b->rpart,
                                                            b->ctl);
  batch_reliable_fin<<<b->max_sys, kSysThreads, 0, s>>>(b->max_sys, b->st, b->stile_ptr, b->rpart, b->sys,
                                                         b->ctl);
}

// while (running && trips < limit) { iteration ; if (update due) reliable }
int build_graph(fgb_batch* b) {
  cudaGraph_t g = nullptr;
  if (cudaGraphCreate(&g, 0) != cudaSuccess) return FGB_ERR_CUDA;
  cudaGraphConditionalHandle hw, hif;
  int rc = FGB_OK;
  cudaStream_t cs = nullptr;
  do {
    if (cudaGraphConditionalHandleCreate(&hw, g, 1, cudaGraphCondAssignDefault) != cudaSuccess) { rc = FGB_ERR_CUDA; break; }
    cudaGraphNodeParams wp = {};
    wp.type = cudaGraphNodeTypeConditional;
    wp.conditional.handle = hw;
    wp.conditional.type = cudaGraphCondTypeWhile;
    wp.conditional.size = 1;
    cudaGraphNode_t wnode;
    if (cudaGraphAddNode(&wnode, g, nullptr, nullptr, 0, &wp) != cudaSuccess) { rc = FGB_ERR_CUDA; break; }
    cudaGraph_t body = wp.conditional.phGraph_out[0];
    if (cudaGraphConditionalHandleCreate(&hif, body, 0, cudaGraphCondAssignDefault) != cudaSuccess) { rc = FGB_ERR_CUDA; break; }
    if (cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking) != cudaSuccess) { rc = FGB_ERR_CUDA; cs = nullptr; break; }
    if (cudaStreamBeginCaptureToGraph(cs, body, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed) != cudaSuccess) {
      rc = FGB_ERR_CUDA;
      break;
    }
    launch_iteration(b, cs, 1, hif, hw);
    // IF node on hif after the control kernel
    cudaStreamCaptureStatus status;
    cudaGraph_t cg = nullptr;
    const cudaGraphNode_t* deps = nullptr;
    size_t nd = 0;
    bool ok = cudaStreamGetCaptureInfo(cs, &status, nullptr, &cg, &deps, nullptr, &nd) == cudaSuccess &&
              status == cudaStreamCaptureStatusActive;
    cudaGraphNodeParams ip = {};
    cudaGraphNode_t inode;
    if (ok) {
      ip.type = cudaGraphNodeTypeConditional;
      ip.conditional.handle = hif;
      ip.conditional.type = cudaGraphCondTypeIf;
      ip.conditional.size = 1;
      ok = cudaGraphAddNode(&inode, cg, deps, nullptr, nd, &ip) == cudaSuccess &&
           cudaStreamUpdateCaptureDependencies(cs, &inode, nullptr, 1, cudaStreamSetCaptureDependencies) == cudaSuccess;
    }
    cudaGraph_t out = nullptr;
    const bool ended = cudaStreamEndCapture(cs, &out) == cudaSuccess;
    if (!ok || !ended) { rc = FGB_ERR_CUDA; break; }
    cudaStream_t bs = nullptr;
    if (cudaStreamCreateWithFlags(&bs, cudaStreamNonBlocking) != cudaSuccess) { rc = FGB_ERR_CUDA; break; }
    if (cudaStreamBeginCaptureToGraph(bs, ip.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                      cudaStreamCaptureModeRelaxed) != cudaSuccess) {
      rc = FGB_ERR_CUDA;
    } else {
      launch_reliable(b, bs);
      cudaGraph_t o2 = nullptr;
      if (cudaStreamEndCapture(bs, &o2) != cudaSuccess) rc = FGB_ERR_CUDA;
    }
    cudaStreamDestroy(bs);
    if (rc) break;
    if (cudaGraphInstantiate(&b->exec, g, 0) != cudaSuccess) { b->exec = nullptr; rc = FGB_ERR_CUDA; break; }
  } while (false);
  if (cs) cudaStreamDestroy(cs);
  if (rc) {
    cudaGraphDestroy(g);
    cudaGetLastError();
    return rc;
  }
  b->graph = g;
  return FGB_OK;
}

bool valid_tiles(int32_t n_sys, const fgb_batch_system* sys, int32_t nt, const fgb_batch_tile* tiles,
                 const int32_t* ptr, bool slices) {
  if (ptr[0] != 0 || ptr[n_sys] != nt) return false;
  for (int32_t s = 0; s < n_sys; ++s) {
    if (ptr[s + 1] < ptr[s]) return false;
    const int64_t lim = slices ? sys[s].n_slices : sys[s].n;
    for (int32_t t = ptr[s]; t < ptr[s + 1]; ++t) {
      if (tiles[t].sys != s || tiles[t].begin < 0 || tiles[t].begin >= tiles[t].end || tiles[t].end > lim) return false;
    }
  }
  return true;
}

}  // namespace

extern "C" {

size_t fgb_batch_bytes(int32_t max_sys, int32_t max_slice_tiles, int32_t max_row_tiles) {
  if (max_sys <= 0 || max_slice_tiles <= 0 || max_row_tiles <= 0) return 0;
  // sizes only: an aligned stand-in base address that is never dereferenced
  void* probe = reinterpret_cast<void*>(static_cast<uintptr_t>(256));
  return batch_layout(max_sys, max_slice_tiles, max_row_tiles, nullptr, probe, static_cast<size_t>(1) << 40);
}

int32_t fgb_batch_create(int32_t max_sys, int32_t max_slice_tiles, int32_t max_row_tiles, int32_t slice_threads,
                         void* device_buffer, size_t bytes, fgb_batch** out) {
  if (!out || max_sys <= 0 || max_slice_tiles <= 0 || max_row_tiles <= 0) return FGB_ERR_ARG;
  if (slice_threads < 64 || slice_threads > 1024 || slice_threads % 32) return FGB_ERR_ARG;
  if (!device_buffer || bytes < fgb_batch_bytes(max_sys, max_slice_tiles, max_row_tiles)) return FGB_ERR_WORKSPACE;
  fgb_batch* b = new (std::nothrow) fgb_batch;
  if (!b) return FGB_ERR_CAPACITY;
  b->max_sys = max_sys; b->max_st = max_slice_tiles; b->max_vt = max_row_tiles; b->slice_threads = slice_threads;
  if (batch_layout(max_sys, max_slice_tiles, max_row_tiles, b, device_buffer, bytes) == 0) {
    delete b;
    return FGB_ERR_WORKSPACE;
  }
  // every slot inactive, no tiles, zero force flags
  if (cudaMemset(device_buffer, 0, bytes) != cudaSuccess) { delete b; return FGB_ERR_CUDA; }
  *out = b;
  return FGB_OK;
}

int32_t fgb_batch_destroy(fgb_batch* b) {
  if (!b) return FGB_ERR_ARG;
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  delete b;
  return FGB_OK;
}

int32_t fgb_batch_set(fgb_batch* b, int32_t n_sys, const fgb_batch_system* systems, int32_t n_slice_tiles,
                      const fgb_batch_tile* slice_tiles, const int32_t* slice_tile_ptr, int32_t n_row_tiles,
                      const fgb_batch_tile* row_tiles, const int32_t* row_tile_ptr, void* stream) {
  if (!b || n_sys < 0 || n_sys > b->max_sys || n_slice_tiles < 0 || n_slice_tiles > b->max_st || n_row_tiles < 0 ||
      n_row_tiles > b->max_vt)
    return FGB_ERR_ARG;
  if (n_sys > 0 && (!systems || !slice_tile_ptr || !row_tile_ptr)) return FGB_ERR_ARG;
  for (int32_t s = 0; s < n_sys; ++s) {
    const fgb_batch_system& A = systems[s];
    if (A.n <= 0) continue;  // an empty slot: it must own no tiles
    if (A.n >= (int64_t(1) << 31) || A.n_slices != fgb_sell_slots(A.n) / kSellC || !A.slice_ptr || !A.perm ||
        !A.col || !A.dinv64 || !A.b || !A.x || !A.r || !A.z || !A.p || !A.Ap || !A.y)
      return FGB_ERR_ARG;
    if (A.fp64 ? !A.val64 : (!A.val32 || !A.dinv32)) return FGB_ERR_ARG;
  }
  if (n_sys > 0 && (!valid_tiles(n_sys, systems, n_slice_tiles, slice_tiles, slice_tile_ptr, true) ||
                    !valid_tiles(n_sys, systems, n_row_tiles, row_tiles, row_tile_ptr, false)))
    return FGB_ERR_ARG;
  cudaStream_t s = as_stream(stream);
  // tile pointers padded to max_sys + 1 entries (the kernels walk every slot)
  int32_t* sp = new (std::nothrow) int32_t[2 * (b->max_sys + 1) + 2];
  if (!sp) return FGB_ERR_CAPACITY;
  int32_t* vp = sp + (b->max_sys + 1);
  for (int32_t k = 0; k <= b->max_sys; ++k) {
    sp[k] = n_sys > 0 ? slice_tile_ptr[k < n_sys ? k : n_sys] : 0;
    vp[k] = n_sys > 0 ? row_tile_ptr[k < n_sys ? k : n_sys] : 0;
  }
  int32_t* counts = vp + (b->max_sys + 1);
  counts[0] = n_slice_tiles;
  counts[1] = n_row_tiles;
  bool ok = true;
  if (n_sys > 0) ok = ok && cudaMemcpyAsync(b->sys, systems, n_sys * sizeof(fgb_batch_system), cudaMemcpyHostToDevice, s) == cudaSuccess;
  if (n_slice_tiles > 0)
    ok = ok && cudaMemcpyAsync(b->stiles, slice_tiles, n_slice_tiles * sizeof(fgb_batch_tile), cudaMemcpyHostToDevice, s) == cudaSuccess;
  if (n_row_tiles > 0)
    ok = ok && cudaMemcpyAsync(b->vtiles, row_tiles, n_row_tiles * sizeof(fgb_batch_tile), cudaMemcpyHostToDevice, s) == cudaSuccess;
  ok = ok && cudaMemcpyAsync(b->stile_ptr, sp, (b->max_sys + 1) * sizeof(int32_t), cudaMemcpyHostToDevice, s) == cudaSuccess;
  ok = ok && cudaMemcpyAsync(b->vtile_ptr, vp, (b->max_sys + 1) * sizeof(int32_t), cudaMemcpyHostToDevice, s) == cudaSuccess;
  ok = ok && cudaMemcpyAsync(b->n_stiles, counts, 2 * sizeof(int32_t), cudaMemcpyHostToDevice, s) == cudaSuccess;
  ok = ok && cudaStreamSynchronize(s) == cudaSuccess;  // the host arrays are freed below
  delete[] sp;
  if (!ok) return FGB_ERR_CUDA;
  b->n_sys = n_sys; b->n_st = n_slice_tiles; b->n_vt = n_row_tiles;
  return FGB_OK;
}

int32_t fgb_batch_admit(fgb_batch* b, int32_t n, const int32_t* slots, const double* rtol, const int64_t* maxit,
                        double delta, void* stream) {
  if (!b || n < 0 || (n > 0 && (!slots || !rtol || !maxit))) return FGB_ERR_ARG;
  if (!(delta > 0.0 && delta < 1.0)) return FGB_ERR_ARG;
  cudaStream_t s = as_stream(stream);
  for (int32_t k = 0; k < n; ++k) {
    if (slots[k] < 0 || slots[k] >= b->n_sys || !(rtol[k] > 0.0) || maxit[k] <= 0) return FGB_ERR_ARG;
    fgb_batch_state h;
    std::memset(&h, 0, sizeof(h));
    h.tol = rtol[k];  // batch_bnorm turns it into rtol * ||b||
    h.delta = delta;
    h.maxit = maxit[k];
    h.active = 1;
    h.need_update = 2;
    if (cudaMemcpyAsync(b->st + slots[k], &h, sizeof(h), cudaMemcpyHostToDevice, s) != cudaSuccess) return FGB_ERR_CUDA;
    if (cudaStreamSynchronize(s) != cudaSuccess) return FGB_ERR_CUDA;  // h lives on this stack frame
  }
  if (n == 0) return FGB_OK;
  batch_fold<<<row_grid(b), kBatchRowThreads, 0, s>>>(b->sys, b->st, b->vtiles, b->n_vtiles, nullptr, b->vpart,
                                                      b->ctl);
  batch_bnorm<<<b->max_sys, kSysThreads, 0, s>>>(b->max_sys, b->st, b->vtile_ptr, b->vpart, b->ctl);
  batch_reliable<<<slice_grid(b), b->slice_threads, 0, s>>>(b->sys, b->st, b->stiles, b->n_stiles, b->rpart,
                                                            b->ctl);
  batch_reliable_fin<<<b->max_sys, kSysThreads, 0, s>>>(b->max_sys, b->st, b->stile_ptr, b->rpart, b->sys,
                                                         b->ctl);
  return launch_status();
}

int32_t fgb_batch_run(fgb_batch* b, int64_t trip_limit, int32_t use_graph, fgb_batch_state* states_host,
                      int32_t* running, int32_t* used_graph, void* stream) {
  if (!b || trip_limit <= 0) return FGB_ERR_ARG;
  cudaStream_t s = as_stream(stream);
  BatchCtl c{};
  c.trip_limit = trip_limit;
  if (cudaMemcpyAsync(b->ctl, &c, sizeof(c), cudaMemcpyHostToDevice, s) != cudaSuccess) return FGB_ERR_CUDA;
  bool graphed = false;
  if (use_graph && !b->graph_failed) {
    if (!b->exec && build_graph(b) != FGB_OK) b->graph_failed = true;
    if (b->exec) {
      if (cudaGraphLaunch(b->exec, s) != cudaSuccess) return FGB_ERR_CUDA;
      graphed = true;
    }
  }
  if (!graphed) {
    // host-driven: the same kernels, the reliable branch launched every trip
    // (its kernels return at once for systems without an update due)
    const int chunk = 16;
    while (true) {
      for (int k = 0; k < chunk; ++k) {
        launch_iteration(b, s, 0, 0, 0);
        launch_reliable(b, s);
      }
      if (cudaGetLastError() != cudaSuccess) return FGB_ERR_CUDA;
      if (cudaMemcpyAsync(&c, b->ctl, sizeof(c), cudaMemcpyDeviceToHost, s) != cudaSuccess) return FGB_ERR_CUDA;
      if (cudaStreamSynchronize(s) != cudaSuccess) return FGB_ERR_CUDA;
      if (!c.running || c.trips >= trip_limit) break;
    }
  }
  if (cudaMemcpyAsync(&c, b->ctl, sizeof(c), cudaMemcpyDeviceToHost, s) != cudaSuccess) return FGB_ERR_CUDA;
  if (states_host && b->n_sys > 0 &&
      cudaMemcpyAsync(states_host, b->st, b->n_sys * sizeof(fgb_batch_state), cudaMemcpyDeviceToHost, s) != cudaSuccess)
    return FGB_ERR_CUDA;
  if (cudaStreamSynchronize(s) != cudaSuccess) return FGB_ERR_CUDA;
  if (running) *running = c.running;
  if (used_graph) *used_graph = graphed ? 1 : 0;
  return FGB_OK;
}

int32_t fgb_batch_retire(fgb_batch* b, int32_t n, const int32_t* slots, void* stream) {
  if (!b || n < 0 || (n > 0 && !slots)) return FGB_ERR_ARG;
  if (n == 0) return FGB_OK;
  cudaStream_t s = as_stream(stream);
  int32_t* flags = new (std::nothrow) int32_t[b->max_sys];
  if (!flags) return FGB_ERR_CAPACITY;
  std::memset(flags, 0, sizeof(int32_t) * b->max_sys);
  for (int32_t k = 0; k < n; ++k) {
    if (slots[k] < 0 || slots[k] >= b->n_sys) { delete[] flags; return FGB_ERR_ARG; }
    flags[slots[k]] = 1;
  }
  bool ok = cudaMemcpyAsync(b->force, flags, sizeof(int32_t) * b->max_sys, cudaMemcpyHostToDevice, s) == cudaSuccess;
  ok = ok && cudaStreamSynchronize(s) == cudaSuccess;
  delete[] flags;
  if (!ok) return FGB_ERR_CUDA;
  batch_fold<<<row_grid(b), kBatchRowThreads, 0, s>>>(b->sys, b->st, b->vtiles, b->n_vtiles, b->force, b->vpart,
                                                      b->ctl);
  batch_deactivate<<<sys_blocks(b->max_sys), 256, 0, s>>>(b->max_sys, b->st, b->force, b->ctl);
  return launch_status();
}

int32_t fgb_batch_spmv(fgb_batch* b, const float* const* x, float* const* y, void* stream) {
  if (!b || (b->n_sys > 0 && (!x || !y))) return FGB_ERR_ARG;
  if (b->n_sys == 0) return FGB_OK;
  cudaStream_t s = as_stream(stream);
  bool ok = cudaMemcpyAsync(b->xs, x, b->n_sys * sizeof(float*), cudaMemcpyHostToDevice, s) == cudaSuccess &&
            cudaMemcpyAsync(b->ys, y, b->n_sys * sizeof(float*), cudaMemcpyHostToDevice, s) == cudaSuccess;
  if (!ok) return FGB_ERR_CUDA;
  batch_spmv_plain<<<slice_grid(b), b->slice_threads, 0, s>>>(b->sys, b->stiles, b->n_stiles, b->xs, b->ys);
  return launch_status();
}

}  // extern "C"
