// SELL-32 (sliced ELLPACK, rows sorted by length inside windows of 256 rows)
// copy of a CSR matrix, its SpMV, and the Jacobi-PCG solvers that iterate on it.
//
// Why: the CG time is the SpMV, and a CSR SpMV with a few lanes per row keeps
// too few bytes in flight to cover HBM latency (rows here hold 10-80 entries).
// In SELL-32 a warp owns 32 rows; entry k of those rows sits in one 128-byte
// line (column-major inside the slice), so every load instruction of the warp
// is a full coalesced line, each lane accumulates its own row with no shuffles,
// and the k-loop is unrolled so several lines per warp are in flight.  Sorting
// rows by length inside 256-row windows keeps the zero padding small while
// preserving locality of the gathered vector entries.
//
// The solvers keep every vector in the original row order; only the matrix is
// permuted (slot -> row map `perm`).  Two drivers are provided: host polling of
// a device flag (as in krylov.cu) and a CUDA graph whose while-conditional node
// runs the iteration body on the device until a loop-control kernel clears the
// condition (converged, breakdown, iteration limit, or a hard trip cap).

#include "fgb_common.cuh"
#include "sell_rows.cuh"

#include <climits>
#include <cmath>
#include <cstring>
#include <type_traits>

namespace fgb {

constexpr int kSellThreads = 256;
constexpr int kSellMaxBlocks = kNumSMs * 8;

struct SellView {
  int64_t n, n_slices;
  const int64_t* slice_ptr;
  const int32_t* perm;
  const int32_t* col;
  int threads;  // launch shape of the slice kernels (0: defaults)
  int blocks;
  const uint16_t* col16;  // delta-coded columns (then col is unused) or null
  const int32_t* col0;    // first column of every slot's row (delta-coded copies)
  int node_triples;       // 1: slots are node triples (col = 3c, three values each)
  int d15;                // 1: col16 holds 15-bit steps and long steps (own numbering)
};

// Storage formats of a SELL copy: 4-byte columns, 16-bit column steps
// (renumbered matrix), node triples, 15-bit steps with long steps (own
// numbering).
constexpr int kColsI32 = 0, kColsD16 = 1, kColsB3 = 2, kColsD15 = 3;

// Row of slot (s, lane): sum over entries of val * g(col), for each storage
// format.  The slice width is a multiple of 4 slots.
template <int FMT, typename V, typename T, typename G>
__device__ __forceinline__ T slice_row(const SellView& A, const V* __restrict__ val, int64_t s, int lane,
                                       const G& g) {
  const int64_t sbase = A.slice_ptr[s];
  const int w = static_cast<int>((A.slice_ptr[s + 1] - sbase) >> 5);
  if constexpr (FMT == kColsD16)
    return sell_row_acc_d16<V, T>(A.col16, A.col0[s * kSellC + lane], val, sbase, w, lane, g);
  else if constexpr (FMT == kColsD15)
    return sell_row_acc_d15<V, T>(A.col16, A.col0[s * kSellC + lane], val, sbase, w, lane, g);
  else if constexpr (FMT == kColsB3)
    return sell_row_acc_b3<V, T>(A.col, val, sbase, w, lane, g);
  else
    return sell_row_acc<V, T>(A.col, val, sbase, w, lane, g);
}

// Launch `f(std::integral_constant<int, FMT>)` for the storage format of A.
template <typename F>
void with_cols(const SellView& A, F&& f) {
  if (A.node_triples) f(std::integral_constant<int, kColsB3>{});
  else if (A.col16 && A.d15) f(std::integral_constant<int, kColsD15>{});
  else if (A.col16) f(std::integral_constant<int, kColsD16>{});
  else f(std::integral_constant<int, kColsI32>{});
}

// Launch shapes.  Vector kernels: two 512-thread blocks per SM (few blocks
// shorten the tail of the deterministic block reduction; measured at 2.1M rows:
// 16.5 us for the mixed update against 20.5 us with one 1024-thread block per
// SM and 24 us with eight 256-thread blocks).  Slice kernels: the shape carried
// by the SELL descriptor (chosen by the autotuner), else 256 threads and up to
// 8 blocks per SM.
struct Launch {
  int blocks, threads;
};

constexpr int kVecThreads = 512;
constexpr int kVecBlocks = 2 * kNumSMs;

inline Launch vec_launch(int64_t n) {
  const int64_t b = (n + kVecThreads - 1) / kVecThreads;
  return {static_cast<int>(b < 1 ? 1 : (b > kVecBlocks ? kVecBlocks : b)), kVecThreads};
}

inline Launch slice_launch(const SellView& A) {
  const int t = A.threads > 0 ? A.threads : kSellThreads;
  const int cap = A.blocks > 0 ? A.blocks : kSellMaxBlocks;
  int64_t b = (A.n_slices * 32 + t - 1) / t;
  if (b < 1) b = 1;
  if (b > cap) b = cap;
  return {static_cast<int>(b), t};
}

#define SLICE_LAUNCH(A, s) slice_launch(A).blocks, slice_launch(A).threads, 0, s

// blocks of a slice-kernel launch (one p.Ap partial each)
inline int slice_blocks(const SellView& A) { return slice_launch(A).blocks; }
#define VEC_LAUNCH(n, s) vec_launch(n).blocks, vec_launch(n).threads, 0, s

// both pointers 16-byte aligned (vector kernels take 16-byte accesses then)
__device__ __forceinline__ bool aligned16(const void* a, const void* b) {
  return ((reinterpret_cast<uintptr_t>(a) | reinterpret_cast<uintptr_t>(b)) & 15u) == 0;
}

// -------------------------------------------------------------- construction
__global__ void sell_sort_windows(int64_t n, const int64_t* __restrict__ indptr, int32_t* __restrict__ perm,
                                  int32_t* __restrict__ slice_entries) {
  __shared__ unsigned long long key[kSellWindow];
  const int64_t base = static_cast<int64_t>(blockIdx.x) * kSellWindow;
  const int64_t row = base + threadIdx.x;
  int len = -1;
  if (row < n) len = static_cast<int>(indptr[row + 1] - indptr[row]);
  // ascending on (INT_MAX - len, local row): longest rows first, padding rows
  // (len = -1) last, ties in row order
  const unsigned long long hi = static_cast<unsigned long long>(static_cast<long long>(INT_MAX) - len);
  key[threadIdx.x] = (hi << 32) | static_cast<unsigned long long>(threadIdx.x);
  __syncthreads();
  for (int k = 2; k <= kSellWindow; k <<= 1) {
    for (int j = k >> 1; j > 0; j >>= 1) {
      const int t = threadIdx.x, u = t ^ j;
      if (u > t) {
        unsigned long long a = key[t], b = key[u];
        bool up = (t & k) == 0;
        if ((a > b) == up) { key[t] = b; key[u] = a; }
      }
      __syncthreads();
    }
  }
  const unsigned long long kk = key[threadIdx.x];
  const int slen = static_cast<int>(static_cast<long long>(INT_MAX) - static_cast<long long>(kk >> 32));
  const int64_t full = base + static_cast<int64_t>(kk & 0xffffffffu);
  const int64_t slot = base + threadIdx.x;
  perm[slot] = (slen >= 0 && full < n) ? static_cast<int32_t>(full) : -1;
  // the first slot of a slice holds its longest row: that is the slice width,
  // rounded up to whole packs of kSellPack entries
  if ((threadIdx.x & 31) == 0) {
    const int w = slen > 0 ? slen : 0;
    slice_entries[slot / kSellC] = kSellC * ((w + kSellPack - 1) / kSellPack) * kSellPack;
  }
}

__global__ void sell_fill_kernel(int64_t n_slices, const int64_t* __restrict__ slice_ptr,
                                 const int32_t* __restrict__ perm, const int64_t* __restrict__ indptr,
                                 const int32_t* __restrict__ indices, const double* __restrict__ v64,
                                 const float* __restrict__ v32, int32_t* __restrict__ scol, double* __restrict__ s64,
                                 float* __restrict__ s32) {
  const int lane = threadIdx.x & 31;
  const int64_t warp = (blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x) >> 5;
  const int64_t nwarps = (static_cast<int64_t>(gridDim.x) * blockDim.x) >> 5;
  for (int64_t s = warp; s < n_slices; s += nwarps) {
    const int64_t base = slice_ptr[s];
    const int w = static_cast<int>((slice_ptr[s + 1] - base) / kSellC);
    const int32_t row = perm[s * kSellC + lane];
    int64_t rs = 0;
    int len = 0;
    if (row >= 0) { rs = indptr[row]; len = static_cast<int>(indptr[row + 1] - rs); }
    for (int k = 0; k < w; ++k) {
      const int64_t pos = base + sell_pos(lane, k);
      const bool real = k < len;
      scol[pos] = real ? indices[rs + k] : (row >= 0 ? row : 0);
      if (s64) s64[pos] = real ? v64[rs + k] : 0.0;
      if (s32) s32[pos] = real ? (v64 ? static_cast<float>(v64[rs + k]) : v32[rs + k]) : 0.0f;
    }
  }
}

// ------------------------------------------------------------------- SpMV
template <typename T, int FMT>
__global__ void __launch_bounds__(1024, 1) sell_spmv_kernel(SellView A, const T* __restrict__ val,
                                                                 const T* __restrict__ x, T* __restrict__ y) {
  const int lane = threadIdx.x & 31;
  const int64_t warp = (blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x) >> 5;
  const int64_t nwarps = (static_cast<int64_t>(gridDim.x) * blockDim.x) >> 5;
  const GatherX<T> g{x};
  for (int64_t s = warp; s < A.n_slices; s += nwarps) {
    const T acc = slice_row<FMT, T, T>(A, val, s, lane, g);
    const int32_t row = A.perm[s * kSellC + lane];
    if (row >= 0) y[row] = acc;
  }
}

// Smoother sweep of an FP32 copy (a multigrid level matrix): mode 0, a
// Chebyshev step d = c1 d + c2 dinv (r - A x_in), x_out = x_in + d (d is not
// read when c1 = 0); mode 1, the residual x_out = r - A x_in.
template <int FMT, typename T>
__global__ void __launch_bounds__(1024, 1) sell_smooth_kernel(SellView A, const T* __restrict__ val,
                                                               const T* __restrict__ dinv, const T* __restrict__ r,
                                                               const T* __restrict__ x_in, T* __restrict__ x_out,
                                                               T* __restrict__ d, T c1, T c2, int mode) {
  const int lane = threadIdx.x & 31;
  const int64_t warp = (blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x) >> 5;
  const int64_t nwarps = (static_cast<int64_t>(gridDim.x) * blockDim.x) >> 5;
  const GatherX<T> g{x_in};
  for (int64_t s = warp; s < A.n_slices; s += nwarps) {
    const T acc = slice_row<FMT, T, T>(A, val, s, lane, g);
    const int32_t row = A.perm[s * kSellC + lane];
    if (row < 0) continue;
    const T res = r[row] - acc;
    if (mode) {
      x_out[row] = res;
    } else {
      const T di = (c1 != T(0) ? c1 * d[row] : T(0)) + c2 * dinv[row] * res;
      d[row] = di;
      x_out[row] = x_in[row] + di;
    }
  }
}

// Ap = A p (FP64 values) with per-block p.Ap partials in bpart (warps'
// sums combined in warp order by the block's last warp).
template <int FMT>
__global__ void __launch_bounds__(1024, 1) sell_spmv_pap_kernel(SellView A, const double* __restrict__ val,
                                                                 const double* __restrict__ p,
                                                                 double* __restrict__ Ap, double* bpart) {
  __shared__ double wslot[32];
  __shared__ unsigned int arrivals;
  if (threadIdx.x == 0) arrivals = 0u;
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int64_t warp = (blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x) >> 5;
  const int64_t nwarps = (static_cast<int64_t>(gridDim.x) * blockDim.x) >> 5;
  double pap = 0.0;
  for (int64_t s = warp; s < A.n_slices; s += nwarps) {
    const double acc = slice_row<FMT, double, double>(A, val, s, lane, GatherX<double>{p});
    const int32_t row = A.perm[s * kSellC + lane];
    if (row >= 0) {
      Ap[row] = acc;
      pap += p[row] * acc;
    }
  }
  pap = warp_sum(pap);
  if (lane == 0) {
    const unsigned int nw = blockDim.x >> 5;
    wslot[threadIdx.x >> 5] = pap;
    __threadfence_block();
    if (atomicAdd(&arrivals, 1u) == nw - 1) {
      __threadfence_block();
      const volatile double* ws = wslot;
      double t = 0.0;
      for (unsigned int k = 0; k < nw; ++k) t += ws[k];
      bpart[blockIdx.x] = t;
    }
  }
}

// ------------------------------------------------------------ PCG kernels
struct SellPcgState {
  double rz, rz_prev, rr, alpha, beta, b_norm, tol, atol, resid, r_upd, true_rel;
  long long niter, maxit, trips, trip_cap;
  int done, need_update, n_updates, norm_rr;
  unsigned int counter[4];
  // mixed solver, plateau detection: best true residual, reliable updates in a
  // row without halving it, iteration of the last update, longest gap between
  // updates triggered by the residual estimate
  double r_best;
  long long last_upd, max_gap;
  int stall, pad;
  // persistent solver: grid barrier (arrivals, generation) and its error flag
  unsigned int bar[2];
  int bar_err, pad2;
};

// Scalar step of the mixed solver after an FP32 iteration (totals r.z, r.r):
// the iteration count, the residual estimate, whether a reliable update (1)
// or a check of the true residual on a plateau (3) is due, and beta.
__device__ void mixed_iteration_scalars(SellPcgState& S, double trz, double trr, double delta) {
  S.niter += 1;
  const double res = sqrt(trr);
  S.resid = res;
  S.rr = trr;
  if (!isfinite(res)) {
    S.done = FGB_PCG_NONFINITE;
  } else {
    // a check of the true residual when the gap since the last update has
    // grown well past the longest earlier one (FP32 iterations on a plateau)
    const long long gap = S.niter - S.last_upd;
    const long long slack = S.max_gap / 2 > 100 ? S.max_gap / 2 : 100;
    const bool plateau = S.max_gap > 0 ? gap > S.max_gap + slack : gap > 1000;
    const bool due = (res < delta * S.r_upd) || (res < S.tol) || (S.niter >= S.maxit);
    S.need_update = due ? 1 : (plateau ? 3 : 0);
  }
  S.rz_prev = S.rz;
  S.beta = trz / S.rz;
  S.rz = trz;
}

// Scalar step of a reliable update (totals of the FP64 residual r64.r64 and of
// the replaced r.z): true-residual test, stall rule, beta from the replaced
// residual.  first = 1 at the start of the solve.
__device__ void mixed_reliable_scalars(SellPcgState& S, double trr, double trz, int first) {
  const double nrm = sqrt(trr);
  S.true_rel = S.b_norm > 0.0 ? nrm / S.b_norm : 0.0;
  S.resid = nrm;
  if (!first) {
    S.n_updates += 1;
    const long long gap = S.niter - S.last_upd;
    if (S.need_update == 1 && gap > S.max_gap) S.max_gap = gap;
    S.last_upd = S.niter;
    if (nrm < 0.5 * S.r_best) {
      S.r_best = nrm;
      S.stall = 0;
    } else {
      S.stall += 1;
    }
  } else {
    S.r_best = nrm;
    S.last_upd = 0;
  }
  if (!isfinite(nrm)) S.done = FGB_PCG_NONFINITE;
  else if (nrm <= S.tol) S.done = FGB_PCG_RTOL;
  else if (S.niter >= S.maxit) S.done = FGB_PCG_MAXIT;
  else if (S.stall >= 1) S.done = FGB_PCG_STAGNATED;  // the caller continues in FP64
  S.beta = first ? 0.0 : trz / S.rz_prev;
  S.rz = trz;
  S.rr = trr;
  S.r_upd = nrm;
  S.need_update = 0;
}

// Last-block-done deterministic reduction of two partials per thread (T =
// float: FP32 per-thread and per-warp sums, as in the FP32 iterations; T =
// double: FP64 throughout).  Per block: warp shuffles, one barrier, then warp
// 0 alone adds the warps' sums in FP64, publishes the block's partials and
// takes a ticket; warp 0 of the last block loads all partials (unrolled, a
// round trip per 320 blocks) and adds them in block order.  FP64 arithmetic is
// kept to a few lanes: its rate on this part is a small fraction of FP32.  The
// totals are valid in thread 0 of the last block, the only thread that returns
// true.  Must be the last block-wide step of the calling kernel: warps other
// than 0 return at once.
template <typename T>
__device__ bool sell_last_block(T v0, T v1, double* partials, unsigned int* counter, double* out0, double* out1) {
  __shared__ double2 ws[32];  // one slot per warp of a block of up to 1024 threads
  constexpr int kPer = 10;    // partials per lane and round trip
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  v0 = warp_sum(v0);
  v1 = warp_sum(v1);
  if (lane == 0) ws[wid] = make_double2(static_cast<double>(v0), static_cast<double>(v1));
  __syncthreads();
  if (wid != 0) return false;
  const int nw = (blockDim.x + 31) >> 5;
  double2 t = lane < nw ? ws[lane] : make_double2(0.0, 0.0);
  t.x = warp_sum(t.x);
  t.y = warp_sum(t.y);
  unsigned int ticket = 0u;
  if (lane == 0) {
    partials[blockIdx.x] = t.x;
    partials[kSellMaxBlocks + blockIdx.x] = t.y;
    __threadfence();
    ticket = atomicAdd(counter, 1u);
  }
  ticket = __shfl_sync(0xffffffffu, ticket, 0);
  if (ticket != gridDim.x - 1) return false;
  __threadfence();
  const int nb = static_cast<int>(gridDim.x);
  double a = 0.0, b = 0.0;
  for (int base = 0; base < nb; base += 32 * kPer) {
    double pa[kPer], pb[kPer];
#pragma unroll
    for (int u = 0; u < kPer; ++u) {
      const int k = base + lane + 32 * u;
      pa[u] = k < nb ? __ldcg(partials + k) : 0.0;
      pb[u] = k < nb ? __ldcg(partials + kSellMaxBlocks + k) : 0.0;
    }
#pragma unroll
    for (int u = 0; u < kPer; ++u) {
      a += pa[u];
      b += pb[u];
    }
  }
  a = warp_sum(a);
  b = warp_sum(b);
  if (lane == 0) { *out0 = a; *out1 = b; *counter = 0u; }
  return lane == 0;
}

#define SELL_WARP_LOOP(A)                                                                   \
  const int lane = threadIdx.x & 31;                                                        \
  const int64_t warp0 = (blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x) >> 5; \
  const int64_t nwarps = (static_cast<int64_t>(gridDim.x) * blockDim.x) >> 5;               \
  for (int64_t s = warp0; s < (A).n_slices; s += nwarps)

// r = b - A x ; z = Dinv r ; p = z ; rz, b.b   (T = FP64 state)
template <typename T, int FMT>
__global__ void __launch_bounds__(1024, 1) sell_pcg_init(SellView A, const T* __restrict__ val,
                                                              const T* __restrict__ dinv, const T* __restrict__ b,
                                                              const T* __restrict__ x, T* __restrict__ r,
                                                              T* __restrict__ z, T* __restrict__ p, double* partials,
                                                              SellPcgState* st) {
  double rz = 0.0, bb = 0.0;
  SELL_WARP_LOOP(A) {
    const T acc = slice_row<FMT, T, T>(A, val, s, lane, GatherX<T>{x});
    const int32_t row = A.perm[s * kSellC + lane];
    if (row >= 0) {
      const T bi = b[row];
      const T ri = bi - acc;
      const T zi = dinv ? dinv[row] * ri : ri;
      r[row] = ri; z[row] = zi; p[row] = zi;
      rz += static_cast<double>(ri) * static_cast<double>(zi);
      bb += static_cast<double>(bi) * static_cast<double>(bi);
    }
  }
  double trz, tbb;
  if (sell_last_block(rz, bb, partials, &st->counter[0], &trz, &tbb) && threadIdx.x == 0) {
    st->rz = trz;
    st->rr = trz;
    st->b_norm = sqrt(tbb);
    st->beta = 0.0;
    st->niter = 0;
    st->n_updates = 0;
    st->need_update = 0;
    if (st->b_norm < 1e-15) st->done = FGB_PCG_ZERO_RHS;
  }
}

// alpha = rz / p.Ap for the update kernels.  p.Ap is the sum of the SpMV
// step's per-block partials, formed by warp 0 of every block of the consuming
// kernel in the same order, so that all blocks hold the bitwise-same value
// without a grid-wide reduction in the SpMV kernel (a last-block pass there
// adds a serial tail of a few microseconds).  Warp 0 loads the partials
// unrolled (a round trip per 608), adds them and lane 0 divides, so that the
// FP64 work stays on one warp; it also reads the done flag (block 0 may set it
// on breakdown while other blocks start), and one barrier hands both to the
// block, so that all its threads take the same branch; the other warps issue
// their first vector loads meanwhile.  Returns false (and block 0 marks the
// solve done) on breakdown or non-finite values, or when the solve has already
// ended: the block then returns without touching the vectors.
__device__ bool block_alpha(const double* bpart, int nwp, SellPcgState* st, double* alpha) {
  __shared__ double sh_alpha;
  __shared__ int sh_ok;
  constexpr int kPer = 19;
  if (threadIdx.x < 32) {
    const int lane = threadIdx.x;
    double acc = 0.0;
    for (int base = 0; base < nwp; base += 32 * kPer) {
      double v[kPer];
#pragma unroll
      for (int u = 0; u < kPer; ++u) {
        const int k = base + lane + 32 * u;
        v[u] = k < nwp ? __ldcg(bpart + k) : 0.0;
      }
#pragma unroll
      for (int u = 0; u < kPer; ++u) acc += v[u];
    }
    const double pap = warp_sum(acc);
    if (lane == 0) {
      const int done = *reinterpret_cast<const volatile int*>(&st->done);
      const bool ok = !done && pap > 0.0 && isfinite(pap);
      if (!done && !ok && blockIdx.x == 0) {
        st->done = isfinite(pap) ? FGB_PCG_BREAKDOWN : FGB_PCG_NONFINITE;
        st->alpha = 0.0;
      }
      sh_ok = ok ? 1 : 0;
      sh_alpha = ok ? st->rz / pap : 0.0;
    }
  }
  __syncthreads();
  *alpha = sh_alpha;
  return sh_ok != 0;
}

// kernel A: Ap = A p and per-block partials of p.Ap; p has been updated in
// place by the p-update kernel beforehand.  (Forming p = z + beta p_old on the
// fly for every gathered column saves that launch but needs two gathers per
// entry: measured on the P2 64^3 system, 57.6 M nonzeros in FP32, 95 us per
// SpMV against 79 us, the p update taking a few microseconds; in FP64 the
// second FMA per entry would also cost FP64 issue slots.)
template <typename T, int FMT>
__global__ void __launch_bounds__(1024, 1) sell_pcg_spmv(SellView A, const T* __restrict__ val,
                                                              const T* __restrict__ p, T* __restrict__ Ap,
                                                              double* bpart, const SellPcgState* st) {
  // per-block combination of the warps' p.Ap without a block barrier at the
  // end: the last warp of the block to arrive adds the warps' slots in order
  __shared__ double wslot[32];
  __shared__ unsigned int arrivals;
  if (threadIdx.x == 0) arrivals = 0u;
  __syncthreads();
  if (st->done) return;
  // p.Ap partials in T per thread and warp (FP32 in the FP32 iterations: FP64
  // arithmetic runs at a small fraction of the FP32 rate on this part), FP64
  // from the warp sums on
  T pap = T(0);
  SELL_WARP_LOOP(A) {
    const T acc = slice_row<FMT, T, T>(A, val, s, lane, GatherX<T>{p});
    const int32_t row = A.perm[s * kSellC + lane];
    if (row >= 0) {
      Ap[row] = acc;
      pap += p[row] * acc;
    }
  }
  pap = warp_sum(pap);
  if (lane == 0) {
    const unsigned int nw = blockDim.x >> 5;
    wslot[threadIdx.x >> 5] = static_cast<double>(pap);
    __threadfence_block();
    if (atomicAdd(&arrivals, 1u) == nw - 1) {
      __threadfence_block();
      const volatile double* ws = wslot;
      double t = 0.0;
      for (unsigned int k = 0; k < nw; ++k) t += ws[k];
      bpart[blockIdx.x] = t;
    }
  }
}

// ------------------------------------------------ pipelined FP32 SpMV (15-bit steps)
// A warp of the one-trip-at-a-time SpMV alternates between waiting for a
// trip's matrix packs and waiting for that trip's gathers; while it gathers,
// none of its matrix loads are in flight, and with the bytes in flight per SM
// capped by the register file, HBM sees each SM's loads only part of the
// time.  This kernel keeps one trip (four packs) in registers and issues the
// next trip's loads, from the same slice or the first trip of the warp's next
// slice (whose bounds, slot map and first columns are loaded one slice
// ahead), before it decodes and gathers the current one.  Every row is summed
// in the same order as slice_row.  Launched as one wave of three 256-thread
// blocks per SM (measured on the P2 64^3 system, 59.7 M stored entries:
// 71.8 us per SpMV against 78-80 us; two-pack trips at four blocks per SM
// 72.0 us, six-pack trips at two blocks 83.5 us, variants held to fewer
// registers spill and run at 84-123 us).
constexpr int kPipeU = 4;
constexpr int kPipeThreads = 256;
constexpr int kPipeBlocksPerSM = 3;

struct PipeMeta {
  int64_t lo;
  int nq;  // packs per row
  int32_t row, c0;
};

__device__ __forceinline__ PipeMeta pipe_meta(const SellView& A, int64_t s, int lane) {
  PipeMeta m{0, 0, -1, 0};
  if (s < A.n_slices) {
    const int64_t lo = A.slice_ptr[s], hi = A.slice_ptr[s + 1];
    m.lo = lo;
    m.nq = static_cast<int>((hi - lo) >> 7);  // entries / (32 rows x 4 per pack)
    m.row = A.perm[s * kSellC + lane];
    m.c0 = A.col0[s * kSellC + lane];
  }
  return m;
}

__device__ __forceinline__ void pipe_load(const uint16_t* __restrict__ d16, const float* __restrict__ val,
                                          int64_t sbase, int q0, int nq, int lane, Pack4FH (&a)[kPipeU]) {
#pragma unroll
  for (int u = 0; u < kPipeU; ++u) {
    if (q0 + u < nq) a[u] = load_pack_d16(d16, val, sbase, lane, q0 + u);
    else a[u] = Pack4FH{};
  }
}

// Row epilogues: the PCG product (Ap and the p.Ap partial), a plain product,
// and a smoother sweep (as sell_smooth_kernel).
struct PipePcg {
  static constexpr bool kPap = true;
  const float* __restrict__ p;
  float* __restrict__ Ap;
  __device__ __forceinline__ void row(int32_t r, float acc, float& pap) const {
    Ap[r] = acc;
    pap += p[r] * acc;
  }
};
struct PipePlain {
  static constexpr bool kPap = false;
  float* __restrict__ y;
  __device__ __forceinline__ void row(int32_t r, float acc, float&) const { y[r] = acc; }
};
struct PipeSmooth {
  static constexpr bool kPap = false;
  const float* __restrict__ dinv;
  const float* __restrict__ rhs;
  const float* __restrict__ x_in;
  float* __restrict__ x_out;
  float* __restrict__ d;
  float c1, c2;
  int mode;
  __device__ __forceinline__ void row(int32_t r, float acc, float&) const {
    const float res = rhs[r] - acc;
    if (mode) {
      x_out[r] = res;
    } else {
      const float di = (c1 != 0.0f ? c1 * d[r] : 0.0f) + c2 * dinv[r] * res;
      d[r] = di;
      x_out[r] = x_in[r] + di;
    }
  }
};

// x: the gathered vector; bpart/st only for the PCG epilogue (st->done ends
// the launch at once, as in sell_pcg_spmv)
template <typename Epi>
__global__ void __launch_bounds__(kPipeThreads, kPipeBlocksPerSM) sell_d15_pipe(SellView A,
                                                                              const float* __restrict__ val,
                                                                              const float* __restrict__ x, Epi epi,
                                                                              double* bpart,
                                                                              const SellPcgState* st) {
  __shared__ double wslot[32];
  __shared__ unsigned int arrivals;
  if constexpr (Epi::kPap) {
    if (threadIdx.x == 0) arrivals = 0u;
    __syncthreads();
    if (st->done) return;
  }
  const int lane = threadIdx.x & 31;
  const int64_t warp0 = (blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x) >> 5;
  const int64_t nwarps = (static_cast<int64_t>(gridDim.x) * blockDim.x) >> 5;
  const GatherX<float> g{x};
  float pap = 0.0f;
  int64_t s = warp0;
  PipeMeta cur = pipe_meta(A, s, lane);
  PipeMeta nxt = pipe_meta(A, s + nwarps, lane);
  Pack4FH a[kPipeU];
  pipe_load(A.col16, val, cur.lo, 0, cur.nq, lane, a);
  int q = 0;
  float acc = 0.0f;
  int32_t c = cur.c0;
  while (s < A.n_slices) {
    const bool same = q + kPipeU < cur.nq;
    Pack4FH b[kPipeU];
    if (same) pipe_load(A.col16, val, cur.lo, q + kPipeU, cur.nq, lane, b);
    else pipe_load(A.col16, val, nxt.lo, 0, nxt.nq, lane, b);  // nq = 0 past the last slice: no loads
    int4 cc[kPipeU];
    int32_t tot[kPipeU];
#pragma unroll
    for (int u = 0; u < kPipeU; ++u) cc[u] = pack_cols_d15(a[u].d, 0, tot[u]);
    int32_t base = c;
#pragma unroll
    for (int u = 0; u < kPipeU; ++u) {
      const int4 k = make_int4(cc[u].x + base, cc[u].y + base, cc[u].z + base, cc[u].w + base);
      if (q + u < cur.nq) acc = pack_dot_cols<float>(a[u], k, g, acc);
      base += tot[u];
    }
    c = base;
    if (same) {
      q += kPipeU;
    } else {
      if (cur.row >= 0) epi.row(cur.row, acc, pap);
      s += nwarps;
      q = 0;
      acc = 0.0f;
      cur = nxt;
      c = cur.c0;
      nxt = pipe_meta(A, s + nwarps, lane);
    }
#pragma unroll
    for (int u = 0; u < kPipeU; ++u) a[u] = b[u];
  }
  if constexpr (Epi::kPap) {
    pap = warp_sum(pap);
    if (lane == 0) {
      const unsigned int nw = blockDim.x >> 5;
      wslot[threadIdx.x >> 5] = static_cast<double>(pap);
      __threadfence_block();
      if (atomicAdd(&arrivals, 1u) == nw - 1) {
        __threadfence_block();
        const volatile double* ws = wslot;
        double t = 0.0;
        for (unsigned int k = 0; k < nw; ++k) t += ws[k];
        bpart[blockIdx.x] = t;
      }
    }
  }
}

// the pipelined kernel serves FP32 products of 15-bit-step copies unless the
// process-wide switch (fgb_sell_set_pipeline) selects the one-trip kernels
int g_sell_pipe = 1;

inline bool use_pipe(const SellView& A) { return g_sell_pipe && A.col16 && A.d15 && !A.node_triples; }

// blocks of one wave (the PCG epilogue writes one p.Ap partial per block)
template <typename Epi>
int pipe_grid() {
  // computed once per process (thread-safe static initialisation: the
  // serving loop and the multigrid lanes call the solvers from several threads)
  static const int grid = [] {
    int dev = 0, sms = kNumSMs, per_sm = 0;
    if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, sell_d15_pipe<Epi>, kPipeThreads, 0) != cudaSuccess ||
        per_sm < 1)
      per_sm = 1;
    const int gr = per_sm * sms;
    return gr < kSellMaxBlocks ? gr : kSellMaxBlocks;
  }();
  return grid;
}

// One wave at most, and at least two slices per warp: a small matrix (a
// multigrid level, a system solved beside others on its own stream) leaves
// the rest of the GPU to concurrent work.
template <typename Epi>
int pipe_launch(const SellView& A, const float* val, const float* x, const Epi& epi, double* bpart,
                const SellPcgState* st, cudaStream_t s) {
  constexpr int64_t kSlicesPerBlock = 2 * (kPipeThreads / 32);
  const int64_t want = (A.n_slices + kSlicesPerBlock - 1) / kSlicesPerBlock;
  const int wave = pipe_grid<Epi>();
  const int grid = static_cast<int>(want < 1 ? 1 : (want < wave ? want : wave));
  sell_d15_pipe<Epi><<<grid, kPipeThreads, 0, s>>>(A, val, x, epi, bpart, st);
  return grid;
}

// ||b|| (mixed solver set-up); marks a zero right-hand side
__global__ void __launch_bounds__(1024, 1) sell_bnorm(int64_t n, const double* __restrict__ b, double* partials,
                                                           SellPcgState* st) {
  double bb = 0.0;
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x)
    bb += b[i] * b[i];
  double tbb, unused;
  if (sell_last_block(bb, 0.0, partials, &st->counter[0], &tbb, &unused) && threadIdx.x == 0) {
    st->b_norm = sqrt(tbb);
    st->niter = 0;
    st->n_updates = 0;
    st->need_update = 0;
    if (st->b_norm < 1e-15) st->done = FGB_PCG_ZERO_RHS;
  }
}

// p = z + beta p, in place (FP64 solver, before kernel A); 16-byte accesses
// when both vectors are 16-byte aligned, the odd last row by thread 0
__global__ void __launch_bounds__(1024, 1) sell_p_update(int64_t n, const double* __restrict__ z,
                                                              double* __restrict__ p, const SellPcgState* st) {
  if (st->done) return;
  const double beta = st->beta;
  const int64_t tid = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  const int64_t n2 = aligned16(z, p) ? n >> 1 : 0;
  const double2* Z = reinterpret_cast<const double2*>(z);
  double2* P = reinterpret_cast<double2*>(p);
  for (int64_t g = tid; g < n2; g += stride) {
    const double2 zv = Z[g];
    double2 pv = P[g];
    pv.x = zv.x + beta * pv.x;
    pv.y = zv.y + beta * pv.y;
    P[g] = pv;
  }
  for (int64_t i = 2 * n2 + tid; i < n; i += stride) p[i] = z[i] + beta * p[i];
}

// p = z + beta p, in place (mixed solver, before kernel A); four rows per
// thread and trip (16-byte accesses) when both vectors are 16-byte aligned
__global__ void __launch_bounds__(1024, 1) sell_p_update_f32(int64_t n, const float* __restrict__ z,
                                                                  float* __restrict__ p, const SellPcgState* st) {
  if (st->done) return;
  const float beta = static_cast<float>(st->beta);
  const int64_t tid = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  const int64_t n4 = aligned16(z, p) ? n >> 2 : 0;
  const float4* Z = reinterpret_cast<const float4*>(z);
  float4* P = reinterpret_cast<float4*>(p);
  for (int64_t g = tid; g < n4; g += stride) {
    const float4 zv = Z[g];
    float4 pv = P[g];
    pv.x = zv.x + beta * pv.x;
    pv.y = zv.y + beta * pv.y;
    pv.z = zv.z + beta * pv.z;
    pv.w = zv.w + beta * pv.w;
    P[g] = pv;
  }
  for (int64_t i = 4 * n4 + tid; i < n; i += stride) p[i] = z[i] + beta * p[i];
}

// kernel B (FP64 solver).  Rows in pairs (16-byte accesses) when every vector
// is 16-byte aligned; the first trip's loads are issued before alpha is known
// (its sum over the SpMV partials ends in a block barrier).
__global__ void __launch_bounds__(1024, 1) sell_pcg_update_f64(int64_t n, const double* __restrict__ dinv,
                                                                    const double* __restrict__ p,
                                                                    const double* __restrict__ Ap,
                                                                    double* __restrict__ x, double* __restrict__ r,
                                                                    double* __restrict__ z, const double* bpart,
                                                                    int nwp, double* partials, SellPcgState* st) {
  const int64_t tid = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  const bool vec = aligned16(p, Ap) && aligned16(x, r) && aligned16(z, dinv ? dinv : z);
  const int64_t n2 = vec ? n >> 1 : 0;
  const double2* P = reinterpret_cast<const double2*>(p);
  const double2* AP = reinterpret_cast<const double2*>(Ap);
  double2* X = reinterpret_cast<double2*>(x);
  double2* R = reinterpret_cast<double2*>(r);
  double2* Z = reinterpret_cast<double2*>(z);
  const double2* D = reinterpret_cast<const double2*>(dinv);
  int64_t g = tid;
  double2 pv, av, xv, rv, dv = make_double2(1.0, 1.0);
  auto load = [&](int64_t gg) {
    pv = P[gg]; av = AP[gg]; xv = X[gg]; rv = R[gg];
    if (dinv) dv = __ldg(D + gg);
  };
  if (g < n2) load(g);
  double alpha;
  if (!block_alpha(bpart, nwp, st, &alpha)) return;
  double rz = 0.0, rr = 0.0;
  while (g < n2) {
    xv.x += alpha * pv.x;
    xv.y += alpha * pv.y;
    rv.x -= alpha * av.x;
    rv.y -= alpha * av.y;
    const double2 zv = make_double2(dv.x * rv.x, dv.y * rv.y);
    X[g] = xv;
    R[g] = rv;
    Z[g] = zv;
    rz += rv.x * zv.x + rv.y * zv.y;
    rr += rv.x * rv.x + rv.y * rv.y;
    g += stride;
    if (g < n2) load(g);
  }
  for (int64_t i = 2 * n2 + tid; i < n; i += stride) {
    x[i] += alpha * p[i];
    const double ri = r[i] - alpha * Ap[i];
    const double zi = dinv ? dinv[i] * ri : ri;
    r[i] = ri;
    z[i] = zi;
    rz += ri * zi;
    rr += ri * ri;
  }
  double trz, trr;
  if (sell_last_block(rz, rr, partials, &st->counter[2], &trz, &trr) && threadIdx.x == 0) {
    st->niter += 1;
    const double res = st->norm_rr ? sqrt(trr) : sqrt(trz);
    st->resid = res;
    st->rr = trr;
    if (!isfinite(res)) st->done = FGB_PCG_NONFINITE;
    else if (res < st->atol) st->done = FGB_PCG_ATOL;
    else if (res < st->tol) st->done = FGB_PCG_RTOL;
    else if (st->niter >= st->maxit) st->done = FGB_PCG_MAXIT;
    st->rz_prev = st->rz;
    st->beta = trz / st->rz;
    st->rz = trz;
  }
}

// kernel B (mixed solver): y += alpha p, r -= alpha Ap and z = Dinv r in FP32;
// decides whether a reliable update is due.  y is the FP32 correction to the
// FP64 iterate x accumulated since the last reliable update (x_true = x + y;
// it is folded into x before each reliable update and at the end), so the
// loop streams no FP64 vector.  Per-thread dot partials are FP32 (a thread
// sums about n / (blocks * threads) terms); blocks and the grid add in FP64.
__global__ void __launch_bounds__(1024, 1) sell_mixed_update(int64_t n, const float* __restrict__ dinv,
                                                                  const float* __restrict__ p,
                                                                  const float* __restrict__ Ap, float* __restrict__ y,
                                                                  float* __restrict__ r, float* __restrict__ z,
                                                                  const double* bpart, int nwp, double* partials,
                                                                  SellPcgState* st, double delta,
                                                                  cudaGraphConditionalHandle hif, int set_if) {
  const int64_t tid = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  const bool vec = aligned16(p, Ap) && aligned16(y, r) && aligned16(z, dinv);
  const int64_t n4 = vec ? n >> 2 : 0;
  const float4* P = reinterpret_cast<const float4*>(p);
  const float4* AP = reinterpret_cast<const float4*>(Ap);
  float4* Y = reinterpret_cast<float4*>(y);
  float4* R = reinterpret_cast<float4*>(r);
  float4* Z = reinterpret_cast<float4*>(z);
  const float4* D = reinterpret_cast<const float4*>(dinv);
  // rows in fours (16-byte accesses); the first trip's loads are issued
  // before alpha is known (its sum over the SpMV partials ends in a block
  // barrier)
  int64_t g = tid;
  float4 pv, av, yv, rv, dv;
  auto load = [&](int64_t gg) {
    pv = P[gg]; av = AP[gg]; yv = Y[gg]; rv = R[gg]; dv = __ldg(D + gg);
  };
  if (g < n4) load(g);
  double alpha;
  if (!block_alpha(bpart, nwp, st, &alpha)) return;
  const float alpha32 = static_cast<float>(alpha);
  float rz = 0.0f, rr = 0.0f;
  while (g < n4) {
    yv.x += alpha32 * pv.x; yv.y += alpha32 * pv.y; yv.z += alpha32 * pv.z; yv.w += alpha32 * pv.w;
    rv.x -= alpha32 * av.x; rv.y -= alpha32 * av.y; rv.z -= alpha32 * av.z; rv.w -= alpha32 * av.w;
    const float4 zv = make_float4(dv.x * rv.x, dv.y * rv.y, dv.z * rv.z, dv.w * rv.w);
    Y[g] = yv;
    R[g] = rv;
    Z[g] = zv;
    rz += (rv.x * zv.x + rv.y * zv.y) + (rv.z * zv.z + rv.w * zv.w);
    rr += (rv.x * rv.x + rv.y * rv.y) + (rv.z * rv.z + rv.w * rv.w);
    g += stride;
    if (g < n4) load(g);
  }
  for (int64_t i = 4 * n4 + tid; i < n; i += stride) {
    y[i] += alpha32 * p[i];
    const float ri = r[i] - alpha32 * Ap[i];
    const float zi = dinv[i] * ri;
    r[i] = ri;
    z[i] = zi;
    rz += ri * zi;
    rr += ri * ri;
  }
  double trz, trr;
  if (sell_last_block(rz, rr, partials, &st->counter[2], &trz, &trr) &&
      threadIdx.x == 0) {
    mixed_iteration_scalars(*st, trz, trr, delta);
    // graph driver: run the reliable-update node only when it is due
    if (set_if) cudaGraphSetConditional(hif, (st->need_update && !st->done) ? 1u : 0u);
  }
}

// x += y ; y = 0 (mixed solver): before a reliable update when one is due, and
// unconditionally (force = 1) when the solve ends.
__global__ void __launch_bounds__(1024, 1) sell_mixed_fold(int64_t n, double* __restrict__ x, float* __restrict__ y,
                                                        const SellPcgState* st, int force) {
  if (!force && (st->done || !st->need_update)) return;
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    x[i] += static_cast<double>(y[i]);
    y[i] = 0.0f;
  }
}

// Reliable update (only when due, or first = 1 at the start): r64 = b - A x in
// FP64 arithmetic (V = double: the FP64 values; V = float: the values of an
// FP32-assembled matrix, the operator the solve is for), true residual test,
// then r = float(r64), z = Dinv r and beta from the replaced residual.  The
// first call also builds the FP32 inverse diagonal and starts p = z.
template <typename V, int FMT>
__global__ void __launch_bounds__(1024, 1) sell_mixed_reliable(SellView A, const V* __restrict__ val,
                                                                    const double* __restrict__ b,
                                                                    const double* __restrict__ x,
                                                                    const double* __restrict__ dinv64,
                                                                    float* __restrict__ dinv32, float* __restrict__ r,
                                                                    float* __restrict__ z, float* __restrict__ p,
                                                                    double* partials, SellPcgState* st, int first) {
  if (!first && (st->done || !st->need_update)) return;
  double rr64 = 0.0, rz = 0.0;
  SELL_WARP_LOOP(A) {
    const double acc = slice_row<FMT, V, double>(A, val, s, lane, GatherX<double>{x});
    const int32_t row = A.perm[s * kSellC + lane];
    if (row >= 0) {
      const double r64 = b[row] - acc;
      rr64 += r64 * r64;
      const float di = first ? static_cast<float>(dinv64[row]) : dinv32[row];
      if (first) dinv32[row] = di;
      const float ri = static_cast<float>(r64);
      const float zi = di * ri;
      r[row] = ri;
      z[row] = zi;
      if (first) p[row] = zi;
      rz += static_cast<double>(ri) * static_cast<double>(zi);
    }
  }
  double trr, trz;
  if (sell_last_block(rr64, rz, partials, &st->counter[3], &trr, &trz) && threadIdx.x == 0)
    mixed_reliable_scalars(*st, trr, trz, first);
}

// ------------------------------------------------ persistent FP32-refined solver
// One cooperative launch runs every iteration of the mixed solver: the grid
// stays resident (two 512-thread blocks per SM) and phases are separated by a
// software grid barrier instead of kernel boundaries, which removes the launch,
// ramp-up and tail of three kernels per iteration (the vector kernels are
// launch-bound: their SMs are busy for less than half of their duration).
// Per iteration: p = z + beta p (own rows) | barrier | Ap = A p, block partial
// of p.Ap | barrier | alpha (every block sums the partials in the same order)
// and y, r, z updates, block partials of r.z, r.r | barrier | beta, the
// stopping test and whether a reliable update is due (every block computes the
// same scalars from the same partials; the scalar code is the one of the
// multi-kernel driver).  A reliable update adds: x += y | barrier | r64 = b -
// A x in FP64 arithmetic, r, z | barrier | true-residual test.
// Vectors rewritten by other blocks inside the kernel are read through L2
// (ld.global.cg): L1 is not coherent across blocks within a launch.
constexpr int kPersistThreads = 512;
constexpr long long kBarrierSpins = 20000000;  // >= 64 ns apart: well above a second

struct PersistArgs {
  SellView A;
  const float* val32;  // FP32 values (the iterations)
  const void* valr;    // values of the FP64 residual: double, or the FP32 ones
  const double* b;
  double* x;
  const float* dinv;
  float *r, *z, *p, *Ap, *y;
  double* bpart;  // kSellMaxBlocks partials of p.Ap
  double* vpart;  // 2 * kSellMaxBlocks partials (two values per block)
  SellPcgState* st;
  double delta;
  long long bar_limit;  // polls before a grid barrier gives up (kBarrierSpins by default)
};

// Grid barrier of a cooperative launch (every block resident): arrivals by an
// atomic counter, release by a generation counter.  A wait longer than
// `limit` polls, or any wait once another block has failed, sets the error
// flag and returns false; the caller then returns, so every block ends.
__device__ bool grid_barrier(SellPcgState* st, long long limit) {
  __shared__ int ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    volatile unsigned int* gen = &st->bar[1];
    volatile int* err = &st->bar_err;
    const unsigned int g = *gen;
    __threadfence();
    int good = 1;
    if (atomicAdd(&st->bar[0], 1u) == gridDim.x - 1) {
      atomicExch(&st->bar[0], 0u);
      __threadfence();
      atomicAdd(&st->bar[1], 1u);
    } else {
      long long spins = 0;
      while (*gen == g) {
        if (*err || ++spins > limit) {
          good = 0;
          atomicExch(&st->bar_err, 1);
          break;
        }
        __nanosleep(64);
      }
    }
    __threadfence();
    ok = good && !*err;
  }
  __syncthreads();
  return ok != 0;
}

// Block sums of two per-thread values (T: float or double; warp shuffles in T,
// the warps' sums added in FP64 in order by warp 0), written by thread 0 to
// part0[blockIdx.x] and (if part1) part1[blockIdx.x].
template <typename T>
__device__ void block_partials2(T v0, T v1, double* part0, double* part1) {
  __shared__ double2 ws[32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  v0 = warp_sum(v0);
  v1 = warp_sum(v1);
  __syncthreads();
  if (lane == 0) ws[wid] = make_double2(static_cast<double>(v0), static_cast<double>(v1));
  __syncthreads();
  if (wid == 0) {
    const int nw = (blockDim.x + 31) >> 5;
    double2 t = lane < nw ? ws[lane] : make_double2(0.0, 0.0);
    t.x = warp_sum(t.x);
    t.y = warp_sum(t.y);
    if (lane == 0) {
      part0[blockIdx.x] = t.x;
      if (part1) part1[blockIdx.x] = t.y;
    }
  }
}

// Sums of the grid's partials (after a barrier), the same in every block:
// warp 0 loads them through L2 in one unrolled round trip per 320 blocks and
// adds them in block order; the result is handed to the block in shared memory.
__device__ double2 grid_totals2(const double* part0, const double* part1, int nb) {
  __shared__ double2 res;
  constexpr int kPer = 10;
  if (threadIdx.x < 32) {
    const int lane = threadIdx.x;
    double a = 0.0, b = 0.0;
    for (int base = 0; base < nb; base += 32 * kPer) {
      double pa[kPer], pb[kPer];
#pragma unroll
      for (int u = 0; u < kPer; ++u) {
        const int k = base + lane + 32 * u;
        pa[u] = k < nb ? __ldcg(part0 + k) : 0.0;
        pb[u] = (part1 && k < nb) ? __ldcg(part1 + k) : 0.0;
      }
#pragma unroll
      for (int u = 0; u < kPer; ++u) {
        a += pa[u];
        b += pb[u];
      }
    }
    a = warp_sum(a);
    b = warp_sum(b);
    if (lane == 0) res = make_double2(a, b);
  }
  __syncthreads();
  return res;
}

template <int FMT, typename V>
__global__ void __launch_bounds__(kPersistThreads, 2) sell_mixed_persistent(PersistArgs P) {
  __shared__ SellPcgState S;
  if (threadIdx.x == 0) S = *P.st;
  __syncthreads();
  const SellView& A = P.A;
  const int64_t n = A.n;
  const int lane = threadIdx.x & 31;
  const int64_t tid = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  const int64_t warp0 = tid >> 5, nwarps = stride >> 5;
  const bool vec = aligned16(P.p, P.Ap) && aligned16(P.y, P.r) && aligned16(P.z, P.dinv);
  const int64_t n4 = vec ? n >> 2 : 0;
  float4* P4 = reinterpret_cast<float4*>(P.p);
  const float4* AP4 = reinterpret_cast<const float4*>(P.Ap);
  float4* Y4 = reinterpret_cast<float4*>(P.y);
  float4* R4 = reinterpret_cast<float4*>(P.r);
  float4* Z4 = reinterpret_cast<float4*>(P.z);
  const float4* D4 = reinterpret_cast<const float4*>(P.dinv);
  const long long cap = S.maxit + 16;
  while (!S.done) {
    // p = z + beta p
    {
      const float beta = static_cast<float>(S.beta);
      for (int64_t g = tid; g < n4; g += stride) {
        const float4 zv = __ldcg(Z4 + g);
        float4 pv = __ldcg(P4 + g);
        pv.x = zv.x + beta * pv.x;
        pv.y = zv.y + beta * pv.y;
        pv.z = zv.z + beta * pv.z;
        pv.w = zv.w + beta * pv.w;
        P4[g] = pv;
      }
      for (int64_t i = 4 * n4 + tid; i < n; i += stride) P.p[i] = __ldcg(P.z + i) + beta * __ldcg(P.p + i);
    }
    if (!grid_barrier(P.st, P.bar_limit)) return;
    // Ap = A p and p.Ap
    {
      float pap = 0.0f;
      const GatherCG<float> gp{P.p};
      for (int64_t s = warp0; s < A.n_slices; s += nwarps) {
        const float acc = slice_row<FMT, float, float>(A, P.val32, s, lane, gp);
        const int32_t row = A.perm[s * kSellC + lane];
        if (row >= 0) {
          P.Ap[row] = acc;
          pap += __ldcg(P.p + row) * acc;
        }
      }
      block_partials2(pap, 0.0f, P.bpart, nullptr);
    }
    if (!grid_barrier(P.st, P.bar_limit)) return;
    // alpha; y += alpha p, r -= alpha Ap, z = Dinv r; r.z, r.r
    {
      const double pap = grid_totals2(P.bpart, nullptr, gridDim.x).x;
      const bool ok = pap > 0.0 && isfinite(pap);
      if (!ok) {
        if (threadIdx.x == 0) {
          S.done = isfinite(pap) ? FGB_PCG_BREAKDOWN : FGB_PCG_NONFINITE;
          S.alpha = 0.0;
        }
        __syncthreads();
        break;
      }
      const double alpha = S.rz / pap;
      const float a32 = static_cast<float>(alpha);
      float rz = 0.0f, rr = 0.0f;
      for (int64_t g = tid; g < n4; g += stride) {
        const float4 pv = __ldcg(P4 + g), av = __ldcg(AP4 + g), dv = __ldg(D4 + g);
        float4 yv = __ldcg(Y4 + g), rv = __ldcg(R4 + g);
        yv.x += a32 * pv.x; yv.y += a32 * pv.y; yv.z += a32 * pv.z; yv.w += a32 * pv.w;
        rv.x -= a32 * av.x; rv.y -= a32 * av.y; rv.z -= a32 * av.z; rv.w -= a32 * av.w;
        const float4 zv = make_float4(dv.x * rv.x, dv.y * rv.y, dv.z * rv.z, dv.w * rv.w);
        Y4[g] = yv;
        R4[g] = rv;
        Z4[g] = zv;
        rz += (rv.x * zv.x + rv.y * zv.y) + (rv.z * zv.z + rv.w * zv.w);
        rr += (rv.x * rv.x + rv.y * rv.y) + (rv.z * rv.z + rv.w * rv.w);
      }
      for (int64_t i = 4 * n4 + tid; i < n; i += stride) {
        P.y[i] += a32 * __ldcg(P.p + i);
        const float ri = __ldcg(P.r + i) - a32 * __ldcg(P.Ap + i);
        const float zi = P.dinv[i] * ri;
        P.r[i] = ri;
        P.z[i] = zi;
        rz += ri * zi;
        rr += ri * ri;
      }
      if (threadIdx.x == 0) S.alpha = alpha;
      block_partials2(rz, rr, P.vpart, P.vpart + kSellMaxBlocks);
    }
    if (!grid_barrier(P.st, P.bar_limit)) return;
    {
      const double2 t = grid_totals2(P.vpart, P.vpart + kSellMaxBlocks, gridDim.x);
      if (threadIdx.x == 0) {
        mixed_iteration_scalars(S, t.x, t.y, P.delta);
        if (S.niter >= cap && !S.done) S.done = FGB_PCG_MAXIT;
      }
      __syncthreads();
    }
    if (S.done || !S.need_update) continue;
    // reliable update: x += y, y = 0 | r64 = b - A x, r, z | test
    for (int64_t i = tid; i < n; i += stride) {
      P.x[i] += static_cast<double>(__ldcg(P.y + i));
      P.y[i] = 0.0f;
    }
    if (!grid_barrier(P.st, P.bar_limit)) return;
    {
      double rr64 = 0.0, rz = 0.0;
      const GatherCG<double> gx{P.x};
      const V* valr = static_cast<const V*>(P.valr);
      for (int64_t s = warp0; s < A.n_slices; s += nwarps) {
        const double acc = slice_row<FMT, V, double>(A, valr, s, lane, gx);
        const int32_t row = A.perm[s * kSellC + lane];
        if (row >= 0) {
          const double r64 = P.b[row] - acc;
          rr64 += r64 * r64;
          const float ri = static_cast<float>(r64);
          const float zi = P.dinv[row] * ri;
          P.r[row] = ri;
          P.z[row] = zi;
          rz += static_cast<double>(ri) * static_cast<double>(zi);
        }
      }
      block_partials2(rr64, rz, P.vpart, P.vpart + kSellMaxBlocks);
    }
    if (!grid_barrier(P.st, P.bar_limit)) return;
    {
      const double2 t = grid_totals2(P.vpart, P.vpart + kSellMaxBlocks, gridDim.x);
      if (threadIdx.x == 0) mixed_reliable_scalars(S, t.x, t.y, 0);
      __syncthreads();
    }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    // the barrier words stay as they are in global memory
    S.bar[0] = 0u;
    S.bar[1] = *reinterpret_cast<volatile unsigned int*>(&P.st->bar[1]);
    S.bar_err = *reinterpret_cast<volatile int*>(&P.st->bar_err);
    *P.st = S;
  }
}

// Loop control of the graph driver: one thread.  Clears the while condition
// when the solve is finished, and in any case after trip_cap body executions,
// so the device loop always ends.
__global__ void sell_loop_ctl(SellPcgState* st, cudaGraphConditionalHandle handle) {
  st->trips += 1;
  if (st->trips >= st->trip_cap && !st->done) st->done = FGB_PCG_MAXIT;
  if (st->done) cudaGraphSetConditional(handle, 0);
}

}  // namespace fgb

using namespace fgb;

namespace {

SellView view_of(const fgb_sell* A) {
  return SellView{A->n,   A->n_slices, A->slice_ptr, A->perm, A->col,       A->threads,
                  A->blocks, A->col16,   A->col0,      A->node_triples, A->col_long};
}

// launch shape in range, and the column arrays the storage format reads present
bool launch_ok(const fgb_sell* A) {
  const bool cols = A->col16 ? (A->col0 != nullptr && !A->node_triples) : (A->col != nullptr && !A->col_long);
  return cols && A->slice_ptr && A->perm && A->threads >= 0 && A->threads <= 1024 && A->threads % 32 == 0 &&
         A->blocks >= 0 && A->blocks <= kSellMaxBlocks;
}

// CUDA events before the SpMV, after the SpMV and after the rest of each
// iteration of a host-polled chunk; only iterations that did work (counted by
// the device iteration counter) are summed.
struct EventPairs {
  static constexpr int kPer = 5;  // body start, before SpMV, after SpMV, after update, body end
  bool on;
  int cap;
  cudaEvent_t* ev = nullptr;
  double ms = 0.0, other = 0.0, extra = 0.0;
  int64_t launches = 0;
  EventPairs(bool enable, int c) : on(enable), cap(c) {
    if (!on) return;
    ev = new cudaEvent_t[kPer * cap];
    for (int k = 0; k < kPer * cap; ++k) cudaEventCreate(&ev[k]);
  }
  ~EventPairs() {
    if (!ev) return;
    for (int k = 0; k < kPer * cap; ++k) cudaEventDestroy(ev[k]);
    delete[] ev;
  }
  const cudaEvent_t* of(int k) const { return on ? ev + kPer * k : nullptr; }
  // spmv = t2 - t1, update = t3 - t2, extra = (t1 - t0) + (t4 - t3)
  void collect(int64_t executed) {
    if (!on) return;
    for (int64_t k = 0; k < executed && k < cap; ++k) {
      float d[4];
      bool ok = true;
      for (int j = 0; j < 4; ++j) ok = ok && cudaEventElapsedTime(&d[j], ev[kPer * k + j], ev[kPer * k + j + 1]) == cudaSuccess;
      if (ok) {
        ms += d[1];
        other += d[2];
        extra += d[0] + d[3];
        ++launches;
      }
    }
  }
};

inline void rec(const cudaEvent_t* e, int j, cudaStream_t s) {
  if (e) cudaEventRecord(e[j], s);
}

// Capture state of the while-loop body.  new_handle() makes a condition
// handle on the body graph; add_if() appends an IF conditional node on that
// handle (set on the device by an earlier kernel of the body) whose body is
// whatever `fn` launches on the stream it is given.  Each IF node needs its
// own handle: a second conditional node on a handle is rejected.
struct CaptureCtx {
  cudaStream_t cs = nullptr;
  cudaGraph_t body = nullptr;
  bool ok = true;

  cudaGraphConditionalHandle new_handle() {
    cudaGraphConditionalHandle h = 0;
    if (cudaGraphConditionalHandleCreate(&h, body, 0, cudaGraphCondAssignDefault) != cudaSuccess) ok = false;
    return h;
  }

  template <typename Fn>
  void add_if(cudaGraphConditionalHandle hif, Fn fn) {
    if (!ok) return;
    cudaStreamCaptureStatus status;
    cudaGraph_t g = nullptr;
    const cudaGraphNode_t* deps = nullptr;
    size_t nd = 0;
    if (cudaStreamGetCaptureInfo(cs, &status, nullptr, &g, &deps, nullptr, &nd) != cudaSuccess ||
        status != cudaStreamCaptureStatusActive) {
      ok = false;
      return;
    }
    cudaGraphNodeParams p = {};
    p.type = cudaGraphNodeTypeConditional;
    p.conditional.handle = hif;
    p.conditional.type = cudaGraphCondTypeIf;
    p.conditional.size = 1;
    cudaGraphNode_t node;
    if (cudaGraphAddNode(&node, g, deps, nullptr, nd, &p) != cudaSuccess) { ok = false; return; }
    if (cudaStreamUpdateCaptureDependencies(cs, &node, nullptr, 1, cudaStreamSetCaptureDependencies) != cudaSuccess) {
      ok = false;
      return;
    }
    cudaStream_t bs;
    cudaStreamCreateWithFlags(&bs, cudaStreamNonBlocking);
    if (cudaStreamBeginCaptureToGraph(bs, p.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                      cudaStreamCaptureModeRelaxed) != cudaSuccess) {
      ok = false;
    } else {
      fn(bs);
      cudaGraph_t out = nullptr;
      if (cudaStreamEndCapture(bs, &out) != cudaSuccess) ok = false;
    }
    cudaStreamDestroy(bs);
  }
};

struct F64Work {
  SellPcgState* st;
  double* partials;
  double* bpart;  // per-block p.Ap partials of the SpMV step
  double *r, *z, *p0, *Ap;
};

struct MixedWork {
  SellPcgState* st;
  double* partials;
  double* bpart;
  float *r, *z, *p0, *Ap, *dinv32, *y;
};

bool carve_f64(Carver& cv, int64_t n, F64Work& w) {
  w.st = cv.take<SellPcgState>(1);
  w.partials = cv.take<double>(2 * kSellMaxBlocks);
  w.bpart = cv.take<double>(kSellMaxBlocks);
  w.r = cv.take<double>(n); w.z = cv.take<double>(n); w.p0 = cv.take<double>(n);
  w.Ap = cv.take<double>(n);
  return cv.ok;
}

bool carve_mixed(Carver& cv, int64_t n, MixedWork& w) {
  w.st = cv.take<SellPcgState>(1);
  w.partials = cv.take<double>(2 * kSellMaxBlocks);
  w.bpart = cv.take<double>(kSellMaxBlocks);
  w.r = cv.take<float>(n); w.z = cv.take<float>(n); w.p0 = cv.take<float>(n);
  w.Ap = cv.take<float>(n); w.dinv32 = cv.take<float>(n); w.y = cv.take<float>(n);
  return cv.ok;
}

// one CG iteration (FP64): p = z + beta p in place, then Ap, then the updates
void f64_body(const SellView& A, const double* val, const double* dinv, double* x, F64Work& w, int parity,
              const cudaEvent_t* ev, cudaStream_t s) {
  (void)parity;
  rec(ev, 0, s);
  sell_p_update<<<VEC_LAUNCH(A.n, s)>>>(A.n, w.z, w.p0, w.st);
  rec(ev, 1, s);
  with_cols(A, [&](auto d16) {
    sell_pcg_spmv<double, decltype(d16)::value><<<SLICE_LAUNCH(A, s)>>>(A, val, w.p0, w.Ap, w.bpart, w.st);
  });
  rec(ev, 2, s);
  sell_pcg_update_f64<<<VEC_LAUNCH(A.n, s)>>>(A.n, dinv, w.p0, w.Ap, x, w.r, w.z, w.bpart, slice_blocks(A),
                                              w.partials, w.st);
  rec(ev, 3, s);
  rec(ev, 4, s);
}

// one CG iteration (mixed): p = z + beta p in place, then Ap, then the
// updates (p lives in w.p0; the parity argument is kept for the two-iteration
// graph body).  With a capture context the reliable update becomes an IF node
// of the graph; otherwise it is launched every iteration and returns at once
// when not due.
void mixed_body(const SellView& A, const float* val32, const double* val64, const double* dinv64, const double* b,
                double* x, MixedWork& w, double delta, int parity, const cudaEvent_t* ev, cudaStream_t s,
                CaptureCtx* ctx = nullptr) {
  (void)parity;
  float* p = w.p0;
  const cudaGraphConditionalHandle hif = ctx ? ctx->new_handle() : 0;
  rec(ev, 0, s);
  sell_p_update_f32<<<VEC_LAUNCH(A.n, s)>>>(A.n, w.z, p, w.st);
  rec(ev, 1, s);
  int nwp = slice_blocks(A);
  if (use_pipe(A)) {
    nwp = pipe_launch(A, val32, p, PipePcg{p, w.Ap}, w.bpart, w.st, s);
  } else {
    with_cols(A, [&](auto d16) {
      sell_pcg_spmv<float, decltype(d16)::value><<<SLICE_LAUNCH(A, s)>>>(A, val32, p, w.Ap, w.bpart, w.st);
    });
  }
  rec(ev, 2, s);
  sell_mixed_update<<<VEC_LAUNCH(A.n, s)>>>(A.n, w.dinv32, p, w.Ap, w.y, w.r, w.z, w.bpart, nwp,
                                            w.partials, w.st, delta, hif, ctx ? 1 : 0);
  rec(ev, 3, s);
  auto reliable = [&](cudaStream_t rs) {
    sell_mixed_fold<<<VEC_LAUNCH(A.n, rs)>>>(A.n, x, w.y, w.st, 0);
    with_cols(A, [&](auto d16) {
      constexpr int D = decltype(d16)::value;
      if (val64)
        sell_mixed_reliable<double, D><<<SLICE_LAUNCH(A, rs)>>>(A, val64, b, x, dinv64, w.dinv32, w.r, w.z,
                                                                nullptr, w.partials, w.st, 0);
      else
        sell_mixed_reliable<float, D><<<SLICE_LAUNCH(A, rs)>>>(A, val32, b, x, dinv64, w.dinv32, w.r, w.z,
                                                               nullptr, w.partials, w.st, 0);
    });
  };
  if (ctx) ctx->add_if(hif, reliable);
  else reliable(s);
  rec(ev, 4, s);
}

// Launches the persistent mixed solver as one cooperative kernel (two blocks
// per SM, as many as stay resident); false when the device cannot run it that
// way, in which case nothing was launched.
template <int FMT, typename V>
bool launch_persistent(const PersistArgs& P, cudaStream_t s) {
  auto kern = sell_mixed_persistent<FMT, V>;
  int dev = 0, coop = 0, sms = 0, per_sm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return false;
  if (cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev) != cudaSuccess || !coop) return false;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return false;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kPersistThreads, 0) != cudaSuccess ||
      per_sm < 1)
    return false;
  const int grid = sms * (per_sm < 2 ? per_sm : 2);
  if (grid > kSellMaxBlocks) return false;
  PersistArgs a = P;
  void* args[] = {&a};
  if (cudaLaunchCooperativeKernel(reinterpret_cast<const void*>(kern), dim3(grid), dim3(kPersistThreads), args, 0,
                                  s) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return true;
}

// Returns FGB_OK after the graph ran to completion.  *launched tells the caller
// whether anything was submitted: when graph construction fails before the
// launch (a feature missing in the CUDA driver), the caller falls back to the
// host-polled loop, which runs the same kernels.
template <typename Body>
int graph_loop(Body body_two_iters, SellPcgState* st, cudaStream_t s, bool* launched) {
  *launched = false;
  // Build: while(cond) { two iterations ; loop_ctl }.  Two iterations per trip
  // keep the p ping-pong parity fixed inside the body.
  cudaGraph_t g = nullptr;
  cudaGraphExec_t ge = nullptr;
  cudaGraphConditionalHandle h;
  int rc = FGB_OK;
  if (cudaGraphCreate(&g, 0) != cudaSuccess) return FGB_ERR_CUDA;
  if (cudaGraphConditionalHandleCreate(&h, g, 1, cudaGraphCondAssignDefault) != cudaSuccess) {
    cudaGraphDestroy(g);
    return FGB_ERR_CUDA;
  }
  cudaGraphNodeParams cp = {};
  cp.type = cudaGraphNodeTypeConditional;
  cp.conditional.handle = h;
  cp.conditional.type = cudaGraphCondTypeWhile;
  cp.conditional.size = 1;
  cudaGraphNode_t node;
  if (cudaGraphAddNode(&node, g, nullptr, nullptr, 0, &cp) != cudaSuccess) {
    cudaGraphDestroy(g);
    return FGB_ERR_CUDA;
  }
  cudaGraph_t body = cp.conditional.phGraph_out[0];
  CaptureCtx ctx;
  ctx.body = body;
  cudaStreamCreateWithFlags(&ctx.cs, cudaStreamNonBlocking);
  if (cudaStreamBeginCaptureToGraph(ctx.cs, body, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed) != cudaSuccess) {
    rc = FGB_ERR_CUDA;
  } else {
    body_two_iters(ctx);
    sell_loop_ctl<<<1, 1, 0, ctx.cs>>>(st, h);
    cudaGraph_t out = nullptr;
    if (cudaStreamEndCapture(ctx.cs, &out) != cudaSuccess || !ctx.ok) rc = FGB_ERR_CUDA;
  }
  cudaStream_t cs = ctx.cs;
  if (rc == FGB_OK && cudaGraphInstantiate(&ge, g, 0) != cudaSuccess) rc = FGB_ERR_CUDA;
  if (rc != FGB_OK) cudaGetLastError();  // clear a non-sticky API error before falling back
  if (rc == FGB_OK) {
    *launched = true;
    if (cudaGraphLaunch(ge, s) != cudaSuccess) rc = FGB_ERR_CUDA;
    else if (cudaStreamSynchronize(s) != cudaSuccess) rc = FGB_ERR_CUDA;
  }
  if (ge) cudaGraphExecDestroy(ge);
  cudaGraphDestroy(g);
  cudaStreamDestroy(cs);
  return rc;
}

int read_state(SellPcgState* d, SellPcgState* h, cudaStream_t s) {
  if (cudaMemcpyAsync(h, d, sizeof(SellPcgState), cudaMemcpyDeviceToHost, s) != cudaSuccess) return FGB_ERR_CUDA;
  if (cudaStreamSynchronize(s) != cudaSuccess) return FGB_ERR_CUDA;
  return FGB_OK;
}

int set_tol(SellPcgState* d, double tol, cudaStream_t s) {
  return cudaMemcpyAsync(reinterpret_cast<char*>(d) + offsetof(SellPcgState, tol), &tol, sizeof(double),
                         cudaMemcpyHostToDevice, s) == cudaSuccess ? FGB_OK : FGB_ERR_CUDA;
}

int finish(int done) {
  return done == FGB_PCG_BREAKDOWN ? FGB_ERR_BREAKDOWN : (done == FGB_PCG_NONFINITE ? FGB_ERR_NONFINITE : FGB_OK);
}

}  // namespace

namespace fgb {

// Smoother sweep on the FP32 (FP64) values of a SELL copy (used by the
// multigrid V-cycle for its large levels); the shape of the copy's launch.
int sell_smooth_f32(const fgb_sell* A, const float* dinv, const float* r, const float* x_in, float* x_out, float* d,
                    float c1, float c2, int mode, cudaStream_t st) {
  if (!A || !A->val32 || !launch_ok(A) || !r || !x_in || !x_out || (mode == 0 && (!dinv || !d))) return FGB_ERR_ARG;
  const SellView V = view_of(A);
  if (use_pipe(V)) {
    pipe_launch(V, A->val32, x_in, PipeSmooth{dinv, r, x_in, x_out, d, c1, c2, mode}, nullptr, nullptr, st);
    return FGB_OK;
  }
  with_cols(V, [&](auto f) {
    constexpr int FMT = decltype(f)::value;
    sell_smooth_kernel<FMT, float><<<SLICE_LAUNCH(V, st)>>>(V, A->val32, dinv, r, x_in, x_out, d, c1, c2, mode);
  });
  return FGB_OK;
}

int sell_smooth_f64(const fgb_sell* A, const double* dinv, const double* r, const double* x_in, double* x_out,
                    double* d, double c1, double c2, int mode, cudaStream_t st) {
  if (!A || !A->val64 || !launch_ok(A) || !r || !x_in || !x_out || (mode == 0 && (!dinv || !d))) return FGB_ERR_ARG;
  const SellView V = view_of(A);
  with_cols(V, [&](auto f) {
    constexpr int FMT = decltype(f)::value;
    sell_smooth_kernel<FMT, double><<<SLICE_LAUNCH(V, st)>>>(V, A->val64, dinv, r, x_in, x_out, d, c1, c2, mode);
  });
  return FGB_OK;
}

// Ap = A p on the FP64 values of a SELL copy; per-block p.Ap partials in
// bpart (at least kSellMaxBlocks doubles), their number in *n_part.
int sell_spmv_pap_f64(const fgb_sell* A, const double* p, double* Ap, double* bpart, int* n_part, cudaStream_t st) {
  if (!A || !A->val64 || !launch_ok(A) || !p || !Ap || !bpart || !n_part) return FGB_ERR_ARG;
  const SellView V = view_of(A);
  *n_part = slice_blocks(V);
  with_cols(V, [&](auto f) {
    constexpr int FMT = decltype(f)::value;
    sell_spmv_pap_kernel<FMT><<<SLICE_LAUNCH(V, st)>>>(V, A->val64, p, Ap, bpart);
  });
  return FGB_OK;
}

}  // namespace fgb

extern "C" {

size_t fgb_sell_workspace_bytes(int64_t n) {
  const int64_t ns = (n + kSellC - 1) / kSellC;
  return align_up(static_cast<size_t>(ns) * sizeof(int32_t)) + scan_workspace_bytes(ns);
}

int64_t fgb_sell_slots(int64_t n) {
  return ((n + kSellWindow - 1) / kSellWindow) * kSellWindow;
}

int32_t fgb_sell_plan(int64_t n, const int64_t* indptr, int32_t* perm, int64_t* slice_ptr, void* workspace,
                      size_t workspace_bytes, void* stream) {
  if (n <= 0 || !indptr || !perm || !slice_ptr) return FGB_ERR_ARG;
  if (n >= (int64_t(1) << 31)) return FGB_ERR_CAPACITY;
  if (!workspace || workspace_bytes < fgb_sell_workspace_bytes(n)) return FGB_ERR_WORKSPACE;
  cudaStream_t st = as_stream(stream);
  const int64_t windows = (n + kSellWindow - 1) / kSellWindow;
  const int64_t slices = windows * (kSellWindow / kSellC);
  Carver cv(workspace, workspace_bytes);
  int32_t* entries = cv.take<int32_t>(slices);
  void* scan_ws = cv.base + cv.off;
  size_t scan_bytes = workspace_bytes - cv.off;
  sell_sort_windows<<<static_cast<unsigned>(windows), kSellWindow, 0, st>>>(n, indptr, perm, entries);
  return exclusive_scan_i32_to_i64(entries, slices, slice_ptr, scan_ws, scan_bytes, st);
}

int32_t fgb_sell_fill(int64_t n, const int64_t* indptr, const int32_t* indices, const double* values64,
                      const float* values32, const int32_t* perm, const int64_t* slice_ptr, int32_t* col,
                      double* val64, float* val32, void* stream) {
  if (n <= 0 || !indptr || !indices || !perm || !slice_ptr || !col) return FGB_ERR_ARG;
  if ((val64 && !values64) || (val32 && !values64 && !values32)) return FGB_ERR_ARG;
  const int64_t slices = fgb_sell_slots(n) / kSellC;
  sell_fill_kernel<<<grid_for(slices * 32, 256, kNumSMs * 16), 256, 0, as_stream(stream)>>>(
      slices, slice_ptr, perm, indptr, indices, values64, values32, col, val64, val32);
  return launch_status();
}

int32_t fgb_sell_spmv(int32_t dtype, const fgb_sell* A, const void* x, void* y, void* stream) {
  if (!A || !x || !y || A->n <= 0 || !launch_ok(A)) return FGB_ERR_ARG;
  SellView v = view_of(A);
  cudaStream_t st = as_stream(stream);
  if (dtype == FGB_F64) {
    if (!A->val64) return FGB_ERR_ARG;
    with_cols(v, [&](auto d16) {
      sell_spmv_kernel<double, decltype(d16)::value>
          <<<SLICE_LAUNCH(v, st)>>>(v, A->val64, static_cast<const double*>(x), static_cast<double*>(y));
    });
  } else if (dtype == FGB_F32) {
    if (!A->val32) return FGB_ERR_ARG;
    if (use_pipe(v)) {
      pipe_launch(v, A->val32, static_cast<const float*>(x), PipePlain{static_cast<float*>(y)}, nullptr, nullptr, st);
    } else {
      with_cols(v, [&](auto d16) {
        sell_spmv_kernel<float, decltype(d16)::value>
            <<<SLICE_LAUNCH(v, st)>>>(v, A->val32, static_cast<const float*>(x), static_cast<float*>(y));
      });
    }
  } else {
    return FGB_ERR_ARG;
  }
  return launch_status();
}

size_t fgb_pcg_sell_workspace_bytes(int64_t n) {
  // sized for the larger (mixed) layout
  return align_up(sizeof(SellPcgState)) + align_up(2 * kSellMaxBlocks * sizeof(double)) +
         align_up(kSellMaxBlocks * sizeof(double)) + 4 * align_up(static_cast<size_t>(n) * sizeof(double)) +
         6 * align_up(static_cast<size_t>(n) * sizeof(float));
}

int32_t fgb_pcg_sell_f64(const fgb_sell* A, const double* diag_inv, const double* b, double* x, double atol,
                         double rtol, int64_t maxit, int32_t check_every, int32_t norm, int32_t use_graph,
                         int32_t profile, void* workspace, size_t workspace_bytes, fgb_pcg_info* info,
                         void* stream) {
  if (!A || A->n <= 0 || !A->val64 || !b || !x || maxit <= 0 || !launch_ok(A)) return FGB_ERR_ARG;
  if (!workspace || workspace_bytes < fgb_pcg_sell_workspace_bytes(A->n)) return FGB_ERR_WORKSPACE;
  if (check_every <= 0) check_every = 16;
  if (use_graph) profile = 0;
  cudaStream_t s = as_stream(stream);
  SellView v = view_of(A);
  const int64_t n = A->n;
  Carver cv(workspace, workspace_bytes);
  F64Work w;
  if (!carve_f64(cv, n, w)) return FGB_ERR_WORKSPACE;
  SellPcgState h{};
  h.atol = atol;
  h.maxit = maxit;
  h.norm_rr = norm;
  h.trip_cap = maxit / 2 + 2;
  int64_t launches = 0;
  cudaMemcpyAsync(w.st, &h, sizeof(SellPcgState), cudaMemcpyHostToDevice, s);
  with_cols(v, [&](auto d16) {
    sell_pcg_init<double, decltype(d16)::value>
        <<<SLICE_LAUNCH(v, s)>>>(v, A->val64, diag_inv, b, x, w.r, w.z, w.p0, w.partials, w.st);
  });
  ++launches;
  int rc = read_state(w.st, &h, s);
  if (rc) return rc;
  EventPairs prof(profile != 0, check_every);
  int used_graph = 0;
  if (h.done == FGB_PCG_ZERO_RHS) {
    cudaMemsetAsync(x, 0, n * sizeof(double), s);
  } else {
    if ((rc = set_tol(w.st, rtol * h.b_norm, s))) return rc;
    bool graphed = false;
    if (use_graph) {
      bool launched = false;
      rc = graph_loop([&](CaptureCtx& c) {
        f64_body(v, A->val64, diag_inv, x, w, 0, nullptr, c.cs);
        f64_body(v, A->val64, diag_inv, x, w, 1, nullptr, c.cs);
      }, w.st, s, &launched);
      if (rc && launched) return rc;
      if (rc == FGB_OK) {
        graphed = true;
        used_graph = 1;
        if ((rc = read_state(w.st, &h, s))) return rc;
        launches += 7 * ((h.niter + 1) / 2 + 1);
      }
      rc = FGB_OK;
    }
    if (!graphed) {
      int64_t it = 0;
      while (true) {
        const int64_t before = h.niter;
        for (int k = 0; k < check_every; ++k, ++it) f64_body(v, A->val64, diag_inv, x, w, static_cast<int>(it & 1), prof.of(k), s);
        launches += 3 * check_every;
        if (cudaGetLastError() != cudaSuccess) return FGB_ERR_CUDA;
        if ((rc = read_state(w.st, &h, s))) return rc;
        prof.collect(h.niter - before);
        if (h.done) break;
      }
    }
  }
  if (info) {
    info->niter = h.niter; info->residual = h.resid; info->b_norm = h.b_norm; info->true_relres = -1.0;
    info->reason = h.done; info->n_updates = 0; info->launches = launches; info->kernel_ms = prof.ms;
    info->kernel_launches = prof.launches;
    info->other_ms = prof.other;
    info->extra_ms = prof.extra;
    info->graph = used_graph;
    info->reserved = 0;
  }
  return finish(h.done);
}

void fgb_sell_set_pipeline(int32_t enable) { g_sell_pipe = enable ? 1 : 0; }

int32_t fgb_pcg_sell_mixed(const fgb_sell* A, const double* diag_inv64, const double* b, double* x, double rtol,
                           double delta, int64_t maxit, int32_t check_every, int32_t use_graph, int32_t profile,
                           void* workspace, size_t workspace_bytes, fgb_pcg_info* info, void* stream) {
  return fgb_pcg_sell_mixed_ex(A, diag_inv64, b, x, rtol, delta, maxit, check_every, use_graph, profile, 0,
                               workspace, workspace_bytes, info, stream);
}

int32_t fgb_pcg_sell_mixed_ex(const fgb_sell* A, const double* diag_inv64, const double* b, double* x, double rtol,
                              double delta, int64_t maxit, int32_t check_every, int32_t use_graph, int32_t profile,
                              int64_t barrier_polls, void* workspace, size_t workspace_bytes, fgb_pcg_info* info,
                              void* stream) {
  if (!A || A->n <= 0 || !A->val32 || !diag_inv64 || !b || !x || maxit <= 0 || !launch_ok(A)) return FGB_ERR_ARG;
  if (!(delta > 0.0 && delta < 1.0)) return FGB_ERR_ARG;
  if (!workspace || workspace_bytes < fgb_pcg_sell_workspace_bytes(A->n)) return FGB_ERR_WORKSPACE;
  if (check_every <= 0) check_every = 16;
  if (use_graph) profile = 0;
  cudaStream_t s = as_stream(stream);
  SellView v = view_of(A);
  const int64_t n = A->n;
  Carver cv(workspace, workspace_bytes);
  MixedWork w;
  if (!carve_mixed(cv, n, w)) return FGB_ERR_WORKSPACE;
  SellPcgState h{};
  h.maxit = maxit;
  h.norm_rr = 1;
  h.trip_cap = maxit / 2 + 2;
  int64_t launches = 0;
  cudaMemcpyAsync(w.st, &h, sizeof(SellPcgState), cudaMemcpyHostToDevice, s);
  sell_bnorm<<<VEC_LAUNCH(n, s)>>>(n, b, w.partials, w.st);
  cudaMemsetAsync(w.y, 0, n * sizeof(float), s);
  ++launches;
  int rc = read_state(w.st, &h, s);
  if (rc) return rc;
  EventPairs prof(profile != 0, check_every);
  int used_graph = 0;
  if (h.done == FGB_PCG_ZERO_RHS) {
    cudaMemsetAsync(x, 0, n * sizeof(double), s);
  } else {
    if ((rc = set_tol(w.st, rtol * h.b_norm, s))) return rc;
    // initial residual in FP64, its FP32 copy, z and p = z
    with_cols(v, [&](auto d16) {
      constexpr int D = decltype(d16)::value;
      if (A->val64)
        sell_mixed_reliable<double, D><<<SLICE_LAUNCH(v, s)>>>(v, A->val64, b, x, diag_inv64, w.dinv32, w.r, w.z,
                                                               w.p0, w.partials, w.st, 1);
      else
        sell_mixed_reliable<float, D><<<SLICE_LAUNCH(v, s)>>>(v, A->val32, b, x, diag_inv64, w.dinv32, w.r, w.z,
                                                              w.p0, w.partials, w.st, 1);
    });
    ++launches;
    bool graphed = false;
    if (use_graph == 2) {
      // every iteration inside one persistent cooperative kernel
      const PersistArgs pa{v, A->val32, A->val64 ? static_cast<const void*>(A->val64)
                                                 : static_cast<const void*>(A->val32),
                           b, x, w.dinv32, w.r, w.z, w.p0, w.Ap, w.y, w.bpart, w.partials, w.st, delta,
                           barrier_polls > 0 ? static_cast<long long>(barrier_polls) : kBarrierSpins};
      bool launched = false;
      with_cols(v, [&](auto d16) {
        constexpr int D = decltype(d16)::value;
        launched = A->val64 ? launch_persistent<D, double>(pa, s) : launch_persistent<D, float>(pa, s);
      });
      if (launched) {
        if ((rc = read_state(w.st, &h, s))) return rc;
        // a grid barrier gave up: every block has returned; with the default
        // limit this cannot happen while all blocks are resident
        if (h.bar_err) return FGB_ERR_CUDA;
        graphed = true;
        used_graph = 2;
        ++launches;
      }
    }
    if (use_graph && !graphed) {
      bool launched = false;
      rc = graph_loop([&](CaptureCtx& c) {
        mixed_body(v, A->val32, A->val64, diag_inv64, b, x, w, delta, 0, nullptr, c.cs, &c);
        mixed_body(v, A->val32, A->val64, diag_inv64, b, x, w, delta, 1, nullptr, c.cs, &c);
      }, w.st, s, &launched);
      if (rc && launched) return rc;
      if (rc == FGB_OK) {
        graphed = true;
        used_graph = 1;
        if ((rc = read_state(w.st, &h, s))) return rc;
        // per trip: 2 x (p update + SpMV + update) + loop control; fold + reliable
        // update when due
        launches += 7 * ((h.niter + 1) / 2 + 1) + 2 * h.n_updates;
      }
      rc = FGB_OK;
    }
    if (!graphed) {
      int64_t it = 0;
      while (true) {
        const int64_t before = h.niter;
        for (int k = 0; k < check_every; ++k, ++it)
          mixed_body(v, A->val32, A->val64, diag_inv64, b, x, w, delta, static_cast<int>(it & 1), prof.of(k), s);
        launches += 5 * check_every;
        if (cudaGetLastError() != cudaSuccess) return FGB_ERR_CUDA;
        if ((rc = read_state(w.st, &h, s))) return rc;
        prof.collect(h.niter - before);
        if (h.done) break;
      }
    }
    // the FP32 correction left over when the loop ended without a final
    // reliable update (breakdown, non-finite values, trip cap)
    sell_mixed_fold<<<VEC_LAUNCH(n, s)>>>(n, x, w.y, w.st, 1);
    ++launches;
    if (cudaStreamSynchronize(s) != cudaSuccess) return FGB_ERR_CUDA;
  }
  if (info) {
    info->niter = h.niter; info->residual = h.resid; info->b_norm = h.b_norm; info->true_relres = h.true_rel;
    info->reason = h.done; info->n_updates = h.n_updates; info->launches = launches; info->kernel_ms = prof.ms;
    info->kernel_launches = prof.launches;
    info->other_ms = prof.other;
    info->extra_ms = prof.extra;
    info->graph = used_graph;
    info->reserved = 0;
  }
  return finish(h.done);
}

}  // extern "C"
