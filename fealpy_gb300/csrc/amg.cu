// Aggregation algebraic multigrid: hierarchy set-up and the V-cycle
// preconditioned CG, for the `M` slot of fealpy/solver/cg.py (FEALPy's
// GAMGSolver, fealpy/solver/gamg_solver.py:14-256, fills it with a
// Ruge-Stuben hierarchy and Gauss-Seidel smoothing; both are sequential
// algorithms, so the GPU version uses their data-parallel counterparts).
//
// Set-up of one level (integer work, deterministic):
//   aggregation  a maximal independent set of the matrix graph (off-diagonal
//                entries with |a_ij| > theta sqrt(|a_ii a_jj|)): every node
//                carries a key (state, hash priority, index); a
//                neighbourhood-max sweep finds the undecided nodes whose key
//                is the largest among their neighbours, which become roots;
//                their neighbours drop out; repeat until every node is
//                decided.  Roots are numbered in index order; every other
//                node joins the aggregate of its largest-keyed assigned
//                neighbour (one sweep reaches all of them: each dropped node
//                has a root neighbour).  Rows without off-diagonal entries
//                (Dirichlet rows) join no aggregate.  Distance-1 independence
//                keeps aggregates at a root and its neighbours, about a dozen
//                rows for Lagrange matrices of degree 2; a distance-2 set makes
//                aggregates of about fifty and more PCG iterations.
//   coarse matrix  A_c = P^T A P with P the aggregate indicator: the members
//                of every aggregate (counting sort, each list sorted), and per
//                coarse row the entries of the member rows mapped to their
//                aggregates and summed per coarse column in a fixed order: by
//                one warp through a shared-memory hash table (rows of up to
//                192 coarse columns), else by a block that sorts the entries
//                by (coarse column, position) in shared memory (count pass,
//                scan, fill pass).
//   bounds       per row 1/a_ii and the Gershgorin bound of D^-1 A (max over
//                rows of sum_j |a_ij| / |a_ii|), for the Chebyshev smoother.
// Apply (V-cycle on r, from x = 0): Chebyshev smoothing of degree `deg` with
// D^-1 on [lmax/10, lmax]; the residual restricted by aggregate sums; the
// coarse correction prolonged and scaled by `omega` (over-correction, which
// plain aggregation needs); the same smoothing after; on the coarsest level
// a Chebyshev solve of degree `cdeg` on [lmax/20, lmax].  Every step is a
// fixed linear map, symmetric in A, so the V-cycle is a valid CG
// preconditioner.  The V-cycle reads the FP32 copy of a level's values when
// the level carries one (half the value bytes of the dominant sweeps; the
// rounded matrix is still symmetric, so the V-cycle stays a symmetric map);
// vectors and the PCG operator stay FP64.

#include "fgb_common.cuh"

#include <climits>
#include <cmath>
#include <type_traits>
#include <vector>

namespace fgb {

constexpr int kAmgThreads = 256;

__device__ __forceinline__ uint32_t amg_hash(uint32_t x) {
  x ^= x >> 16;
  x *= 0x7feb352dU;
  x ^= x >> 15;
  x *= 0x846ca68bU;
  x ^= x >> 16;
  return x & 0x7fffffffU;
}

// key = rank (2 root, 1 undecided, 0 out) | 31-bit priority | 31-bit index
__device__ __forceinline__ unsigned long long amg_key(int rank, int64_t i) {
  return (static_cast<unsigned long long>(rank) << 62) |
         (static_cast<unsigned long long>(amg_hash(static_cast<uint32_t>(i))) << 31) |
         static_cast<unsigned long long>(i);
}

// Strong coupling of entry (i, j): with theta = 0 every nonzero (no diagonal
// read); otherwise |a_ij| > theta sqrt(|a_ii a_jj|).
__device__ __forceinline__ bool amg_strong_at(double aij, double dii, const double* __restrict__ diag, int32_t j,
                                              double theta) {
  if (aij == 0.0) return false;
  if (theta == 0.0) return true;
  return fabs(aij) > theta * sqrt(fabs(dii * diag[j]));
}

// Rows in groups of 32 / G per warp (G lanes per row, G in {4, 8, 16, 32});
// the trip count is the same for every lane of a warp (the bound is tested
// on the warp's first row), so full-warp shuffles always have all 32 lanes
// present; rows past n take part with active = false.
#define AMG_ROW_LOOP(n, G)                                                                                   \
  const int sub = threadIdx.x & ((G) - 1);                                                                   \
  const int64_t wfirst = ((blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x) >> 5) * (32 / (G));  \
  const int64_t wstep = ((static_cast<int64_t>(gridDim.x) * blockDim.x) >> 5) * (32 / (G));                  \
  for (int64_t wr = wfirst, i = wfirst + (threadIdx.x & 31) / (G); wr < (n); wr += wstep, i += wstep)

template <int G, typename T>
__device__ __forceinline__ T group_max(T v) {
#pragma unroll
  for (int o = G >> 1; o > 0; o >>= 1) {
    const T u = __shfl_xor_sync(0xffffffffu, v, o, G);
    v = u > v ? u : v;
  }
  return v;
}

// diag and the Gershgorin bound of D^-1 A (G lanes per row)
template <int G>
__global__ void amg_diag_kernel(int64_t n, const int64_t* __restrict__ indptr, const int32_t* __restrict__ indices,
                                const double* __restrict__ values, double* __restrict__ diag,
                                unsigned long long* __restrict__ bound_bits, int32_t* status) {
  unsigned long long bmax = 0ull;
  AMG_ROW_LOOP(n, G) {
    const bool active = i < n;
    double d = 0.0, s = 0.0;
    if (active)
      for (int64_t e = indptr[i] + sub; e < indptr[i + 1]; e += G) {
        const double a = values[e];
        if (indices[e] == i) d += a;
        s += fabs(a);
      }
#pragma unroll
    for (int o = G >> 1; o > 0; o >>= 1) {
      d += __shfl_xor_sync(0xffffffffu, d, o, G);
      s += __shfl_xor_sync(0xffffffffu, s, o, G);
    }
    if (active && sub == 0) {
      diag[i] = d;
      if (!(d > 0.0) || !isfinite(d)) {
        set_status(status, FGB_ERR_BREAKDOWN);  // an SPD matrix has a positive diagonal
      } else {
        const unsigned long long b = static_cast<unsigned long long>(__double_as_longlong(s / d));
        bmax = b > bmax ? b : bmax;  // positive doubles order as integers
      }
    }
  }
  // one atomic per warp
  bmax = group_max<32>(bmax);
  if ((threadIdx.x & 31) == 0 && bmax) atomicMax(bound_bits, bmax);
}

// state: 1 undecided, 2 root, 0 out, -1 isolated (no strong off-diagonal)
template <int G>
__global__ void amg_init_state(int64_t n, const int64_t* __restrict__ indptr, const int32_t* __restrict__ indices,
                               const double* __restrict__ values, const double* __restrict__ diag, double theta,
                               int32_t* __restrict__ state) {
  AMG_ROW_LOOP(n, G) {
    const bool active = i < n;
    int strong = 0;
    if (active) {
      const double di = diag[i];
      for (int64_t e = indptr[i] + sub; e < indptr[i + 1]; e += G) {
        const int32_t j = indices[e];
        if (j < 0 || j >= n || j == i) continue;
        if (amg_strong_at(values[e], di, diag, j, theta)) strong = 1;
      }
    }
    strong = group_max<G>(strong);
    if (active && sub == 0) state[i] = strong ? 1 : -1;
  }
}

__global__ void amg_keys(int64_t n, const int32_t* __restrict__ state, unsigned long long* __restrict__ key) {
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int s = state[i];
    key[i] = s < 0 ? 0ull : amg_key(s == 2 ? 2 : (s == 1 ? 1 : 0), i);
  }
}

// One maximal-independent-set round: m = max of key over the strong
// neighbours of i; an undecided node whose own key exceeds it becomes a root,
// one that sees a root drops out; counts the nodes still undecided.  Reads
// only the keys of the round (written by amg_keys before), so the result does
// not depend on the order of the threads.
template <int G>
__global__ void amg_mis_round(int64_t n, const int64_t* __restrict__ indptr, const int32_t* __restrict__ indices,
                              const double* __restrict__ values, const double* __restrict__ diag, double theta,
                              const unsigned long long* __restrict__ key, int32_t* __restrict__ state,
                              int32_t* __restrict__ undecided) {
  int local = 0;
  AMG_ROW_LOOP(n, G) {
    const bool active = i < n && state[i] == 1;  // uniform within the row's lanes
    unsigned long long m = 0ull;
    if (active) {
      const double di = diag[i];
      for (int64_t e = indptr[i] + sub; e < indptr[i + 1]; e += G) {
        const int32_t j = indices[e];
        if (j < 0 || j >= n || j == i) continue;
        if (amg_strong_at(values[e], di, diag, j, theta)) {
          const unsigned long long v = key[j];
          m = v > m ? v : m;
        }
      }
    }
    m = group_max<G>(m);
    if (active && sub == 0) {
      const unsigned long long k = key[i];
      if (k > m) state[i] = 2;
      else if ((m >> 62) == 2ull) state[i] = 0;
      else ++local;
    }
  }
  if (local) atomicAdd(undecided, local);
}

__global__ void amg_root_flags(int64_t n, const int32_t* __restrict__ state, int32_t* __restrict__ flag) {
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x)
    flag[i] = state[i] == 2 ? 1 : 0;
}

__global__ void amg_root_ids(int64_t n, const int32_t* __restrict__ state, const int64_t* __restrict__ off,
                             int32_t* __restrict__ agg) {
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x)
    agg[i] = state[i] == 2 ? static_cast<int32_t>(off[i]) : -1;
}

// One assignment sweep: an unassigned node with strong neighbours takes the
// aggregate of the assigned strong neighbour with the largest (priority,
// index); reads agg_in, writes agg_out (so the sweep does not depend on the
// order of the threads); counts the nodes still unassigned.
template <int G>
__global__ void amg_assign(int64_t n, const int64_t* __restrict__ indptr, const int32_t* __restrict__ indices,
                           const double* __restrict__ values, const double* __restrict__ diag, double theta,
                           const int32_t* __restrict__ state, const int32_t* __restrict__ agg_in,
                           int32_t* __restrict__ agg_out, int32_t* __restrict__ left) {
  int local = 0;
  AMG_ROW_LOOP(n, G) {
    const bool active = i < n;
    const int32_t a0 = active ? agg_in[i] : 0;
    const bool need = active && a0 < 0 && state[i] >= 0;  // uniform within the row's lanes
    // best assigned neighbour as amg_key(1, j): nonzero when found
    unsigned long long best = 0ull;
    if (need) {
      const double di = diag[i];
      for (int64_t e = indptr[i] + sub; e < indptr[i + 1]; e += G) {
        const int32_t j = indices[e];
        if (j < 0 || j >= n || j == i || agg_in[j] < 0 || !amg_strong_at(values[e], di, diag, j, theta)) continue;
        const unsigned long long k = amg_key(1, j);
        best = k > best ? k : best;
      }
    }
    best = group_max<G>(best);
    if (active && sub == 0) {
      int32_t a = a0;
      if (need) {
        a = best ? agg_in[static_cast<int32_t>(best & 0x7fffffffull)] : -1;
        if (a < 0) ++local;
      }
      agg_out[i] = a;
    }
  }
  if (local) atomicAdd(left, local);
}

// ------------------------------------------------------------ coarse matrix
__global__ void amg_member_count(int64_t n, const int32_t* __restrict__ agg, int32_t* __restrict__ cnt) {
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x)
    if (agg[i] >= 0) atomicAdd(cnt + agg[i], 1);
}

__global__ void amg_member_fill(int64_t n, const int32_t* __restrict__ agg, const int64_t* __restrict__ mptr,
                                int32_t* __restrict__ cursor, int32_t* __restrict__ members) {
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x)
    if (agg[i] >= 0) members[mptr[agg[i]] + atomicAdd(cursor + agg[i], 1)] = static_cast<int32_t>(i);
}

// each member list in ascending row order (insertion sort by one thread;
// aggregates hold tens of rows)
__global__ void amg_member_sort(int64_t nc, const int64_t* __restrict__ mptr, int32_t* __restrict__ members) {
  for (int64_t c = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; c < nc;
       c += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int64_t a = mptr[c], b = mptr[c + 1];
    for (int64_t k = a + 1; k < b; ++k) {
      const int32_t v = members[k];
      int64_t u = k - 1;
      while (u >= a && members[u] > v) {
        members[u + 1] = members[u];
        --u;
      }
      members[u + 1] = v;
    }
  }
}

constexpr int kCoarseThreads = 256;
constexpr int kCoarseCap = 2048;      // candidates per coarse row, first pass (shared memory)
constexpr int kCoarseBigCap = 8192;  // second pass (dynamic shared memory, 128 KB)

// Coarse row I: candidates (J << 32 | position, value) of the member rows in
// order, sorted in shared memory, summed per J in position order.  mode 0:
// the number of distinct J to cnt[I]; mode 1: columns and values at
// cptr[I].  Returns false when the candidates exceed cap (nothing written).
__device__ bool amg_coarse_row(int64_t n, int64_t I, int mode, const int64_t* __restrict__ indptr,
                               const int32_t* __restrict__ indices, const double* __restrict__ values,
                               const int32_t* __restrict__ agg, const int64_t* __restrict__ mptr,
                               const int32_t* __restrict__ members, int32_t* __restrict__ cnt,
                               const int64_t* __restrict__ cptr, int32_t* __restrict__ ccol,
                               double* __restrict__ cval, unsigned long long* kbuf, double* vbuf, int cap,
                               int* sh_m, int* sh_u) {
  const int tid = threadIdx.x, nt = blockDim.x;
  // candidate count: sum of the member rows' lengths
  if (tid == 0) {
    int64_t m = 0;
    for (int64_t k = mptr[I]; k < mptr[I + 1]; ++k) {
      const int32_t r = members[k];
      m += indptr[r + 1] - indptr[r];
    }
    *sh_m = m > cap ? -1 : static_cast<int>(m);
  }
  __syncthreads();
  const int m = *sh_m;
  if (m < 0) return false;
  int np2 = 1;
  while (np2 < m) np2 <<= 1;
  // fill: walk member rows in order; positions are the running entry index
  if (tid == 0) *sh_u = 0;
  for (int64_t k = mptr[I]; k < mptr[I + 1]; ++k) {
    const int32_t r = members[k];
    const int64_t a = indptr[r];
    const int len = static_cast<int>(indptr[r + 1] - a);
    __syncthreads();
    const int base = *sh_u;
    for (int t = tid; t < len; t += nt) {
      const int32_t j = indices[a + t];
      const int32_t J = (j >= 0 && j < n) ? agg[j] : -1;
      const int pos = base + t;
      kbuf[pos] = J >= 0 ? ((static_cast<unsigned long long>(static_cast<uint32_t>(J)) << 32) | static_cast<uint32_t>(pos))
                         : ULLONG_MAX;
      vbuf[pos] = values[a + t];
    }
    __syncthreads();
    if (tid == 0) *sh_u = base + len;
  }
  __syncthreads();
  for (int t = m + tid; t < np2; t += nt) {
    kbuf[t] = ULLONG_MAX;
    vbuf[t] = 0.0;
  }
  __syncthreads();
  for (int kk = 2; kk <= np2; kk <<= 1) {
    for (int j = kk >> 1; j > 0; j >>= 1) {
      for (int t = tid; t < np2; t += nt) {
        const int u = t ^ j;
        if (u > t) {
          const unsigned long long a = kbuf[t], b = kbuf[u];
          const bool up = (t & kk) == 0;
          if ((a > b) == up) {
            kbuf[t] = b;
            kbuf[u] = a;
            const double va = vbuf[t];
            vbuf[t] = vbuf[u];
            vbuf[u] = va;
          }
        }
      }
      __syncthreads();
    }
  }
  // distinct coarse columns (entries with J < 0 sorted last as ULLONG_MAX):
  // thread tid owns the sorted positions [tid * chunk, (tid + 1) * chunk),
  // counts the run heads there, takes its output offset from a block scan of
  // the counts, and sums each of its runs serially in position order (a run
  // may extend past the chunk), which is the order of a serial merge.
  const int chunk = (m + nt - 1) / nt;
  const int t0 = min(m, tid * chunk), t1 = min(m, t0 + chunk);
  auto head = [&](int t) -> bool {
    const unsigned long long k = kbuf[t];
    return k != ULLONG_MAX && (t == 0 || (kbuf[t - 1] >> 32) != (k >> 32));
  };
  int heads = 0;
  for (int t = t0; t < t1; ++t) heads += head(t) ? 1 : 0;
  // exclusive block scan of heads (warp scans, then the warp totals)
  const int lane = tid & 31, wid = tid >> 5;
  int incl = heads;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int u = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += u;
  }
  int* wsum = sh_u + 1;  // nt / 32 ints after sh_u
  if (lane == 31) wsum[wid] = incl;
  __syncthreads();
  int base = 0;
  for (int w = 0; w < wid; ++w) base += wsum[w];
  int u = base + incl - heads;
  if (mode == 1) {
    const int64_t out0 = cptr[I];
    for (int t = t0; t < t1; ++t) {
      if (!head(t)) continue;
      const unsigned long long J = kbuf[t] >> 32;
      double s = 0.0;
      for (int q = t; q < m && kbuf[q] != ULLONG_MAX && (kbuf[q] >> 32) == J; ++q) s += vbuf[q];
      ccol[out0 + u] = static_cast<int32_t>(J);
      cval[out0 + u] = s;
      ++u;
    }
  }
  if (mode == 0 && tid == nt - 1) cnt[I] = base + incl;
  __syncthreads();
  return true;
}

constexpr int kWarpRowWarps = 8;   // warps per block of the warp path
constexpr int kHashSlots = 256;    // coarse columns per warp (open addressing)
constexpr int kHashMax = 192;      // distinct coarse columns the warp path takes

// Coarse row I by one warp (the common case): the member rows' entries,
// member by member in CSR order, 32 at a time; lanes with the same coarse
// column J (the aggregate of the entry's column) sum their values in lane
// order, and the lowest of them adds that sum to J's slot of a shared-memory
// hash table (chunks in order, so every J's sum is taken in a fixed order).
// mode 0: the number of distinct J to cnt[I]; mode 1: columns ascending and
// values at cptr[I].  A row with more than kHashMax distinct J goes to the
// overflow list (block path).
__global__ void __launch_bounds__(kWarpRowWarps * 32) amg_coarse_rows_warp(
    int64_t n, int64_t nc, int mode, const int64_t* __restrict__ indptr, const int32_t* __restrict__ indices,
    const double* __restrict__ values, const int32_t* __restrict__ agg, const int64_t* __restrict__ mptr,
    const int32_t* __restrict__ members, int32_t* __restrict__ cnt, const int64_t* __restrict__ cptr,
    int32_t* __restrict__ ccol, double* __restrict__ cval, int32_t* __restrict__ ovf, int32_t* __restrict__ ovf_len) {
  __shared__ int32_t hkey[kWarpRowWarps][kHashSlots];
  __shared__ double hval[kWarpRowWarps][kHashSlots];
  __shared__ double stage[kWarpRowWarps][32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  int32_t* K = hkey[w];
  double* V = hval[w];
  double* S = stage[w];
  const int64_t gw = (blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x) >> 5;
  const int64_t nw = (static_cast<int64_t>(gridDim.x) * blockDim.x) >> 5;
  for (int64_t I = gw; I < nc; I += nw) {
    for (int t = lane; t < kHashSlots; t += 32) {
      K[t] = -1;
      V[t] = 0.0;
    }
    __syncwarp();
    bool over = false;  // warp-uniform
    int distinct = 0;   // warp-uniform
    const int64_t m0 = mptr[I], m1 = mptr[I + 1];
    for (int64_t k = m0; k < m1 && !over; ++k) {
      const int32_t row = members[k];
      const int64_t a = indptr[row], b = indptr[row + 1];
      for (int64_t e0 = a; e0 < b && !over; e0 += 32) {
        const int64_t e = e0 + lane;
        int32_t J = -1;
        double v = 0.0;
        if (e < b) {
          const int32_t j = indices[e];
          if (j >= 0 && j < n) J = agg[j];
          v = values[e];
        }
        S[lane] = v;
        __syncwarp();
        const unsigned grp = __match_any_sync(0xffffffffu, J);
        int claimed = 0, fail = 0;
        if (J >= 0 && __ffs(grp) - 1 == lane) {
          double sum = 0.0;
          for (unsigned m = grp; m; m &= m - 1) sum += S[__ffs(m) - 1];
          unsigned h = (static_cast<unsigned>(J) * 2654435761u) >> 24;
          int probes = 0;
          while (true) {
            const int32_t old = atomicCAS(&K[h], -1, J);
            if (old == -1) {
              claimed = 1;
              break;
            }
            if (old == J) break;
            h = (h + 1) & (kHashSlots - 1);
            if (++probes >= kHashSlots) {
              fail = 1;
              break;
            }
          }
          if (!fail) V[h] += sum;
        }
        distinct += __popc(__ballot_sync(0xffffffffu, claimed));
        over = __any_sync(0xffffffffu, fail) || distinct > kHashMax;
        __syncwarp();
      }
    }
    if (over) {
      if (lane == 0) ovf[atomicAdd(ovf_len, 1)] = static_cast<int32_t>(I);
    } else if (mode == 0) {
      if (lane == 0) cnt[I] = distinct;
    } else {
      // ascending J: each occupied slot's rank among the occupied keys
      const int64_t out0 = cptr[I];
      for (int t = lane; t < kHashSlots; t += 32) {
        const int32_t J = K[t];
        if (J < 0) continue;
        int rank = 0;
        for (int u = 0; u < kHashSlots; ++u) {
          const int32_t q = K[u];
          rank += (q >= 0 && q < J) ? 1 : 0;
        }
        ccol[out0 + rank] = J;
        cval[out0 + rank] = V[t];
      }
    }
    __syncwarp();
  }
}

// Coarse rows of a list (the warp path's overflow) by a block each; rows
// above kCoarseCap candidates go on to the next list.
__global__ void __launch_bounds__(kCoarseThreads) amg_coarse_rows(int64_t n, int mode,
                                                                 const int64_t* __restrict__ indptr,
                                                                 const int32_t* __restrict__ indices,
                                                                 const double* __restrict__ values,
                                                                 const int32_t* __restrict__ agg,
                                                                 const int64_t* __restrict__ mptr,
                                                                 const int32_t* __restrict__ members,
                                                                 int32_t* __restrict__ cnt,
                                                                 const int64_t* __restrict__ cptr,
                                                                 int32_t* __restrict__ ccol, double* __restrict__ cval,
                                                                 const int32_t* __restrict__ rows,
                                                                 const int32_t* __restrict__ rows_len,
                                                                 int32_t* __restrict__ ovf, int32_t* __restrict__ ovf_len) {
  __shared__ unsigned long long kbuf[kCoarseCap];
  __shared__ double vbuf[kCoarseCap];
  __shared__ int sh[2 + kCoarseThreads / 32];  // candidate count, fill offset, warp totals
  const int nr = *rows_len;
  for (int r = blockIdx.x; r < nr; r += gridDim.x) {
    const int32_t I = rows[r];
    const bool ok = amg_coarse_row(n, I, mode, indptr, indices, values, agg, mptr, members, cnt, cptr, ccol, cval, kbuf,
                                   vbuf, kCoarseCap, sh, sh + 1);
    if (!ok && threadIdx.x == 0) ovf[atomicAdd(ovf_len, 1)] = I;
    __syncthreads();
  }
}

__global__ void __launch_bounds__(kCoarseThreads) amg_coarse_rows_big(int64_t n, int mode,
                                                                     const int64_t* __restrict__ indptr,
                                                                     const int32_t* __restrict__ indices,
                                                                     const double* __restrict__ values,
                                                                     const int32_t* __restrict__ agg,
                                                                     const int64_t* __restrict__ mptr,
                                                                     const int32_t* __restrict__ members,
                                                                     int32_t* __restrict__ cnt,
                                                                     const int64_t* __restrict__ cptr,
                                                                     int32_t* __restrict__ ccol,
                                                                     double* __restrict__ cval,
                                                                     const int32_t* __restrict__ ovf,
                                                                     const int32_t* __restrict__ ovf_len,
                                                                     int32_t* status) {
  extern __shared__ __align__(16) unsigned char dsm[];
  unsigned long long* kbuf = reinterpret_cast<unsigned long long*>(dsm);
  double* vbuf = reinterpret_cast<double*>(dsm + static_cast<size_t>(kCoarseBigCap) * 8);
  __shared__ int sh[2 + kCoarseThreads / 32];
  const int n_ovf = *ovf_len;
  for (int r = blockIdx.x; r < n_ovf; r += gridDim.x) {
    const bool ok = amg_coarse_row(n, ovf[r], mode, indptr, indices, values, agg, mptr, members, cnt, cptr, ccol, cval,
                                   kbuf, vbuf, kCoarseBigCap, sh, sh + 1);
    if (!ok && threadIdx.x == 0) set_status(status, FGB_ERR_CAPACITY);
    __syncthreads();
  }
}

// ------------------------------------------------------------ apply kernels
// Rows with G lanes each (G in {4, 8, 16, 32}); y = A x fused with a
// per-row epilogue.  V: type of the matrix values, T: type of the vectors and
// of the arithmetic (float for the FP32 V-cycle: GB300's FP64 pipe is narrow
// enough that FP64 products bound a sweep's time well above its bytes).
// (A x)_i by the G lanes of row i; every lane of the warp calls it (rows past
// n pass active = false and contribute nothing), so the full-warp shuffles
// always have all 32 lanes present.
template <int G, typename V, typename T>
__device__ __forceinline__ T csr_row_dot(int64_t i, bool active, const int64_t* __restrict__ indptr,
                                         const int32_t* __restrict__ indices, const V* __restrict__ values,
                                         const T* __restrict__ x, int sub) {
  T acc = T(0);
  if (active) {
    const int64_t e1 = indptr[i + 1];
#pragma unroll 4
    for (int64_t e = indptr[i] + sub; e < e1; e += G) acc += static_cast<T>(values[e]) * x[indices[e]];
  }
#pragma unroll
  for (int o = G >> 1; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o, G);
  return acc;
}

// Chebyshev step: d = c1 d + c2 Dinv (r - A x_in); x_out = x_in + d
template <int G, typename V, typename T>
__global__ void amg_cheb_step(int64_t n, const int64_t* __restrict__ indptr, const int32_t* __restrict__ indices,
                              const V* __restrict__ values, const T* __restrict__ dinv, const T* __restrict__ r,
                              const T* __restrict__ x_in, T* __restrict__ x_out, T* __restrict__ d, T c1, T c2) {
  AMG_ROW_LOOP(n, G) {
    const bool active = i < n;
    const T ax = csr_row_dot<G, V, T>(i, active, indptr, indices, values, x_in, sub);
    if (active && sub == 0) {
      const T di = (c1 != T(0) ? c1 * d[i] : T(0)) + c2 * dinv[i] * (r[i] - ax);
      d[i] = di;
      x_out[i] = x_in[i] + di;
    }
  }
}

__global__ void amg_invert(int64_t n, const double* __restrict__ diag, double* __restrict__ dinv) {
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x)
    dinv[i] = 1.0 / diag[i];
}

template <typename A, typename B>
__global__ void amg_convert(int64_t n, const A* __restrict__ a, B* __restrict__ b) {
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x)
    b[i] = static_cast<B>(a[i]);
}

// first Chebyshev step from x = 0: d = c2 Dinv r, x = d
template <typename T>
__global__ void amg_cheb_first(int64_t n, const T* __restrict__ dinv, const T* __restrict__ r, T* __restrict__ x,
                               T* __restrict__ d, T c2) {
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const T di = c2 * dinv[i] * r[i];
    d[i] = di;
    x[i] = di;
  }
}

// res = r - A x
template <int G, typename V, typename T>
__global__ void amg_residual(int64_t n, const int64_t* __restrict__ indptr, const int32_t* __restrict__ indices,
                             const V* __restrict__ values, const T* __restrict__ r, const T* __restrict__ x,
                             T* __restrict__ res) {
  AMG_ROW_LOOP(n, G) {
    const bool active = i < n;
    const T ax = csr_row_dot<G, V, T>(i, active, indptr, indices, values, x, sub);
    if (active && sub == 0) res[i] = r[i] - ax;
  }
}

// rc[I] = sum of res over the members of aggregate I, in row order
template <typename T>
__global__ void amg_restrict(int64_t nc, const int64_t* __restrict__ mptr, const int32_t* __restrict__ members,
                             const T* __restrict__ res, T* __restrict__ rc) {
  for (int64_t I = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; I < nc;
       I += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    T s = T(0);
    for (int64_t k = mptr[I]; k < mptr[I + 1]; ++k) s += res[members[k]];
    rc[I] = s;
  }
}

// x[i] += omega * ec[agg[i]]
template <typename T>
__global__ void amg_prolong(int64_t n, const int32_t* __restrict__ agg, const T* __restrict__ ec, T omega,
                            T* __restrict__ x) {
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int32_t a = agg[i];
    if (a >= 0) x[i] += omega * ec[a];
  }
}

// ------------------------------------------------------------ PCG kernels
constexpr int kDotBlocks = 2 * kNumSMs;
constexpr int kMaxGrid = kNumSMs * 16;  // grids of every kernel here (grid_for caps)
static_assert(2 * kMaxGrid >= kNumSMs * 8, "the partials buffer holds a SELL launch's block partials");

// Deterministic two-value reduction: per-block sums in a fixed order, the last
// block adds the blocks' sums in block order into out[0..1].
__device__ void amg_reduce2(double a, double b, double* partials, unsigned int* counter, double* out) {
  __shared__ double sa[32], sb[32];
  __shared__ bool last;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  a = warp_sum(a);
  b = warp_sum(b);
  if (lane == 0) {
    sa[wid] = a;
    sb[wid] = b;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double ta = 0.0, tb = 0.0;
    for (int w = 0; w < static_cast<int>(blockDim.x >> 5); ++w) {
      ta += sa[w];
      tb += sb[w];
    }
    partials[blockIdx.x] = ta;
    partials[gridDim.x + blockIdx.x] = tb;
    __threadfence();
    last = atomicAdd(counter, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!last) return;  // uniform within the block
  // last block: thread t sums the partials t, t + blockDim.x, ... in order,
  // then the block's sums combine as above (a fixed order for a fixed grid)
  __threadfence();
  double ta = 0.0, tb = 0.0;
  for (unsigned int k = threadIdx.x; k < gridDim.x; k += blockDim.x) {
    ta += __ldcg(partials + k);
    tb += __ldcg(partials + gridDim.x + k);
  }
  ta = warp_sum(ta);
  tb = warp_sum(tb);
  __syncthreads();  // the first combine's reads of sa, sb are done
  if (lane == 0) {
    sa[wid] = ta;
    sb[wid] = tb;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double fa = 0.0, fb = 0.0;
    for (int w = 0; w < static_cast<int>(blockDim.x >> 5); ++w) {
      fa += sa[w];
      fb += sb[w];
    }
    out[0] = fa;
    out[1] = fb;
    *counter = 0u;
  }
}

// Ap = A p; out = (p.Ap, 0)
template <int G, typename V>
__global__ void amg_pcg_spmv(int64_t n, const int64_t* __restrict__ indptr, const int32_t* __restrict__ indices,
                             const V* __restrict__ values, const double* __restrict__ p, double* __restrict__ Ap,
                             double* partials, unsigned int* counter, double* out) {
  double pap = 0.0;
  AMG_ROW_LOOP(n, G) {
    const bool active = i < n;
    const double ax = csr_row_dot<G, V, double>(i, active, indptr, indices, values, p, sub);
    if (active && sub == 0) {
      Ap[i] = ax;
      pap += p[i] * ax;
    }
  }
  amg_reduce2(pap, 0.0, partials, counter, out);
}

// x += alpha p, r -= alpha Ap; out = (r.r, 0)
__global__ void amg_pcg_update(int64_t n, double alpha, const double* __restrict__ p, const double* __restrict__ Ap,
                               double* __restrict__ x, double* __restrict__ r, double* partials, unsigned int* counter,
                               double* out) {
  double rr = 0.0;
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    x[i] += alpha * p[i];
    const double ri = r[i] - alpha * Ap[i];
    r[i] = ri;
    rr += ri * ri;
  }
  amg_reduce2(rr, 0.0, partials, counter, out);
}

// out = (a.b, a.a)
__global__ void amg_dot2(int64_t n, const double* __restrict__ a, const double* __restrict__ b, double* partials,
                         unsigned int* counter, double* out) {
  double ab = 0.0, aa = 0.0;
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    ab += a[i] * b[i];
    aa += a[i] * a[i];
  }
  amg_reduce2(ab, aa, partials, counter, out);
}

// Device state of the PCG loop (the loop runs as a CUDA-graph while node:
// alpha, beta and the stopping test are computed on the device).
struct AmgPcgState {
  double rz, beta, tol, atol, resid;
  double red[6];  // reduction outputs: [0] p.Ap, [2] r.r, [4] r.z
  long long niter, maxit, trips, trip_cap;
  int done, norm;
};

// x += alpha p, r -= alpha Ap with alpha = rz / p.Ap; a non-positive or
// non-finite p.Ap ends the solve and leaves x and r as they are; r.r to red[2]
__global__ void amg_pcg_update_dev(int64_t n, AmgPcgState* s, const double* __restrict__ p,
                                   const double* __restrict__ Ap, double* __restrict__ x, double* __restrict__ r,
                                   double* partials, unsigned int* counter) {
  const double pap = s->red[0];
  const bool bad = !(pap > 0.0) || !isfinite(pap);
  double rr = 0.0;
  if (!bad) {
    const double alpha = s->rz / pap;
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
      x[i] += alpha * p[i];
      const double ri = r[i] - alpha * Ap[i];
      r[i] = ri;
      rr += ri * ri;
    }
  } else if (blockIdx.x == 0 && threadIdx.x == 0) {
    s->done = isfinite(pap) ? FGB_PCG_BREAKDOWN : FGB_PCG_NONFINITE;
  }
  amg_reduce2(rr, 0.0, partials, counter, s->red + 2);
}

// End of an iteration (one thread): FEALPy's stopping rule on the residual
// (norm 0: sqrt(r.z), 1: ||r||), then beta = rz_new / rz; clears the while
// condition when the solve ends, and in any case after trip_cap iterations.
__global__ void amg_pcg_ctl(AmgPcgState* s, cudaGraphConditionalHandle handle) {
  if (!s->done) {
    const double rr = s->red[2], rzn = s->red[4];
    s->niter += 1;
    const double resid = s->norm ? sqrt(rr) : sqrt(fabs(rzn));
    s->resid = resid;
    if (!isfinite(resid)) s->done = FGB_PCG_NONFINITE;
    else if (resid < s->atol) s->done = FGB_PCG_ATOL;
    else if (resid < s->tol) s->done = FGB_PCG_RTOL;
    else if (s->niter >= s->maxit) s->done = FGB_PCG_MAXIT;
    else {
      s->beta = rzn / s->rz;
      s->rz = rzn;
    }
  }
  s->trips += 1;
  if (!s->done && s->trips >= s->trip_cap) s->done = FGB_PCG_MAXIT;
  if (s->done) cudaGraphSetConditional(handle, 0);
}

// p = z + beta p (nothing once the solve has ended)
__global__ void amg_pupdate_dev(int64_t n, const AmgPcgState* s, const double* __restrict__ z,
                                double* __restrict__ p) {
  if (s->done) return;
  const double beta = s->beta;
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x)
    p[i] = z[i] + beta * p[i];
}

// lanes per row: rows of up to about two entries per lane per pass
inline int amg_lanes(int64_t n, int64_t nnz) {
  const double avg = n > 0 ? static_cast<double>(nnz) / n : 0.0;
  return avg <= 10 ? 4 : (avg <= 48 ? 8 : (avg <= 96 ? 16 : 32));
}

inline int rows_grid(int64_t n, int G) { return grid_for(n * G, kAmgThreads, kNumSMs * 16); }
inline int vec_grid(int64_t n) { return grid_for(n, kAmgThreads, kNumSMs * 16); }

#define AMG_DISPATCH_ROWS(G, KERNEL, ...)                                                              \
  switch (G) {                                                                                         \
    case 4: KERNEL<4><<<rows_grid(n, 4), kAmgThreads, 0, st>>>(__VA_ARGS__); break;                   \
    case 8: KERNEL<8><<<rows_grid(n, 8), kAmgThreads, 0, st>>>(__VA_ARGS__); break;                   \
    case 16: KERNEL<16><<<rows_grid(n, 16), kAmgThreads, 0, st>>>(__VA_ARGS__); break;                \
    default: KERNEL<32><<<rows_grid(n, 32), kAmgThreads, 0, st>>>(__VA_ARGS__); break;                \
  }

// f(std::integral_constant<int, G>) for the lanes count G of a level
template <typename F>
void with_lanes(int G, F&& f) {
  switch (G) {
    case 4: f(std::integral_constant<int, 4>{}); break;
    case 8: f(std::integral_constant<int, 8>{}); break;
    case 16: f(std::integral_constant<int, 16>{}); break;
    default: f(std::integral_constant<int, 32>{}); break;
  }
}

// smoother sweep of a level's SELL copy, and Ap = A p with per-block p.Ap
// partials on its FP64 values (sell.cu)
int sell_smooth_f32(const fgb_sell* A, const float* dinv, const float* r, const float* x_in, float* x_out, float* d,
                    float c1, float c2, int mode, cudaStream_t st);
int sell_smooth_f64(const fgb_sell* A, const double* dinv, const double* r, const double* x_in, double* x_out,
                    double* d, double c1, double c2, int mode, cudaStream_t st);
int sell_spmv_pap_f64(const fgb_sell* A, const double* p, double* Ap, double* bpart, int* n_part, cudaStream_t st);

// the level's SELL sweep in the V-cycle's type (false: the level has no copy
// with values of that type)
inline bool sell_sweep(const fgb_amg_level& L, const float* dinv, const float* r, const float* x_in, float* x_out,
                       float* d, double c1, double c2, int mode, cudaStream_t st) {
  if (!L.sell || !L.sell->val32) return false;
  sell_smooth_f32(L.sell, dinv, r, x_in, x_out, d, static_cast<float>(c1), static_cast<float>(c2), mode, st);
  return true;
}
inline bool sell_sweep(const fgb_amg_level& L, const double* dinv, const double* r, const double* x_in,
                       double* x_out, double* d, double c1, double c2, int mode, cudaStream_t st) {
  if (!L.sell || !L.sell->val64) return false;
  sell_smooth_f64(L.sell, dinv, r, x_in, x_out, d, c1, c2, mode, st);
  return true;
}

// out[0] = sum of part[0..nb) in a fixed order (one block), out[1] = 0
__global__ void amg_sum_partials(const double* __restrict__ part, int nb, double* __restrict__ out) {
  __shared__ double ws[32];
  double t = 0.0;
  for (int k = threadIdx.x; k < nb; k += blockDim.x) t += part[k];
  t = warp_sum(t);
  if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = t;
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0.0;
    for (int w = 0; w < static_cast<int>(blockDim.x >> 5); ++w) a += ws[w];
    out[0] = a;
    out[1] = 0.0;
  }
}

}  // namespace fgb

using namespace fgb;

namespace {

// scratch vectors of one level in the V-cycle workspace (T: the V-cycle's
// arithmetic type)
template <typename T>
struct LevelVecs {
  T *r, *x, *x2, *d, *res;
};

size_t level_vec_bytes(int64_t n) { return 5 * align_up(static_cast<size_t>(n) * sizeof(double)); }

template <typename T>
LevelVecs<T> carve_level(Carver& cv, int64_t n) {
  LevelVecs<T> v;
  v.r = cv.take<T>(n);
  v.x = cv.take<T>(n);
  v.x2 = cv.take<T>(n);
  v.d = cv.take<T>(n);
  v.res = cv.take<T>(n);
  return v;
}

// a level's values and 1 / a_ii in the V-cycle's type
template <typename T>
const T* level_values(const fgb_amg_level& L) {
  if constexpr (std::is_same<T, float>::value) return L.values32;
  else return L.values;
}
template <typename T>
const T* level_dinv(const fgb_amg_level& L) {
  if constexpr (std::is_same<T, float>::value) return L.dinv32;
  else return L.dinv;
}

template <typename T>
void cheb_sweep(const fgb_amg_level& L, const T* r, const T* x_in, T* x_out, T* d, double c1, double c2,
                cudaStream_t st) {
  if (sell_sweep(L, level_dinv<T>(L), r, x_in, x_out, d, c1, c2, 0, st)) return;
  const int64_t n = L.n;
  const T* vals = level_values<T>(L);
  const T* dinv = level_dinv<T>(L);
  with_lanes(amg_lanes(n, L.nnz), [&](auto g) {
    constexpr int GG = decltype(g)::value;
    amg_cheb_step<GG, T, T><<<rows_grid(n, GG), kAmgThreads, 0, st>>>(n, L.indptr, L.indices, vals, dinv, r, x_in,
                                                                       x_out, d, static_cast<T>(c1),
                                                                       static_cast<T>(c2));
  });
}

// Chebyshev polynomial in D^-1 A of degree deg on [lmax * lo, lmax], applied
// to r from x = 0 (from_zero) or as a correction of the x in xa; the result
// ends in *xout (one of the two buffers).
template <typename T>
void cheb(const fgb_amg_level& L, const T* r, T* xa, T* xb, T* d, int deg, double lo, bool from_zero, T** xout,
          cudaStream_t st) {
  const int64_t n = L.n;
  const double lmax = L.lmax, lmin = L.lmax * lo;
  const double theta = 0.5 * (lmax + lmin), delta = 0.5 * (lmax - lmin), sigma = theta / delta;
  double rho = 1.0 / sigma;
  T* cur = xa;
  T* nxt = xb;
  int k = 0;
  if (from_zero) {
    amg_cheb_first<T><<<vec_grid(n), kAmgThreads, 0, st>>>(n, level_dinv<T>(L), r, cur, d,
                                                            static_cast<T>(1.0 / theta));
    k = 1;
  } else {
    // first correction of a given x: d = Dinv (r - A x) / theta
    cheb_sweep<T>(L, r, cur, nxt, d, 0.0, 1.0 / theta, st);
    T* t = cur;
    cur = nxt;
    nxt = t;
    k = 1;
  }
  for (; k < deg; ++k) {
    const double rho1 = 1.0 / (2.0 * sigma - rho);
    cheb_sweep<T>(L, r, cur, nxt, d, rho1 * rho, 2.0 * rho1 / delta, st);
    T* t = cur;
    cur = nxt;
    nxt = t;
    rho = rho1;
  }
  *xout = cur;
}

template <typename T>
int vcycle(const fgb_amg_level* levels, int nl, const double* r0, double* x_out, int deg, int cdeg, double omega,
           LevelVecs<T>* V, cudaStream_t st) {
  const int64_t n0 = levels[0].n;
  const T* r_top;
  if constexpr (std::is_same<T, float>::value) {
    amg_convert<double, float><<<vec_grid(n0), kAmgThreads, 0, st>>>(n0, r0, V[0].r);
    r_top = V[0].r;
  } else {
    r_top = r0;
  }
  // down: smoothing from zero, residual, restriction
  T* xs[FGB_AMG_MAX_LEVELS];
  const T* rin = r_top;
  for (int l = 0; l < nl; ++l) {
    const fgb_amg_level& L = levels[l];
    const int64_t n = L.n;
    if (l == nl - 1) {
      T* xo = nullptr;
      cheb<T>(L, rin, V[l].x, V[l].x2, V[l].d, cdeg, 0.05, true, &xo, st);
      xs[l] = xo;
      break;
    }
    T* xo = nullptr;
    cheb<T>(L, rin, V[l].x, V[l].x2, V[l].d, deg, 0.1, true, &xo, st);
    xs[l] = xo;
    const T* vals = level_values<T>(L);
    if (!sell_sweep(L, static_cast<const T*>(nullptr), rin, xo, V[l].res, static_cast<T*>(nullptr), 0.0, 0.0, 1, st))
      with_lanes(amg_lanes(n, L.nnz), [&](auto g) {
        constexpr int GG = decltype(g)::value;
        amg_residual<GG, T, T><<<rows_grid(n, GG), kAmgThreads, 0, st>>>(n, L.indptr, L.indices, vals, rin, xo,
                                                                          V[l].res);
      });
    amg_restrict<T><<<vec_grid(L.n_coarse), kAmgThreads, 0, st>>>(L.n_coarse, L.member_ptr, L.members, V[l].res,
                                                                  V[l + 1].r);
    rin = V[l + 1].r;
  }
  // up: prolongation with over-correction, smoothing of the corrected x
  for (int l = nl - 2; l >= 0; --l) {
    const fgb_amg_level& L = levels[l];
    const T* rl = l == 0 ? r_top : V[l].r;
    amg_prolong<T><<<vec_grid(L.n), kAmgThreads, 0, st>>>(L.n, L.agg, xs[l + 1], static_cast<T>(omega), xs[l]);
    T* other = xs[l] == V[l].x ? V[l].x2 : V[l].x;
    T* xo = nullptr;
    cheb<T>(L, rl, xs[l], other, V[l].d, deg, 0.1, false, &xo, st);
    xs[l] = xo;
  }
  if constexpr (std::is_same<T, float>::value) {
    amg_convert<float, double><<<vec_grid(n0), kAmgThreads, 0, st>>>(n0, xs[0], x_out);
    return launch_status();
  } else {
    return cudaMemcpyAsync(x_out, xs[0], n0 * sizeof(double), cudaMemcpyDeviceToDevice, st) == cudaSuccess
               ? launch_status()
               : FGB_ERR_CUDA;
  }
}

size_t vcycle_bytes(const fgb_amg_level* levels, int nl) {
  size_t b = 0;
  for (int l = 0; l < nl; ++l) b += level_vec_bytes(levels[l].n);
  return b;
}

// -1: inconsistent levels; 0: FP64 V-cycle; 1: FP32 V-cycle (every level
// carries values32 and dinv32)
int levels_mode(const fgb_amg_level* levels, int nl) {
  if (!levels || nl < 1 || nl > FGB_AMG_MAX_LEVELS) return -1;
  int n32 = 0;
  for (int l = 0; l < nl; ++l) {
    const fgb_amg_level& L = levels[l];
    if (L.n <= 0 || !L.indptr || !L.indices || !L.values || !L.dinv || !(L.lmax > 0.0)) return -1;
    if (l < nl - 1 && (!L.agg || !L.member_ptr || !L.members || L.n_coarse != levels[l + 1].n)) return -1;
    if ((L.values32 == nullptr) != (L.dinv32 == nullptr)) return -1;
    if (L.sell && L.sell->n != L.n) return -1;
    n32 += L.values32 ? 1 : 0;
  }
  if (n32 != 0 && n32 != nl) return -1;
  return n32 ? 1 : 0;
}

// the V-cycle's scratch in either type
struct VcycleScratch {
  int mode = 0;
  LevelVecs<float> f[FGB_AMG_MAX_LEVELS];
  LevelVecs<double> d[FGB_AMG_MAX_LEVELS];
  void carve(Carver& cv, const fgb_amg_level* levels, int nl) {
    for (int l = 0; l < nl; ++l) {
      if (mode) f[l] = carve_level<float>(cv, levels[l].n);
      else d[l] = carve_level<double>(cv, levels[l].n);
    }
  }
  int run(const fgb_amg_level* levels, int nl, const double* r, double* x, int deg, int cdeg, double omega,
          cudaStream_t st) {
    return mode ? vcycle<float>(levels, nl, r, x, deg, cdeg, omega, f, st)
                : vcycle<double>(levels, nl, r, x, deg, cdeg, omega, d, st);
  }
};

}  // namespace

extern "C" {

size_t fgb_amg_setup_workspace_bytes(int64_t n) {
  const size_t un = static_cast<size_t>(n);
  return align_up(un * 8) * 2 + align_up((un + 1) * 4) * 3 + align_up(8) + align_up(8) + align_up((un + 1) * 8) +
         scan_workspace_bytes(n + 1);
}

int32_t fgb_amg_aggregate(int64_t n, const int64_t* indptr, const int32_t* indices, const double* values,
                          double theta, int32_t* agg, int64_t* n_agg_host, double* dinv, double* lmax_host,
                          int32_t* status, void* workspace, size_t workspace_bytes, void* stream) {
  if (n <= 0 || !indptr || !indices || !values || !agg || !n_agg_host || !dinv || !lmax_host || !status ||
      !(theta >= 0.0))
    return FGB_ERR_ARG;
  if (n >= (int64_t(1) << 31)) return FGB_ERR_CAPACITY;
  if (!workspace || workspace_bytes < fgb_amg_setup_workspace_bytes(n)) return FGB_ERR_WORKSPACE;
  cudaStream_t st = as_stream(stream);
  Carver cv(workspace, workspace_bytes);
  double* diag = cv.take<double>(n);
  unsigned long long* key = cv.take<unsigned long long>(n);
  int32_t* state = cv.take<int32_t>(n + 1);
  int32_t* flag = cv.take<int32_t>(n + 1);
  int32_t* agg2 = cv.take<int32_t>(n + 1);
  unsigned long long* bound = cv.take<unsigned long long>(1);
  int32_t* counter = cv.take<int32_t>(2);
  int64_t* off = cv.take<int64_t>(n + 1);
  void* scan_ws = cv.base + cv.off;
  const size_t scan_bytes = workspace_bytes - cv.off;
  if (!cv.ok) return FGB_ERR_WORKSPACE;
  int64_t nnz = 0;
  if (cudaMemcpyAsync(&nnz, indptr + n, sizeof(int64_t), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return FGB_ERR_CUDA;
  if (nnz < 0) return FGB_ERR_ARG;
  const int G = amg_lanes(n, nnz);
  const int g = vec_grid(n);
  if (cudaMemsetAsync(bound, 0, sizeof(unsigned long long), st) != cudaSuccess) return FGB_ERR_CUDA;
  AMG_DISPATCH_ROWS(G, amg_diag_kernel, n, indptr, indices, values, diag, bound, status);
  amg_invert<<<g, kAmgThreads, 0, st>>>(n, diag, dinv);
  AMG_DISPATCH_ROWS(G, amg_init_state, n, indptr, indices, values, diag, theta, state);
  // maximal independent set (each round decides at least the undecided node
  // of largest key; 64 rounds bound the loop)
  int32_t und = 1;
  for (int round = 0; round < 64 && und > 0; ++round) {
    amg_keys<<<g, kAmgThreads, 0, st>>>(n, state, key);
    if (cudaMemsetAsync(counter, 0, sizeof(int32_t), st) != cudaSuccess) return FGB_ERR_CUDA;
    AMG_DISPATCH_ROWS(G, amg_mis_round, n, indptr, indices, values, diag, theta, key, state, counter);
    if (cudaMemcpyAsync(&und, counter, sizeof(int32_t), cudaMemcpyDeviceToHost, st) != cudaSuccess) return FGB_ERR_CUDA;
    if (cudaStreamSynchronize(st) != cudaSuccess) return FGB_ERR_CUDA;
  }
  if (und > 0) return FGB_ERR_CAPACITY;
  // roots numbered in index order
  amg_root_flags<<<g, kAmgThreads, 0, st>>>(n, state, flag);
  int rc = exclusive_scan_i32_to_i64(flag, n, off, scan_ws, scan_bytes, st);
  if (rc) return rc;
  int64_t nroot = 0;
  if (cudaMemcpyAsync(&nroot, off + n, sizeof(int64_t), cudaMemcpyDeviceToHost, st) != cudaSuccess) return FGB_ERR_CUDA;
  amg_root_ids<<<g, kAmgThreads, 0, st>>>(n, state, off, agg);
  // assignment sweeps (ping-pong between agg and agg2) until every node with
  // strong neighbours belongs to an aggregate
  int32_t left = 1;
  int32_t* cur = agg;
  int32_t* nxt = agg2;
  for (int sweep = 0; sweep < 8 && left > 0; ++sweep) {
    if (cudaMemsetAsync(counter, 0, sizeof(int32_t), st) != cudaSuccess) return FGB_ERR_CUDA;
    AMG_DISPATCH_ROWS(G, amg_assign, n, indptr, indices, values, diag, theta, state, cur, nxt, counter);
    if (cudaMemcpyAsync(&left, counter, sizeof(int32_t), cudaMemcpyDeviceToHost, st) != cudaSuccess)
      return FGB_ERR_CUDA;
    if (cudaStreamSynchronize(st) != cudaSuccess) return FGB_ERR_CUDA;
    int32_t* t = cur;
    cur = nxt;
    nxt = t;
  }
  if (left > 0) return FGB_ERR_CAPACITY;
  if (cur != agg && cudaMemcpyAsync(agg, cur, n * sizeof(int32_t), cudaMemcpyDeviceToDevice, st) != cudaSuccess)
    return FGB_ERR_CUDA;
  unsigned long long bbits = 0;
  if (cudaMemcpyAsync(&bbits, bound, sizeof(bbits), cudaMemcpyDeviceToHost, st) != cudaSuccess) return FGB_ERR_CUDA;
  if (cudaStreamSynchronize(st) != cudaSuccess) return FGB_ERR_CUDA;
  *n_agg_host = nroot;
  double b = 0.0;
  memcpy(&b, &bbits, sizeof(b));
  *lmax_host = b;
  return launch_status();
}

size_t fgb_amg_coarse_workspace_bytes(int64_t n, int64_t n_coarse) {
  const size_t c = static_cast<size_t>(n_coarse) + 1;
  (void)n;
  return align_up(c * 4) * 4 + align_up(4 * sizeof(int32_t)) + scan_workspace_bytes(n_coarse + 1);
}

namespace {

// Rows of the next level, count (mode 0, to rowcnt) or fill (mode 1): the
// warp path, its overflow by blocks, theirs by blocks with 128 KB of shared
// memory (above that: capacity error).
void coarse_rows(int64_t n, int mode, const int64_t* indptr, const int32_t* indices, const double* values,
                 const int32_t* agg, int64_t n_coarse, const int64_t* member_ptr, const int32_t* members,
                 int32_t* rowcnt, const int64_t* cptr, int32_t* ccol, double* cval, int32_t* ovf, int32_t* ovf2,
                 int32_t* lens, int32_t* status, cudaStream_t st) {
  amg_coarse_rows_warp<<<grid_for(n_coarse * 32, kWarpRowWarps * 32, kNumSMs * 16), kWarpRowWarps * 32, 0, st>>>(
      n, n_coarse, mode, indptr, indices, values, agg, member_ptr, members, rowcnt, cptr, ccol, cval, ovf, lens);
  amg_coarse_rows<<<kNumSMs * 2, kCoarseThreads, 0, st>>>(n, mode, indptr, indices, values, agg, member_ptr, members,
                                                          rowcnt, cptr, ccol, cval, ovf, lens, ovf2, lens + 1);
  const size_t big = static_cast<size_t>(kCoarseBigCap) * 16;
  cudaFuncSetAttribute(amg_coarse_rows_big, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(big));
  amg_coarse_rows_big<<<kNumSMs, kCoarseThreads, big, st>>>(n, mode, indptr, indices, values, agg, member_ptr,
                                                             members, rowcnt, cptr, ccol, cval, ovf2, lens + 1, status);
}

}  // namespace

int32_t fgb_amg_coarse_count(int64_t n, const int64_t* indptr, const int32_t* indices, const double* values,
                             const int32_t* agg, int64_t n_coarse, int64_t* member_ptr, int32_t* members,
                             int64_t* coarse_indptr, int64_t* nnz_host, int32_t* status, void* workspace,
                             size_t workspace_bytes, void* stream) {
  if (n <= 0 || n_coarse <= 0 || !indptr || !indices || !values || !agg || !member_ptr || !members ||
      !coarse_indptr || !nnz_host || !status)
    return FGB_ERR_ARG;
  if (n_coarse >= (int64_t(1) << 31)) return FGB_ERR_CAPACITY;
  if (!workspace || workspace_bytes < fgb_amg_coarse_workspace_bytes(n, n_coarse)) return FGB_ERR_WORKSPACE;
  cudaStream_t st = as_stream(stream);
  Carver cv(workspace, workspace_bytes);
  int32_t* cnt = cv.take<int32_t>(n_coarse + 1);
  int32_t* ovf = cv.take<int32_t>(n_coarse + 1);
  int32_t* ovf2 = cv.take<int32_t>(n_coarse + 1);
  int32_t* rowcnt = cv.take<int32_t>(n_coarse + 1);
  int32_t* lens = cv.take<int32_t>(4);
  void* scan_ws = cv.base + cv.off;
  const size_t scan_bytes = workspace_bytes - cv.off;
  if (!cv.ok) return FGB_ERR_WORKSPACE;
  if (cudaMemsetAsync(cnt, 0, (n_coarse + 1) * sizeof(int32_t), st) != cudaSuccess) return FGB_ERR_CUDA;
  amg_member_count<<<vec_grid(n), kAmgThreads, 0, st>>>(n, agg, cnt);
  int rc = exclusive_scan_i32_to_i64(cnt, n_coarse, member_ptr, scan_ws, scan_bytes, st);
  if (rc) return rc;
  if (cudaMemsetAsync(cnt, 0, (n_coarse + 1) * sizeof(int32_t), st) != cudaSuccess) return FGB_ERR_CUDA;
  amg_member_fill<<<vec_grid(n), kAmgThreads, 0, st>>>(n, agg, member_ptr, cnt, members);
  amg_member_sort<<<vec_grid(n_coarse), kAmgThreads, 0, st>>>(n_coarse, member_ptr, members);
  if (cudaMemsetAsync(lens, 0, 4 * sizeof(int32_t), st) != cudaSuccess) return FGB_ERR_CUDA;
  coarse_rows(n, 0, indptr, indices, values, agg, n_coarse, member_ptr, members, rowcnt, nullptr, nullptr, nullptr,
              ovf, ovf2, lens, status, st);
  rc = exclusive_scan_i32_to_i64(rowcnt, n_coarse, coarse_indptr, scan_ws, scan_bytes, st);
  if (rc) return rc;
  if (cudaMemcpyAsync(nnz_host, coarse_indptr + n_coarse, sizeof(int64_t), cudaMemcpyDeviceToHost, st) != cudaSuccess)
    return FGB_ERR_CUDA;
  if (cudaStreamSynchronize(st) != cudaSuccess) return FGB_ERR_CUDA;
  return launch_status();
}

int32_t fgb_amg_coarse_fill(int64_t n, const int64_t* indptr, const int32_t* indices, const double* values,
                            const int32_t* agg, int64_t n_coarse, const int64_t* member_ptr, const int32_t* members,
                            const int64_t* coarse_indptr, int32_t* coarse_indices, double* coarse_values,
                            int32_t* status, void* workspace, size_t workspace_bytes, void* stream) {
  if (n <= 0 || n_coarse <= 0 || !indptr || !indices || !values || !agg || !member_ptr || !members ||
      !coarse_indptr || !coarse_indices || !coarse_values || !status)
    return FGB_ERR_ARG;
  if (n_coarse >= (int64_t(1) << 31)) return FGB_ERR_CAPACITY;
  if (!workspace || workspace_bytes < fgb_amg_coarse_workspace_bytes(n, n_coarse)) return FGB_ERR_WORKSPACE;
  cudaStream_t st = as_stream(stream);
  Carver cv(workspace, workspace_bytes);
  int32_t* cnt = cv.take<int32_t>(n_coarse + 1);
  int32_t* ovf = cv.take<int32_t>(n_coarse + 1);
  int32_t* ovf2 = cv.take<int32_t>(n_coarse + 1);
  int32_t* rowcnt = cv.take<int32_t>(n_coarse + 1);
  int32_t* lens = cv.take<int32_t>(4);
  if (!cv.ok) return FGB_ERR_WORKSPACE;
  (void)cnt;
  if (cudaMemsetAsync(lens, 0, 4 * sizeof(int32_t), st) != cudaSuccess) return FGB_ERR_CUDA;
  coarse_rows(n, 1, indptr, indices, values, agg, n_coarse, member_ptr, members, rowcnt, coarse_indptr, coarse_indices,
              coarse_values, ovf, ovf2, lens, status, st);
  return launch_status();
}

size_t fgb_amg_workspace_bytes(const fgb_amg_level* levels, int32_t n_levels) {
  if (levels_mode(levels, n_levels) < 0) return 0;
  const int64_t n = levels[0].n;
  return vcycle_bytes(levels, n_levels) + 4 * align_up(static_cast<size_t>(n) * sizeof(double)) +
         align_up(2 * kMaxGrid * sizeof(double)) + align_up(sizeof(AmgPcgState)) + align_up(4 * sizeof(unsigned int));
}

int32_t fgb_amg_vcycle(const fgb_amg_level* levels, int32_t n_levels, int32_t deg, int32_t cdeg, double omega,
                       const double* r, double* x, void* workspace, size_t workspace_bytes, void* stream) {
  const int mode = levels_mode(levels, n_levels);
  if (mode < 0 || !r || !x || deg < 1 || cdeg < 1 || !(omega > 0.0)) return FGB_ERR_ARG;
  if (!workspace || workspace_bytes < fgb_amg_workspace_bytes(levels, n_levels)) return FGB_ERR_WORKSPACE;
  Carver cv(workspace, workspace_bytes);
  VcycleScratch V;
  V.mode = mode;
  V.carve(cv, levels, n_levels);
  if (!cv.ok) return FGB_ERR_WORKSPACE;
  return V.run(levels, n_levels, r, x, deg, cdeg, omega, as_stream(stream));
}

int32_t fgb_pcg_amg(const fgb_amg_level* levels, int32_t n_levels, int32_t deg, int32_t cdeg, double omega,
                    const double* b, double* x, double atol, double rtol, int64_t maxit, int32_t norm,
                    fgb_pcg_info* info, void* workspace, size_t workspace_bytes, void* stream) {
  const int mode = levels_mode(levels, n_levels);
  if (mode < 0 || !b || !x || deg < 1 || cdeg < 1 || !(omega > 0.0) || maxit <= 0) return FGB_ERR_ARG;
  if (!workspace || workspace_bytes < fgb_amg_workspace_bytes(levels, n_levels)) return FGB_ERR_WORKSPACE;
  cudaStream_t st = as_stream(stream);
  Carver cv(workspace, workspace_bytes);
  VcycleScratch V;
  V.mode = mode;
  V.carve(cv, levels, n_levels);
  const fgb_amg_level& L = levels[0];
  const int64_t n = L.n;
  double* r = cv.take<double>(n);
  double* z = cv.take<double>(n);
  double* p = cv.take<double>(n);
  double* Ap = cv.take<double>(n);
  double* partials = cv.take<double>(2 * kMaxGrid);
  AmgPcgState* s = cv.take<AmgPcgState>(1);
  unsigned int* counter = cv.take<unsigned int>(4);
  if (!cv.ok) return FGB_ERR_WORKSPACE;
  if (cudaMemsetAsync(counter, 0, 4 * sizeof(unsigned int), st) != cudaSuccess) return FGB_ERR_CUDA;
  const int G = amg_lanes(n, L.nnz);
  AmgPcgState h = {};
  auto read = [&]() -> int {
    if (cudaMemcpyAsync(&h, s, sizeof(h), cudaMemcpyDeviceToHost, st) != cudaSuccess) return FGB_ERR_CUDA;
    return cudaStreamSynchronize(st) == cudaSuccess ? FGB_OK : FGB_ERR_CUDA;
  };
  // kernels of one iteration: SpMV, update, the V-cycle, r.z, control, p
  int per_vcycle = mode ? 2 : 0;
  for (int l = 0; l < n_levels; ++l) per_vcycle += l == n_levels - 1 ? cdeg : 2 * deg + 3;
  const int64_t per_iter = 5 + per_vcycle;
  int64_t launches = 0;
  int reason = FGB_PCG_RUNNING;
  // ||b||, r = b - A x, z = M r, rz (host-synchronous, once)
  amg_dot2<<<kDotBlocks, kAmgThreads, 0, st>>>(n, b, b, partials, counter, s->red);
  int rc = read();
  if (rc) return rc;
  const double bnorm = sqrt(h.red[0]);
  if (bnorm < 1e-15) {
    if (cudaMemsetAsync(x, 0, n * sizeof(double), st) != cudaSuccess) return FGB_ERR_CUDA;
    reason = FGB_PCG_ZERO_RHS;
    h.niter = 0;
    h.resid = 0.0;
  } else {
    with_lanes(G, [&](auto g) {
      constexpr int GG = decltype(g)::value;
      amg_residual<GG, double, double><<<rows_grid(n, GG), kAmgThreads, 0, st>>>(n, L.indptr, L.indices, L.values, b,
                                                                                  x, r);
    });
    if ((rc = V.run(levels, n_levels, r, z, deg, cdeg, omega, st))) return rc;
    if (cudaMemcpyAsync(p, z, n * sizeof(double), cudaMemcpyDeviceToDevice, st) != cudaSuccess) return FGB_ERR_CUDA;
    amg_dot2<<<kDotBlocks, kAmgThreads, 0, st>>>(n, r, z, partials, counter, s->red + 4);
    if ((rc = read())) return rc;
    launches += 3 + per_vcycle;
    AmgPcgState init = {};
    init.rz = h.red[4];
    init.tol = rtol * bnorm;
    init.atol = atol;
    init.maxit = maxit;
    init.trip_cap = maxit + 1;
    init.norm = norm;
    if (cudaMemcpyAsync(s, &init, sizeof(init), cudaMemcpyHostToDevice, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
      return FGB_ERR_CUDA;
    // while (!done) { iteration } as one graph launch
    cudaGraph_t g = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaStream_t cs = nullptr;
    rc = FGB_OK;
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
      if (L.sell && L.sell->val64) {
        // the operator on the level's SELL copy: Ap and block partials of p.Ap
        int nb = 0;
        if ((rc = sell_spmv_pap_f64(L.sell, p, Ap, partials, &nb, cs)) != FGB_OK) {
          cudaGraph_t dummy = nullptr;
          cudaStreamEndCapture(cs, &dummy);
          break;
        }
        amg_sum_partials<<<1, 256, 0, cs>>>(partials, nb, s->red);
      } else {
        with_lanes(G, [&](auto gl) {
          constexpr int GG = decltype(gl)::value;
          amg_pcg_spmv<GG, double><<<rows_grid(n, GG), kAmgThreads, 0, cs>>>(n, L.indptr, L.indices, L.values, p,
                                                                              Ap, partials, counter, s->red);
        });
      }
      amg_pcg_update_dev<<<kDotBlocks, kAmgThreads, 0, cs>>>(n, s, p, Ap, x, r, partials, counter);
      const int vrc = V.run(levels, n_levels, r, z, deg, cdeg, omega, cs);
      amg_dot2<<<kDotBlocks, kAmgThreads, 0, cs>>>(n, r, z, partials, counter, s->red + 4);
      amg_pcg_ctl<<<1, 1, 0, cs>>>(s, hw);
      amg_pupdate_dev<<<vec_grid(n), kAmgThreads, 0, cs>>>(n, s, z, p);
      cudaGraph_t captured = nullptr;
      const bool ended = cudaStreamEndCapture(cs, &captured) == cudaSuccess;
      if (vrc || !ended) { rc = vrc ? vrc : FGB_ERR_CUDA; break; }
      if (cudaGraphInstantiate(&exec, g, 0) != cudaSuccess) { exec = nullptr; rc = FGB_ERR_CUDA; break; }
      if (cudaGraphLaunch(exec, st) != cudaSuccess) { rc = FGB_ERR_CUDA; break; }
      rc = read();
    } while (false);
    if (exec) cudaGraphExecDestroy(exec);
    if (g) cudaGraphDestroy(g);
    if (cs) cudaStreamDestroy(cs);
    if (rc) {
      cudaGetLastError();
      return rc;
    }
    reason = h.done;
    launches += per_iter * h.trips;
  }
  if (cudaStreamSynchronize(st) != cudaSuccess) return FGB_ERR_CUDA;
  if (info) {
    memset(info, 0, sizeof(*info));
    info->niter = h.niter;
    info->residual = h.resid;
    info->b_norm = bnorm;
    info->true_relres = -1.0;
    info->reason = reason;
    info->launches = launches;
    info->graph = reason == FGB_PCG_ZERO_RHS ? 0 : 1;
  }
  if (reason == FGB_PCG_BREAKDOWN) return FGB_ERR_BREAKDOWN;
  if (reason == FGB_PCG_NONFINITE) return FGB_ERR_NONFINITE;
  return launch_status();
}

}  // extern "C"
