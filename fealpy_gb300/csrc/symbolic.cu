// Symbolic phase of the assembly: dof->cell adjacency and the canonical CSR
// pattern, plus the int32->int64 exclusive scan they are built on.
//
// FEALPy builds the pattern by materialising every (row, col) COO pair of every
// cell (NC*ldof^2 pairs), lexsorting them and removing duplicates
// (fealpy/sparse/coo_tensor.py:184-213).  Here each row is produced by one
// warp from the cells around its dof: candidates are the dofs of those cells,
// sorted (bitonic, in shared memory) and de-duplicated.  That gives the same
// canonical (row-sorted, column-sorted, unique) pattern while reading only
// cell2dof and the adjacency.

#include "fgb_common.cuh"

#include <climits>

namespace fgb {

// ---------------------------------------------------------------------------
// scan
// ---------------------------------------------------------------------------
constexpr int kScanThreads = 256;
constexpr int kScanItems = 8;
constexpr int kScanTile = kScanThreads * kScanItems;

size_t scan_workspace_bytes(int64_t n) {
  int64_t tiles = (n + kScanTile - 1) / kScanTile + 1;
  return align_up(static_cast<size_t>(tiles) * sizeof(int64_t));
}

__global__ void scan_tile_sums(const int32_t* __restrict__ in, int64_t n, int64_t* __restrict__ tile_sum) {
  __shared__ int64_t red[kScanThreads / 32];
  const int64_t base = static_cast<int64_t>(blockIdx.x) * kScanTile;
  int64_t s = 0;
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    int64_t idx = base + static_cast<int64_t>(k) * kScanThreads + threadIdx.x;
    if (idx < n) s += in[idx];
  }
  s = block_sum(s, red);
  if (threadIdx.x == 0) tile_sum[blockIdx.x] = s;
}

// Single block: in-place exclusive scan of the tile sums; writes the total to *total.
__global__ void scan_tile_offsets(int64_t* __restrict__ tile_sum, int64_t n_tiles, int64_t* __restrict__ total) {
  __shared__ int64_t warp_tot[32];
  __shared__ int64_t carry_s;
  if (threadIdx.x == 0) carry_s = 0;
  __syncthreads();
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int64_t base = 0; base < n_tiles; base += blockDim.x) {
    int64_t idx = base + threadIdx.x;
    int64_t v = idx < n_tiles ? tile_sum[idx] : 0;
    int64_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int64_t y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) warp_tot[wid] = x;
    __syncthreads();
    if (wid == 0) {
      int nw = blockDim.x >> 5;
      int64_t w = lane < nw ? warp_tot[lane] : 0;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        int64_t y = __shfl_up_sync(0xffffffffu, w, o);
        if (lane >= o) w += y;
      }
      if (lane < nw) warp_tot[lane] = w;  // inclusive warp prefix
    }
    __syncthreads();
    int64_t warp_off = wid > 0 ? warp_tot[wid - 1] : 0;
    int64_t carry = carry_s;
    if (idx < n_tiles) tile_sum[idx] = carry + warp_off + x - v;
    __syncthreads();
    if (threadIdx.x == blockDim.x - 1) carry_s = carry + warp_off + x;
    __syncthreads();
  }
  if (threadIdx.x == 0) *total = carry_s;
}

__global__ void scan_tiles(const int32_t* __restrict__ in, int64_t n, const int64_t* __restrict__ tile_off,
                           int64_t* __restrict__ out) {
  __shared__ int64_t warp_tot[kScanThreads / 32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int64_t base = static_cast<int64_t>(blockIdx.x) * kScanTile + static_cast<int64_t>(threadIdx.x) * kScanItems;
  int64_t v[kScanItems];
  int64_t s = 0;
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    int64_t idx = base + k;
    v[k] = idx < n ? in[idx] : 0;
    s += v[k];
  }
  int64_t x = s;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int64_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp_tot[wid] = x;
  __syncthreads();
  if (wid == 0) {
    int64_t w = lane < (kScanThreads / 32) ? warp_tot[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int64_t y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += y;
    }
    if (lane < kScanThreads / 32) warp_tot[lane] = w;
  }
  __syncthreads();
  int64_t run = tile_off[blockIdx.x] + (wid > 0 ? warp_tot[wid - 1] : 0) + x - s;
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    int64_t idx = base + k;
    if (idx < n) out[idx] = run;
    run += v[k];
  }
}

int exclusive_scan_i32_to_i64(const int32_t* in, int64_t n, int64_t* out, void* ws, size_t ws_bytes,
                              cudaStream_t stream) {
  if (n < 0 || out == nullptr || (n > 0 && in == nullptr)) return FGB_ERR_ARG;
  if (ws == nullptr || ws_bytes < scan_workspace_bytes(n)) return FGB_ERR_WORKSPACE;
  int64_t n_tiles = (n + kScanTile - 1) / kScanTile;
  int64_t* tile_sum = static_cast<int64_t*>(ws);
  if (n_tiles > 0) scan_tile_sums<<<static_cast<unsigned>(n_tiles), kScanThreads, 0, stream>>>(in, n, tile_sum);
  scan_tile_offsets<<<1, 1024, 0, stream>>>(tile_sum, n_tiles, out + n);
  if (n_tiles > 0) scan_tiles<<<static_cast<unsigned>(n_tiles), kScanThreads, 0, stream>>>(in, n, tile_sum, out);
  return launch_status();
}

// ---------------------------------------------------------------------------
// adjacency: dof -> sorted list of packed (cell*ldof + local index)
// ---------------------------------------------------------------------------
__global__ void adjacency_count(const int32_t* __restrict__ c2d, int64_t total, int64_t n_dof,
                                int32_t* __restrict__ cnt, int32_t* status) {
  for (int64_t k = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; k < total;
       k += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    int32_t d = c2d[k];
    if (d < 0 || d >= n_dof) { set_status(status, FGB_ERR_INDEX); continue; }
    atomicAdd(cnt + d, 1);
  }
}

__global__ void adjacency_fill(const int32_t* __restrict__ c2d, int64_t total, int64_t n_dof,
                               const int64_t* __restrict__ adj_ptr, int32_t* __restrict__ cursor,
                               int32_t* __restrict__ adj) {
  for (int64_t k = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; k < total;
       k += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    int32_t d = c2d[k];
    if (d < 0 || d >= n_dof) continue;
    int32_t slot = atomicAdd(cursor + d, 1);
    adj[adj_ptr[d] + slot] = static_cast<int32_t>(k);
  }
}

// One warp per dof: sort its adjacency segment ascending (so contributions are
// later summed in cell order, like FEALPy's stable lexsort) and track the
// maximum degree.  Segments of <= 32 entries are sorted in registers by a warp
// bitonic network; longer ones (not produced by conforming simplex meshes of
// reasonable quality) by an insertion sort on lane 0.
__global__ void adjacency_sort(int64_t n_dof, const int64_t* __restrict__ adj_ptr, int32_t* __restrict__ adj,
                               int32_t* max_degree) {
  const int lane = threadIdx.x & 31;
  const int64_t warp = (blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x) >> 5;
  const int64_t nwarps = (static_cast<int64_t>(gridDim.x) * blockDim.x) >> 5;
  int32_t local_max = 0;
  for (int64_t i = warp; i < n_dof; i += nwarps) {
    const int64_t s = adj_ptr[i], e = adj_ptr[i + 1];
    const int len = static_cast<int>(e - s);
    local_max = max(local_max, len);
    if (len <= 1) continue;
    if (len <= 32) {
      int32_t v = lane < len ? adj[s + lane] : INT_MAX;
#pragma unroll
      for (int k = 2; k <= 32; k <<= 1) {
#pragma unroll
        for (int j = k >> 1; j > 0; j >>= 1) {
          int32_t o = __shfl_xor_sync(0xffffffffu, v, j);
          bool up = (lane & k) == 0;
          bool low = (lane & j) == 0;
          v = (low == up) ? min(v, o) : max(v, o);
        }
      }
      if (lane < len) adj[s + lane] = v;
    } else if (lane == 0) {
      for (int a = 1; a < len; ++a) {
        int32_t key = adj[s + a];
        int b = a - 1;
        while (b >= 0 && adj[s + b] > key) { adj[s + b + 1] = adj[s + b]; --b; }
        adj[s + b + 1] = key;
      }
    }
    __syncwarp();
  }
  if (lane == 0 && max_degree) atomicMax(max_degree, local_max);
}

// ---------------------------------------------------------------------------
// row pattern
// ---------------------------------------------------------------------------
constexpr int kPatWarps = 8;        // warps per block, first pass (hash set per warp)
constexpr int kPatBigCap = 8192;    // second pass (bitonic over all candidates), one warp per block (32 KB)

__device__ __forceinline__ int next_pow2(int x) {
  int p = 32;
  while (p < x) p <<= 1;
  return p;
}

// Processes row i with `cap` int32 slots of shared memory at `buf`.  Returns
// false (and does nothing) if the row has more candidates than `cap`.
// mode 0: write the number of unique columns to row_cnt[i]; mode 1: write the
// sorted unique columns to indices[indptr[i]...].
__device__ bool pattern_row(int64_t i, int mode, const int64_t* __restrict__ adj_ptr, const int32_t* __restrict__ adj,
                            const int32_t* __restrict__ c2d, int ldof, int32_t* __restrict__ row_cnt,
                            const int64_t* __restrict__ indptr, int32_t* __restrict__ indices, int32_t* buf, int cap) {
  const int lane = threadIdx.x & 31;
  const int64_t s = adj_ptr[i];
  const int deg = static_cast<int>(adj_ptr[i + 1] - s);
  const int m = deg * ldof;
  if (m > cap) return false;
  const int np2 = next_pow2(m > 0 ? m : 1);
  if (np2 > cap) {
    // pad area does not fit; treat as overflow so a larger pass handles it
    return false;
  }
  for (int t = lane; t < np2; t += 32) {
    int32_t v = INT_MAX;
    if (t < m) {
      int k = t / ldof, j = t - k * ldof;
      int32_t e = adj[s + k];
      int32_t c = e / ldof;
      v = c2d[static_cast<int64_t>(c) * ldof + j];
    }
    buf[t] = v;
  }
  __syncwarp();
  for (int k = 2; k <= np2; k <<= 1) {
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int t = lane; t < np2; t += 32) {
        int u = t ^ j;
        if (u > t) {
          int32_t a = buf[t], b = buf[u];
          bool up = (t & k) == 0;
          if ((a > b) == up) { buf[t] = b; buf[u] = a; }
        }
      }
      __syncwarp();
    }
  }
  int running = 0;
  const int64_t out0 = mode == 1 ? indptr[i] : 0;
  for (int base = 0; base < m; base += 32) {
    int t = base + lane;
    bool first = false;
    int32_t v = 0;
    if (t < m) {
      v = buf[t];
      first = (t == 0) || (buf[t - 1] != v);
    }
    unsigned ball = __ballot_sync(0xffffffffu, first);
    if (mode == 1 && first) {
      int rank = __popc(ball & ((1u << lane) - 1u));
      indices[out0 + running + rank] = v;
    }
    running += __popc(ball);
  }
  if (mode == 0 && lane == 0) row_cnt[i] = running;
  __syncwarp();
  return true;
}

// First-pass row builder: the candidates are inserted into a per-warp
// open-addressing hash set in shared memory (kHashSlots slots), the distinct
// columns are compacted and only those (at most kHashMaxUnique) are sorted.
// For a P2 tetrahedral row that is ~240 candidates but <= 65 distinct columns,
// so the sort is 4-8x smaller than sorting all candidates.  Returns false when
// the row has more distinct columns than kHashMaxUnique (the bitonic pass 2
// handles it).  The result does not depend on insertion order.
constexpr int kHashSlots = 256;
constexpr int kHashMaxUnique = 128;
static_assert(kHashMaxUnique >= kRowMapMax, "rows the numeric pass indexes directly must have positions");
static_assert(kHashMaxUnique <= 256, "positions are one byte");

// Ascending sort of one value per lane across the warp (bitonic network on
// registers, 15 shuffle steps).
__device__ __forceinline__ int32_t warp_sort32(int32_t v) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int k = 2; k <= 32; k <<= 1) {
#pragma unroll
    for (int j = k >> 1; j > 0; j >>= 1) {
      const int32_t o = __shfl_xor_sync(0xffffffffu, v, j);
      const bool up = (lane & k) == 0;
      const bool low = (lane & j) == 0;
      v = (low == up) ? min(v, o) : max(v, o);
    }
  }
  return v;
}

__device__ __forceinline__ unsigned hash8(int32_t v) { return (static_cast<unsigned>(v) * 2654435761u) >> 24; }

// slot of column v in a warp's hash set (v was inserted: linear probing from
// its hash meets v before any empty slot); -1 if absent
__device__ __forceinline__ int hash_slot(const int32_t* tab, int32_t v) {
  const unsigned h = hash8(v);
  for (int pr = 0; pr < kHashSlots; ++pr) {
    const int sl = static_cast<int>((h + pr) & (kHashSlots - 1));
    const int32_t t = tab[sl];
    if (t == v) return sl;
    if (t == -1) return -1;
  }
  return -1;
}

// pos[s * ldof + t] = rank of candidate t's column in the row (the hash set
// `tab` of the row and the slot -> rank map `rk` are complete)
__device__ __forceinline__ void row_positions(int64_t s, int m, int ldof, const int32_t* __restrict__ adj,
                                              const int32_t* __restrict__ c2d, const int32_t* tab, const uint8_t* rk,
                                              uint8_t* __restrict__ pos) {
  const int lane = threadIdx.x & 31;
  for (int t = lane; t < m; t += 32) {
    const int k = t / ldof, j = t - k * ldof;
    const int32_t c = adj[s + k] / ldof;
    const int32_t v = c2d[static_cast<int64_t>(c) * ldof + j];
    const int sl = hash_slot(tab, v);
    pos[s * ldof + t] = sl >= 0 ? rk[sl] : static_cast<uint8_t>(0xFF);
  }
}

// mode 0: count (row_cnt); 1: write the sorted row into indices at indptr[i];
// 2: count and stage the sorted row at stage[adj_ptr[i] * ldof] (its upper
// bound of entries), so that the values need no second pass.  With `pos`
// (mode 2), the position within the row of every candidate column is
// recorded as one byte at pos[adj_ptr[i] * ldof + t], t = k * ldof + j for
// local dof j of the row's k-th adjacent cell, so that the numeric assembly
// adds each contribution at a known slot instead of searching the row.  `rk`
// (kHashSlots bytes per warp) maps a hash slot to the rank of its column.
__device__ bool pattern_row_hash(int64_t i, int mode, const int64_t* __restrict__ adj_ptr,
                                 const int32_t* __restrict__ adj, const int32_t* __restrict__ c2d, int ldof,
                                 int32_t* __restrict__ row_cnt, const int64_t* __restrict__ indptr,
                                 int32_t* __restrict__ indices, int32_t* __restrict__ stage, int32_t* tab,
                                 int32_t* srt, uint8_t* __restrict__ pos, uint8_t* rk) {
  const int lane = threadIdx.x & 31;
  const int64_t s = adj_ptr[i];
  const int m = static_cast<int>(adj_ptr[i + 1] - s) * ldof;
  for (int t = lane; t < kHashSlots; t += 32) tab[t] = -1;
  __syncwarp();
  bool full = false;
  for (int base = 0; base < m; base += 32) {
    const int t = base + lane;
    if (t < m) {
      const int k = t / ldof, j = t - k * ldof;
      const int32_t c = adj[s + k] / ldof;
      const int32_t v = c2d[static_cast<int64_t>(c) * ldof + j];
      const unsigned h = hash8(v);
      int pr = 0;
      for (; pr < kHashSlots; ++pr) {
        const int32_t old = atomicCAS(tab + ((h + pr) & (kHashSlots - 1)), -1, v);
        if (old == -1 || old == v) break;
      }
      if (pr == kHashSlots) full = true;
    }
  }
  __syncwarp();
  if (__any_sync(0xffffffffu, full)) return false;
  int u = 0;
  for (int base = 0; base < kHashSlots; base += 32) {
    const int32_t v = tab[base + lane];
    const bool keep = v >= 0;
    const unsigned ball = __ballot_sync(0xffffffffu, keep);
    const int pos = u + __popc(ball & ((1u << lane) - 1u));
    if (keep && pos < kHashMaxUnique) srt[pos] = v;
    u += __popc(ball);
  }
  if (u > kHashMaxUnique) return false;
  if (u <= 32) {
    __syncwarp();
    const int32_t v = warp_sort32(lane < u ? srt[lane] : INT_MAX);
    if (mode == 0 || mode == 2) {
      if (lane == 0) row_cnt[i] = u;
    }
    if (mode == 1 && lane < u) indices[indptr[i] + lane] = v;
    if (mode == 2 && lane < u) stage[adj_ptr[i] * ldof + lane] = v;
    if (pos != nullptr && mode == 2) {
      if (lane < u) {
        const int sl = hash_slot(tab, v);
        if (sl >= 0) rk[sl] = static_cast<uint8_t>(lane);
      }
      __syncwarp();
      row_positions(s, m, ldof, adj, c2d, tab, rk, pos);
    }
    __syncwarp();
    return true;
  }
  const int np2 = next_pow2(u > 0 ? u : 1);
  for (int t = u + lane; t < np2; t += 32) srt[t] = INT_MAX;
  __syncwarp();
  for (int k = 2; k <= np2; k <<= 1) {
    for (int jj = k >> 1; jj > 0; jj >>= 1) {
      for (int t = lane; t < np2; t += 32) {
        const int w = t ^ jj;
        if (w > t) {
          const int32_t a = srt[t], b = srt[w];
          const bool up = (t & k) == 0;
          if ((a > b) == up) { srt[t] = b; srt[w] = a; }
        }
      }
      __syncwarp();
    }
  }
  if (mode == 0 || mode == 2) {
    if (lane == 0) row_cnt[i] = u;
  }
  if (mode == 1) {
    const int64_t out0 = indptr[i];
    for (int t = lane; t < u; t += 32) indices[out0 + t] = srt[t];
  } else if (mode == 2) {
    const int64_t out0 = adj_ptr[i] * ldof;
    for (int t = lane; t < u; t += 32) stage[out0 + t] = srt[t];
    if (pos != nullptr) {
      for (int t = lane; t < u; t += 32) {
        const int sl = hash_slot(tab, srt[t]);
        if (sl >= 0) rk[sl] = static_cast<uint8_t>(t);
      }
      __syncwarp();
      row_positions(s, m, ldof, adj, c2d, tab, rk, pos);
    }
  }
  __syncwarp();
  return true;
}

__global__ void __launch_bounds__(kPatWarps * 32) pattern_pass1(int64_t n_dof, int mode, const int64_t* __restrict__ adj_ptr,
                                                                const int32_t* __restrict__ adj, const int32_t* __restrict__ c2d,
                                                                int ldof, int32_t* __restrict__ row_cnt,
                                                                const int64_t* __restrict__ indptr, int32_t* __restrict__ indices,
                                                                int32_t* __restrict__ ovf, int32_t* __restrict__ ovf_len,
                                                                int32_t* __restrict__ stage, uint8_t* __restrict__ pos) {
  __shared__ int32_t stab[kPatWarps * kHashSlots];
  __shared__ int32_t ssrt[kPatWarps * kHashMaxUnique];
  __shared__ uint8_t srk[kPatWarps * kHashSlots];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  int32_t* tab = stab + wib * kHashSlots;
  int32_t* srt = ssrt + wib * kHashMaxUnique;
  uint8_t* rk = srk + wib * kHashSlots;
  const int64_t warp = (blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x) >> 5;
  const int64_t nwarps = (static_cast<int64_t>(gridDim.x) * blockDim.x) >> 5;
  for (int64_t i = warp; i < n_dof; i += nwarps) {
    bool done = pattern_row_hash(i, mode, adj_ptr, adj, c2d, ldof, row_cnt, indptr, indices, stage, tab, srt, pos, rk);
    if (!done && lane == 0) {
      int slot = atomicAdd(ovf_len, 1);
      ovf[slot] = static_cast<int32_t>(i);
      if (mode == 2) stage[adj_ptr[i] * ldof] = -1;  // this row is not staged: pass 2 writes it
    }
  }
}

// Staged rows -> indices (warp per row); rows marked -1 are left to pass 2.
__global__ void pattern_compact(int64_t n_dof, const int64_t* __restrict__ adj_ptr, int ldof,
                                const int64_t* __restrict__ indptr, const int32_t* __restrict__ stage,
                                int32_t* __restrict__ indices) {
  const int lane = threadIdx.x & 31;
  const int64_t warp = (blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x) >> 5;
  const int64_t nwarps = (static_cast<int64_t>(gridDim.x) * blockDim.x) >> 5;
  for (int64_t i = warp; i < n_dof; i += nwarps) {
    const int64_t o = indptr[i];
    const int len = static_cast<int>(indptr[i + 1] - o);
    const int64_t src = adj_ptr[i] * ldof;
    if (len == 0 || stage[src] < 0) continue;  // empty row (no staged slot to read) / row left to pass 2
    for (int t = lane; t < len; t += 32) indices[o + t] = stage[src + t];
  }
}

__global__ void pattern_pass2(int mode, const int64_t* __restrict__ adj_ptr, const int32_t* __restrict__ adj,
                              const int32_t* __restrict__ c2d, int ldof, int32_t* __restrict__ row_cnt,
                              const int64_t* __restrict__ indptr, int32_t* __restrict__ indices,
                              const int32_t* __restrict__ ovf, const int32_t* __restrict__ ovf_len, int32_t* status) {
  extern __shared__ int32_t dbuf[];
  const int n = *ovf_len;
  for (int r = blockIdx.x; r < n; r += gridDim.x) {
    int64_t i = ovf[r];
    bool done = pattern_row(i, mode, adj_ptr, adj, c2d, ldof, row_cnt, indptr, indices, dbuf, kPatBigCap);
    if (!done && (threadIdx.x & 31) == 0) set_status(status, FGB_ERR_CAPACITY);
  }
}

// Expand a scalar node pattern to bs x bs blocks.
__global__ void expand_blocks_indptr(int64_t n_node, int bs, int dof_priority, const int64_t* __restrict__ indptr,
                                     int64_t* __restrict__ out) {
  const int64_t nnz_s = indptr[n_node];
  for (int64_t r = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; r <= n_node * bs;
       r += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    if (r == n_node * bs) { out[r] = nnz_s * bs * bs; continue; }
    int64_t node, comp;
    if (dof_priority) { comp = r / n_node; node = r - comp * n_node; }
    else { node = r / bs; comp = r - node * bs; }
    int64_t len = indptr[node + 1] - indptr[node];
    int64_t start;
    if (dof_priority) start = comp * nnz_s * bs + indptr[node] * bs;
    else start = indptr[node] * bs * bs + comp * len * bs;
    out[r] = start;
  }
}

__global__ void expand_blocks_indices(int64_t n_node, int bs, int dof_priority, const int64_t* __restrict__ indptr,
                                      const int32_t* __restrict__ indices, const int64_t* __restrict__ out_indptr,
                                      int32_t* __restrict__ out) {
  const int lane = threadIdx.x & 31;
  const int64_t warp = (blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x) >> 5;
  const int64_t nwarps = (static_cast<int64_t>(gridDim.x) * blockDim.x) >> 5;
  for (int64_t r = warp; r < n_node * bs; r += nwarps) {
    int64_t node = dof_priority ? (r % n_node) : (r / bs);
    const int64_t s = indptr[node];
    const int64_t len = indptr[node + 1] - s;
    const int64_t o = out_indptr[r];
    for (int64_t t = lane; t < len * bs; t += 32) {
      int64_t k, b;
      if (dof_priority) { b = t / len; k = t - b * len; }
      else { k = t / bs; b = t - k * bs; }
      int64_t j = indices[s + k];
      out[o + t] = static_cast<int32_t>(dof_priority ? b * n_node + j : j * bs + b);
    }
  }
}

}  // namespace fgb

using namespace fgb;

extern "C" {

size_t fgb_scan_workspace_bytes(int64_t n) { return scan_workspace_bytes(n); }

int32_t fgb_exclusive_scan_i32(const int32_t* in, int64_t n, int64_t* out, void* workspace,
                               size_t workspace_bytes, void* stream) {
  return exclusive_scan_i32_to_i64(in, n, out, workspace, workspace_bytes, as_stream(stream));
}

size_t fgb_adjacency_workspace_bytes(int64_t n_dof) {
  return align_up(static_cast<size_t>(n_dof) * sizeof(int32_t)) + scan_workspace_bytes(n_dof);
}

int32_t fgb_adjacency_build(int64_t n_cell, int32_t ldof, const int32_t* cell2dof, int64_t n_dof, int64_t* adj_ptr,
                            int32_t* adj, int32_t* max_degree, int32_t* status, void* workspace,
                            size_t workspace_bytes, void* stream) {
  if (n_cell < 0 || ldof <= 0 || n_dof <= 0 || adj_ptr == nullptr) return FGB_ERR_ARG;
  if (n_cell > 0 && (cell2dof == nullptr || adj == nullptr)) return FGB_ERR_ARG;
  if (n_cell * static_cast<int64_t>(ldof) >= (int64_t(1) << 31)) return FGB_ERR_CAPACITY;
  if (n_dof >= (int64_t(1) << 31)) return FGB_ERR_CAPACITY;
  if (workspace_bytes < fgb_adjacency_workspace_bytes(n_dof) || workspace == nullptr) return FGB_ERR_WORKSPACE;
  cudaStream_t st = as_stream(stream);
  Carver cv(workspace, workspace_bytes);
  int32_t* cnt = cv.take<int32_t>(n_dof);
  void* scan_ws = cv.base + cv.off;
  size_t scan_bytes = workspace_bytes - cv.off;
  const int64_t total = n_cell * ldof;
  cudaMemsetAsync(cnt, 0, n_dof * sizeof(int32_t), st);
  if (max_degree) cudaMemsetAsync(max_degree, 0, sizeof(int32_t), st);
  if (total > 0) adjacency_count<<<grid_for(total, 256, kNumSMs * 16), 256, 0, st>>>(cell2dof, total, n_dof, cnt, status);
  int rc = exclusive_scan_i32_to_i64(cnt, n_dof, adj_ptr, scan_ws, scan_bytes, st);
  if (rc != FGB_OK) return rc;
  cudaMemsetAsync(cnt, 0, n_dof * sizeof(int32_t), st);
  if (total > 0) adjacency_fill<<<grid_for(total, 256, kNumSMs * 16), 256, 0, st>>>(cell2dof, total, n_dof, adj_ptr, cnt, adj);
  adjacency_sort<<<grid_for(n_dof * 32, 256, kNumSMs * 16), 256, 0, st>>>(n_dof, adj_ptr, adj, max_degree);
  return launch_status();
}

size_t fgb_pattern_workspace_bytes(int64_t n_dof) {
  return align_up(static_cast<size_t>(n_dof) * sizeof(int32_t)) * 2 + align_up(sizeof(int32_t)) +
         scan_workspace_bytes(n_dof);
}

static int pattern_launch(int mode, int64_t n_dof, const int64_t* adj_ptr, const int32_t* adj, const int32_t* c2d,
                          int32_t ldof, int32_t* row_cnt, const int64_t* indptr, int32_t* indices, int32_t* ovf,
                          int32_t* ovf_len, int32_t* status, cudaStream_t st) {
  cudaMemsetAsync(ovf_len, 0, sizeof(int32_t), st);
  pattern_pass1<<<grid_for(n_dof * 32, kPatWarps * 32, kNumSMs * 8), kPatWarps * 32, 0, st>>>(
      n_dof, mode, adj_ptr, adj, c2d, ldof, row_cnt, indptr, indices, ovf, ovf_len, nullptr, nullptr);
  cudaFuncSetAttribute(pattern_pass2, cudaFuncAttributeMaxDynamicSharedMemorySize, kPatBigCap * 4);
  pattern_pass2<<<kNumSMs, 32, kPatBigCap * 4, st>>>(mode, adj_ptr, adj, c2d, ldof, row_cnt, indptr, indices, ovf,
                                                     ovf_len, status);
  return launch_status();
}

int32_t fgb_pattern_count(int64_t n_dof, const int64_t* adj_ptr, const int32_t* adj, const int32_t* cell2dof,
                          int32_t ldof, int64_t* indptr, int32_t* status, void* workspace, size_t workspace_bytes,
                          void* stream) {
  if (n_dof <= 0 || ldof <= 0 || adj_ptr == nullptr || indptr == nullptr || adj == nullptr || cell2dof == nullptr)
    return FGB_ERR_ARG;
  if (workspace == nullptr || workspace_bytes < fgb_pattern_workspace_bytes(n_dof)) return FGB_ERR_WORKSPACE;
  cudaStream_t st = as_stream(stream);
  Carver cv(workspace, workspace_bytes);
  int32_t* cnt = cv.take<int32_t>(n_dof);
  int32_t* ovf = cv.take<int32_t>(n_dof);
  int32_t* ovf_len = cv.take<int32_t>(1);
  void* scan_ws = cv.base + cv.off;
  size_t scan_bytes = workspace_bytes - cv.off;
  cudaMemsetAsync(cnt, 0, n_dof * sizeof(int32_t), st);
  int rc = pattern_launch(0, n_dof, adj_ptr, adj, cell2dof, ldof, cnt, nullptr, nullptr, ovf, ovf_len, status, st);
  if (rc != FGB_OK) return rc;
  return exclusive_scan_i32_to_i64(cnt, n_dof, indptr, scan_ws, scan_bytes, st);
}

int32_t fgb_pattern_fill(int64_t n_dof, const int64_t* adj_ptr, const int32_t* adj, const int32_t* cell2dof,
                         int32_t ldof, const int64_t* indptr, int32_t* indices, int32_t* status, void* workspace,
                         size_t workspace_bytes, void* stream) {
  if (n_dof <= 0 || ldof <= 0 || adj_ptr == nullptr || indptr == nullptr || indices == nullptr || adj == nullptr ||
      cell2dof == nullptr)
    return FGB_ERR_ARG;
  if (workspace == nullptr || workspace_bytes < fgb_pattern_workspace_bytes(n_dof)) return FGB_ERR_WORKSPACE;
  cudaStream_t st = as_stream(stream);
  Carver cv(workspace, workspace_bytes);
  cv.take<int32_t>(n_dof);
  int32_t* ovf = cv.take<int32_t>(n_dof);
  int32_t* ovf_len = cv.take<int32_t>(1);
  return pattern_launch(1, n_dof, adj_ptr, adj, cell2dof, ldof, nullptr, indptr, indices, ovf, ovf_len, status, st);
}

int32_t fgb_pattern_build(int64_t n_dof, const int64_t* adj_ptr, const int32_t* adj, const int32_t* cell2dof,
                          int32_t ldof, int64_t n_adj, int64_t* indptr, int32_t* stage, size_t stage_bytes,
                          uint8_t* positions, int32_t* status, void* workspace, size_t workspace_bytes,
                          void* stream) {
  if (n_dof <= 0 || ldof <= 0 || n_adj <= 0 || !adj_ptr || !adj || !cell2dof || !indptr || !stage) return FGB_ERR_ARG;
  if (stage_bytes < static_cast<size_t>(n_adj) * ldof * sizeof(int32_t)) return FGB_ERR_WORKSPACE;
  if (workspace == nullptr || workspace_bytes < fgb_pattern_workspace_bytes(n_dof)) return FGB_ERR_WORKSPACE;
  cudaStream_t st = as_stream(stream);
  Carver cv(workspace, workspace_bytes);
  int32_t* cnt = cv.take<int32_t>(n_dof);
  int32_t* ovf = cv.take<int32_t>(n_dof);
  int32_t* ovf_len = cv.take<int32_t>(1);
  void* scan_ws = cv.base + cv.off;
  size_t scan_bytes = workspace_bytes - cv.off;
  cudaMemsetAsync(ovf_len, 0, sizeof(int32_t), st);
  pattern_pass1<<<grid_for(n_dof * 32, kPatWarps * 32, kNumSMs * 8), kPatWarps * 32, 0, st>>>(
      n_dof, 2, adj_ptr, adj, cell2dof, ldof, cnt, nullptr, nullptr, ovf, ovf_len, stage, positions);
  cudaFuncSetAttribute(pattern_pass2, cudaFuncAttributeMaxDynamicSharedMemorySize, kPatBigCap * 4);
  pattern_pass2<<<kNumSMs, 32, kPatBigCap * 4, st>>>(0, adj_ptr, adj, cell2dof, ldof, cnt, nullptr, nullptr, ovf,
                                                     ovf_len, status);
  const int rc = launch_status();
  if (rc != FGB_OK) return rc;
  return exclusive_scan_i32_to_i64(cnt, n_dof, indptr, scan_ws, scan_bytes, st);
}

int32_t fgb_pattern_compact(int64_t n_dof, const int64_t* adj_ptr, const int32_t* adj, const int32_t* cell2dof,
                            int32_t ldof, const int64_t* indptr, const int32_t* stage, int32_t* indices,
                            int32_t* status, void* workspace, size_t workspace_bytes, void* stream) {
  if (n_dof <= 0 || ldof <= 0 || !adj_ptr || !adj || !cell2dof || !indptr || !stage || !indices) return FGB_ERR_ARG;
  if (workspace == nullptr || workspace_bytes < fgb_pattern_workspace_bytes(n_dof)) return FGB_ERR_WORKSPACE;
  cudaStream_t st = as_stream(stream);
  Carver cv(workspace, workspace_bytes);
  cv.take<int32_t>(n_dof);
  int32_t* ovf = cv.take<int32_t>(n_dof);
  int32_t* ovf_len = cv.take<int32_t>(1);
  pattern_compact<<<grid_for(n_dof * 32, 256, kNumSMs * 16), 256, 0, st>>>(n_dof, adj_ptr, ldof, indptr, stage,
                                                                          indices);
  // rows that did not fit the hash pass (listed by fgb_pattern_build in the same workspace)
  cudaFuncSetAttribute(pattern_pass2, cudaFuncAttributeMaxDynamicSharedMemorySize, kPatBigCap * 4);
  pattern_pass2<<<kNumSMs, 32, kPatBigCap * 4, st>>>(1, adj_ptr, adj, cell2dof, ldof, nullptr, indptr, indices, ovf,
                                                     ovf_len, status);
  return launch_status();
}

int32_t fgb_pattern_expand_blocks(int64_t n_node, int32_t bs, int32_t dof_priority, const int64_t* indptr,
                                  const int32_t* indices, int64_t* out_indptr, int32_t* out_indices, void* stream) {
  if (n_node <= 0 || bs <= 0 || indptr == nullptr || out_indptr == nullptr) return FGB_ERR_ARG;
  if (n_node * bs >= (int64_t(1) << 31)) return FGB_ERR_CAPACITY;
  cudaStream_t st = as_stream(stream);
  expand_blocks_indptr<<<grid_for(n_node * bs + 1, 256, kNumSMs * 16), 256, 0, st>>>(n_node, bs, dof_priority, indptr,
                                                                                    out_indptr);
  if (out_indices != nullptr && indices != nullptr)
    expand_blocks_indices<<<grid_for(n_node * bs * 32, 256, kNumSMs * 16), 256, 0, st>>>(
        n_node, bs, dof_priority, indptr, indices, out_indptr, out_indices);
  return launch_status();
}

}  // extern "C"
