// Delta-coded SELL copy (2-byte column steps) and the renumbering it needs.
//
// Why: the FP32 SpMV streams 4 bytes of value and 4 bytes of column per
// nonzero; with 2-byte column steps it streams 6.  The steps are small only
// when every row's columns lie close together, which FEALPy's dof numbering
// (all vertex dofs, then all edge dofs, then faces, then cells) does not give:
// a vertex row reaches from the vertex block into the edge block.  Sorting the
// rows by their smallest column (ties by row) interleaves the blocks by
// location: every edge, face or cell dof lands next to the lowest vertex it
// couples to.  The solve then runs on P A P^T with b, x and the inverse
// diagonal permuted alike; the result is permuted back.
//
// Construction (all on the device, deterministic):
//   renumber     with the dof blocks of the space (vertex, edge, face, cell
//                dofs; per component for vector spaces): a stable merge of
//                the blocks by relative position, key(i) = floor(i_rel *
//                n_0 / n_b), which puts every edge/face/cell dof next to the
//                vertex dofs of the same region (FEALPy numbers entities by
//                their vertices); closed form, no sort.  Without blocks: keys
//                = smallest column per row; counting sort by key, each key
//                group sorted by row (a group above 64 rows makes the whole
//                order the identity)
//   csr_permute  rows in the new order, columns mapped and sorted (rank sort
//                by a warp per row, staged in shared memory)
//   d16_indptr   row lengths with the bridge entries for steps above 65535
//   fill_d16     per slot the first column, per entry the step and the value

#include "fgb_common.cuh"
#include "sell_rows.cuh"

namespace fgb {

constexpr int kGroupMax = 64;     // largest key group sorted in place
constexpr int kMaxBlocks = 16;    // dof blocks of the block-merge order

struct DofBlocks {
  int n;
  int64_t start[kMaxBlocks + 1];
};

// Rows of block b (relative index j) whose key is below k: key(j) =
// floor(j * n0 / nb) < k  <=>  j < ceil(k * nb / n0).
__device__ __forceinline__ int64_t keys_below(int64_t k, int64_t nb, int64_t n0) {
  const int64_t c = (k * nb + n0 - 1) / n0;
  return c < nb ? c : nb;
}

// Stable merge of the blocks by key: row i (block b, relative index j, key k)
// goes to j + sum_{b' < b} |{key <= k} in b'| + sum_{b' > b} |{key < k} in b'|.
__global__ void renumber_blocks(int64_t n, DofBlocks B, int32_t* __restrict__ order, int32_t* __restrict__ inv) {
  const int64_t n0 = B.start[1] - B.start[0];
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    int b = 0;
    while (b + 1 < B.n && i >= B.start[b + 1]) ++b;
    const int64_t nb = B.start[b + 1] - B.start[b];
    const int64_t j = i - B.start[b];
    const int64_t k = (j * n0) / nb;
    int64_t pos = j;
    for (int q = 0; q < B.n; ++q) {
      if (q == b) continue;
      const int64_t nq = B.start[q + 1] - B.start[q];
      pos += keys_below(q < b ? k + 1 : k, nq, n0);
    }
    order[pos] = static_cast<int32_t>(i);
    inv[i] = static_cast<int32_t>(pos);
  }
}

constexpr int kPermWarps = 4;     // warps per block of the row permutation
constexpr int kPermStage = 1024;  // row entries staged in shared memory per warp

// smallest column of every row (the row itself when it is empty)
__global__ void renumber_keys(int64_t n, const int64_t* __restrict__ indptr, const int32_t* __restrict__ indices,
                              int32_t* __restrict__ key, int32_t* __restrict__ cnt) {
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int64_t a = indptr[i], b = indptr[i + 1];
    int32_t k = static_cast<int32_t>(i);
    for (int64_t e = a; e < b; ++e) {
      const int32_t c = indices[e];
      if (c < k && c >= 0) k = c;
    }
    key[i] = k;
    atomicAdd(cnt + k, 1);
  }
}

// order[start[key] + t] = row, t taken by atomic (sorted per group next)
__global__ void renumber_place(int64_t n, const int32_t* __restrict__ key, const int64_t* __restrict__ start,
                               int32_t* __restrict__ fill, int32_t* __restrict__ order) {
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int32_t k = key[i];
    const int t = atomicAdd(fill + k, 1);
    order[start[k] + t] = static_cast<int32_t>(i);
  }
}

// each key group in ascending row order (insertion sort; groups are small)
__global__ void renumber_sort_groups(int64_t n, const int64_t* __restrict__ start, int32_t* __restrict__ order,
                                     int32_t* __restrict__ too_big) {
  for (int64_t k = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; k < n;
       k += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int64_t a = start[k];
    const int m = static_cast<int>(start[k + 1] - a);
    if (m <= 1) continue;
    if (m > kGroupMax) {
      atomicMax(too_big, 1);
      continue;
    }
    int32_t v[kGroupMax];
    for (int t = 0; t < m; ++t) {
      const int32_t x = order[a + t];
      int u = t;
      while (u > 0 && v[u - 1] > x) {
        v[u] = v[u - 1];
        --u;
      }
      v[u] = x;
    }
    for (int t = 0; t < m; ++t) order[a + t] = v[t];
  }
}

__global__ void renumber_inverse(int64_t n, int32_t* __restrict__ order, int32_t* __restrict__ inv,
                                 const int32_t* __restrict__ too_big) {
  const bool identity = *too_big != 0;
  for (int64_t k = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; k < n;
       k += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    if (identity) {
      order[k] = static_cast<int32_t>(k);
      inv[k] = static_cast<int32_t>(k);
    } else {
      inv[order[k]] = static_cast<int32_t>(k);
    }
  }
}

__global__ void permuted_lengths(int64_t n, const int64_t* __restrict__ indptr, const int32_t* __restrict__ order,
                                 int32_t* __restrict__ len) {
  for (int64_t k = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; k < n;
       k += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int32_t o = order[k];
    len[k] = static_cast<int32_t>(indptr[o + 1] - indptr[o]);
  }
}

// Row k of P A P^T: row order[k] of A with columns inv[col], in ascending
// order.  A warp per row; the rank of an entry is the number of entries with a
// smaller column (equal columns by position, so that duplicates keep distinct
// slots).  Rows longer than the shared-memory stage read the mapped columns
// from global memory instead.
__global__ void __launch_bounds__(kPermWarps * 32) csr_permute_fill(
    int64_t n, const int64_t* __restrict__ indptr, const int32_t* __restrict__ indices,
    const double* __restrict__ v64, const float* __restrict__ v32, const int32_t* __restrict__ order,
    const int32_t* __restrict__ inv, const int64_t* __restrict__ new_indptr, int32_t* __restrict__ new_indices,
    double* __restrict__ new_v64, float* __restrict__ new_v32) {
  __shared__ int32_t stage[kPermWarps][kPermStage];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  int32_t* sc = stage[wib];
  const int64_t warp = (blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x) >> 5;
  const int64_t nwarps = (static_cast<int64_t>(gridDim.x) * blockDim.x) >> 5;
  for (int64_t k = warp; k < n; k += nwarps) {
    const int32_t o = order[k];
    const int64_t rs = indptr[o];
    const int len = static_cast<int>(indptr[o + 1] - rs);
    const int64_t dst = new_indptr[k];
    const bool staged = len <= kPermStage;
    if (staged)
      for (int e = lane; e < len; e += 32) sc[e] = inv[indices[rs + e]];
    __syncwarp();
    for (int e = lane; e < len; e += 32) {
      const int32_t c = staged ? sc[e] : inv[indices[rs + e]];
      int rank = 0;
      for (int j = 0; j < len; ++j) {
        const int32_t q = staged ? sc[j] : inv[indices[rs + j]];
        rank += (q < c || (q == c && j < e)) ? 1 : 0;
      }
      new_indices[dst + rank] = c;
      if (new_v64) new_v64[dst + rank] = v64 ? v64[rs + e] : static_cast<double>(v32[rs + e]);
      if (new_v32) new_v32[dst + rank] = v32 ? v32[rs + e] : static_cast<float>(v64[rs + e]);
    }
    __syncwarp();
  }
}

// entries of a row in the delta-coded copy: its entries plus one zero-valued
// bridge per 65535 of every step above 65535 (columns ascending)
__global__ void d16_lengths(int64_t n, const int64_t* __restrict__ indptr, const int32_t* __restrict__ indices,
                            int32_t* __restrict__ len) {
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int64_t a = indptr[i], b = indptr[i + 1];
    int64_t m = b - a;
    for (int64_t e = a + 1; e < b; ++e) {
      const int64_t step = static_cast<int64_t>(indices[e]) - indices[e - 1];
      if (step > 65535) m += (step - 1) / 65535;
    }
    len[i] = static_cast<int32_t>(m);
  }
}

// Lane per slot, as the 4-byte fill: the slot's row written entry by entry,
// bridges inserted, zero steps and values up to the slice width.
__global__ void sell_fill_d16_kernel(int64_t n_slices, const int64_t* __restrict__ slice_ptr,
                                     const int32_t* __restrict__ perm, const int64_t* __restrict__ indptr,
                                     const int32_t* __restrict__ indices, const double* __restrict__ v64,
                                     const float* __restrict__ v32, int32_t* __restrict__ col0,
                                     uint16_t* __restrict__ col16, double* __restrict__ s64,
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
    if (row >= 0) {
      rs = indptr[row];
      len = static_cast<int>(indptr[row + 1] - rs);
    }
    int32_t c = len > 0 ? indices[rs] : (row >= 0 ? row : 0);
    col0[s * kSellC + lane] = c;
    int k = 0;
    auto put = [&](uint32_t step, double a, float b) {
      if (k >= w) return;  // cannot happen: the plan's width covers the bridged length
      const int64_t pos = base + sell_pos(lane, k);
      col16[pos] = static_cast<uint16_t>(step);
      if (s64) s64[pos] = a;
      if (s32) s32[pos] = b;
      ++k;
    };
    for (int e = 0; e < len; ++e) {
      const int32_t col = indices[rs + e];
      int64_t step = static_cast<int64_t>(col) - c;
      while (step > 65535) {
        put(65535u, 0.0, 0.0f);
        c += 65535;
        step -= 65535;
      }
      const double a = s64 ? (v64 ? v64[rs + e] : static_cast<double>(v32[rs + e])) : 0.0;
      const float b = s32 ? (v32 ? v32[rs + e] : static_cast<float>(v64[rs + e])) : 0.0f;
      put(static_cast<uint32_t>(step), a, b);
      c = col;
    }
    while (k < w) put(0u, 0.0, 0.0f);
  }
}

// entries of a row in the 15-bit copy: its entries plus one long-step entry
// per 2^30 - 1 of every step above 32767 (columns ascending)
__device__ __forceinline__ int d15_long_entries(int64_t step) {
  int m = 0;
  while (step > 32767) {
    const int64_t h = (step >> 15) < 0x7fff ? (step >> 15) : 0x7fff;
    step -= h << 15;
    ++m;
  }
  return m;
}

__global__ void d15_lengths(int64_t n, const int64_t* __restrict__ indptr, const int32_t* __restrict__ indices,
                            int32_t* __restrict__ len, int32_t* __restrict__ status) {
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int64_t a = indptr[i], b = indptr[i + 1];
    int64_t m = b - a;
    for (int64_t e = a + 1; e < b; ++e) {
      const int64_t step = static_cast<int64_t>(indices[e]) - indices[e - 1];
      if (step <= 0) set_status(status, FGB_ERR_ARG);  // columns must ascend strictly
      else if (step > 32767) m += d15_long_entries(step);
    }
    len[i] = static_cast<int32_t>(m);
  }
}

// Lane per slot: the slot's first column, then per entry a 15-bit step (or
// long steps before a far entry), padding with code 0 and value 0 up to the
// slice width.
__global__ void sell_fill_d15_kernel(int64_t n_slices, const int64_t* __restrict__ slice_ptr,
                                     const int32_t* __restrict__ perm, const int64_t* __restrict__ indptr,
                                     const int32_t* __restrict__ indices, const double* __restrict__ v64,
                                     const float* __restrict__ v32, int32_t* __restrict__ col0,
                                     uint16_t* __restrict__ col16, double* __restrict__ s64,
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
    if (row >= 0) {
      rs = indptr[row];
      len = static_cast<int>(indptr[row + 1] - rs);
    }
    int64_t c = len > 0 ? indices[rs] : (row >= 0 ? row : 0);
    col0[s * kSellC + lane] = static_cast<int32_t>(c);
    int k = 0;
    auto put = [&](uint32_t code, double a, float b) {
      if (k >= w) return;  // cannot happen: the plan's width covers the row with its long steps
      const int64_t pos = base + sell_pos(lane, k);
      col16[pos] = static_cast<uint16_t>(code);
      if (s64) s64[pos] = a;
      if (s32) s32[pos] = b;
      ++k;
    };
    for (int e = 0; e < len; ++e) {
      const int64_t col = indices[rs + e];
      int64_t step = col - c;
      while (step > 32767) {
        const int64_t h = (step >> 15) < 0x7fff ? (step >> 15) : 0x7fff;
        put(0x8000u | static_cast<uint32_t>(h), 0.0, 0.0f);
        step -= h << 15;
      }
      const double a = s64 ? (v64 ? v64[rs + e] : static_cast<double>(v32[rs + e])) : 0.0;
      const float b = s32 ? (v32 ? v32[rs + e] : static_cast<float>(v64[rs + e])) : 0.0f;
      put(static_cast<uint32_t>(step), a, b);
      c = col;
    }
    while (k < w) put(0u, 0.0, 0.0f);
  }
}

template <typename T>
__global__ void permute_kernel(int64_t n, const int32_t* __restrict__ order, const T* __restrict__ src,
                               T* __restrict__ dst, int scatter) {
  for (int64_t k = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; k < n;
       k += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    if (scatter) dst[order[k]] = src[k];
    else dst[k] = src[order[k]];
  }
}

}  // namespace fgb

using namespace fgb;

namespace {

constexpr int kThreads = 256;

int grid_rows(int64_t n) { return grid_for(n, kThreads, kNumSMs * 16); }

}  // namespace

extern "C" {

size_t fgb_sell_d16_workspace_bytes(int64_t n) {
  if (n <= 0) return 0;
  const size_t un = static_cast<size_t>(n);
  return align_up(un * sizeof(int32_t)) + align_up((un + 1) * sizeof(int32_t)) +
         align_up((un + 1) * sizeof(int64_t)) + align_up(sizeof(int32_t)) + scan_workspace_bytes(n);
}

int32_t fgb_sell_renumber(int64_t n, const int64_t* indptr, const int32_t* indices, int32_t n_blocks,
                          const int64_t* block_sizes_host, int32_t* order, int32_t* inv, void* workspace,
                          size_t workspace_bytes, void* stream) {
  if (n <= 0 || !order || !inv || n_blocks < 0 || n_blocks > kMaxBlocks) return FGB_ERR_ARG;
  if (n >= (int64_t(1) << 31)) return FGB_ERR_CAPACITY;
  cudaStream_t st = as_stream(stream);
  if (n_blocks > 0) {
    if (!block_sizes_host) return FGB_ERR_ARG;
    DofBlocks B{};
    B.n = n_blocks;
    B.start[0] = 0;
    for (int b = 0; b < n_blocks; ++b) {
      if (block_sizes_host[b] <= 0) return FGB_ERR_ARG;
      B.start[b + 1] = B.start[b] + block_sizes_host[b];
    }
    if (B.start[n_blocks] != n) return FGB_ERR_ARG;
    renumber_blocks<<<grid_rows(n), kThreads, 0, st>>>(n, B, order, inv);
    return launch_status();
  }
  if (!indptr || !indices) return FGB_ERR_ARG;
  if (!workspace || workspace_bytes < fgb_sell_d16_workspace_bytes(n)) return FGB_ERR_WORKSPACE;
  Carver cv(workspace, workspace_bytes);
  int32_t* key = cv.take<int32_t>(n);
  int32_t* cnt = cv.take<int32_t>(n + 1);
  int64_t* start = cv.take<int64_t>(n + 1);
  int32_t* too_big = cv.take<int32_t>(1);
  void* scan_ws = cv.base + cv.off;
  const size_t scan_bytes = workspace_bytes - cv.off;
  if (!cv.ok) return FGB_ERR_WORKSPACE;
  if (cudaMemsetAsync(cnt, 0, (n + 1) * sizeof(int32_t), st) != cudaSuccess) return FGB_ERR_CUDA;
  if (cudaMemsetAsync(too_big, 0, sizeof(int32_t), st) != cudaSuccess) return FGB_ERR_CUDA;
  renumber_keys<<<grid_rows(n), kThreads, 0, st>>>(n, indptr, indices, key, cnt);
  int rc = exclusive_scan_i32_to_i64(cnt, n, start, scan_ws, scan_bytes, st);
  if (rc) return rc;
  if (cudaMemsetAsync(cnt, 0, (n + 1) * sizeof(int32_t), st) != cudaSuccess) return FGB_ERR_CUDA;
  renumber_place<<<grid_rows(n), kThreads, 0, st>>>(n, key, start, cnt, order);
  renumber_sort_groups<<<grid_rows(n), kThreads, 0, st>>>(n, start, order, too_big);
  renumber_inverse<<<grid_rows(n), kThreads, 0, st>>>(n, order, inv, too_big);
  return launch_status();
}

int32_t fgb_csr_permute(int64_t n, const int64_t* indptr, const int32_t* indices, const double* values64,
                        const float* values32, const int32_t* order, const int32_t* inv, int64_t* new_indptr,
                        int32_t* new_indices, double* new_values64, float* new_values32, void* workspace,
                        size_t workspace_bytes, void* stream) {
  if (n <= 0 || !indptr || !indices || !order || !inv || !new_indptr || !new_indices) return FGB_ERR_ARG;
  if ((new_values64 || new_values32) && !values64 && !values32) return FGB_ERR_ARG;
  if (!workspace || workspace_bytes < fgb_sell_d16_workspace_bytes(n)) return FGB_ERR_WORKSPACE;
  cudaStream_t st = as_stream(stream);
  Carver cv(workspace, workspace_bytes);
  int32_t* len = cv.take<int32_t>(n);
  void* scan_ws = cv.base + cv.off;
  const size_t scan_bytes = workspace_bytes - cv.off;
  if (!cv.ok) return FGB_ERR_WORKSPACE;
  permuted_lengths<<<grid_rows(n), kThreads, 0, st>>>(n, indptr, order, len);
  int rc = exclusive_scan_i32_to_i64(len, n, new_indptr, scan_ws, scan_bytes, st);
  if (rc) return rc;
  csr_permute_fill<<<grid_for(n * 32, kPermWarps * 32, kNumSMs * 16), kPermWarps * 32, 0, st>>>(
      n, indptr, indices, values64, values32, order, inv, new_indptr, new_indices, new_values64, new_values32);
  return launch_status();
}

int32_t fgb_sell_d16_indptr(int64_t n, const int64_t* indptr, const int32_t* indices, int64_t* bridged_indptr,
                            void* workspace, size_t workspace_bytes, void* stream) {
  if (n <= 0 || !indptr || !indices || !bridged_indptr) return FGB_ERR_ARG;
  if (!workspace || workspace_bytes < fgb_sell_d16_workspace_bytes(n)) return FGB_ERR_WORKSPACE;
  cudaStream_t st = as_stream(stream);
  Carver cv(workspace, workspace_bytes);
  int32_t* len = cv.take<int32_t>(n);
  void* scan_ws = cv.base + cv.off;
  const size_t scan_bytes = workspace_bytes - cv.off;
  if (!cv.ok) return FGB_ERR_WORKSPACE;
  d16_lengths<<<grid_rows(n), kThreads, 0, st>>>(n, indptr, indices, len);
  return exclusive_scan_i32_to_i64(len, n, bridged_indptr, scan_ws, scan_bytes, st);
}

int32_t fgb_sell_fill_d16(int64_t n, const int64_t* indptr, const int32_t* indices, const double* values64,
                          const float* values32, const int32_t* perm, const int64_t* slice_ptr, int32_t* col0,
                          uint16_t* col16, double* val64, float* val32, void* stream) {
  if (n <= 0 || !indptr || !indices || !perm || !slice_ptr || !col0 || !col16) return FGB_ERR_ARG;
  if ((val64 || val32) && !values64 && !values32) return FGB_ERR_ARG;
  const int64_t slices = fgb_sell_slots(n) / kSellC;
  sell_fill_d16_kernel<<<grid_for(slices * 32, 256, kNumSMs * 16), 256, 0, as_stream(stream)>>>(
      slices, slice_ptr, perm, indptr, indices, values64, values32, col0, col16, val64, val32);
  return launch_status();
}

int32_t fgb_sell_d15_indptr(int64_t n, const int64_t* indptr, const int32_t* indices, int64_t* entry_indptr,
                            int32_t* status, void* workspace, size_t workspace_bytes, void* stream) {
  if (n <= 0 || !indptr || !indices || !entry_indptr || !status) return FGB_ERR_ARG;
  if (!workspace || workspace_bytes < fgb_sell_d16_workspace_bytes(n)) return FGB_ERR_WORKSPACE;
  cudaStream_t st = as_stream(stream);
  Carver cv(workspace, workspace_bytes);
  int32_t* len = cv.take<int32_t>(n);
  void* scan_ws = cv.base + cv.off;
  const size_t scan_bytes = workspace_bytes - cv.off;
  if (!cv.ok) return FGB_ERR_WORKSPACE;
  d15_lengths<<<grid_rows(n), kThreads, 0, st>>>(n, indptr, indices, len, status);
  return exclusive_scan_i32_to_i64(len, n, entry_indptr, scan_ws, scan_bytes, st);
}

int32_t fgb_sell_fill_d15(int64_t n, const int64_t* indptr, const int32_t* indices, const double* values64,
                          const float* values32, const int32_t* perm, const int64_t* slice_ptr, int32_t* col0,
                          uint16_t* col16, double* val64, float* val32, void* stream) {
  if (n <= 0 || !indptr || !indices || !perm || !slice_ptr || !col0 || !col16) return FGB_ERR_ARG;
  if ((val64 || val32) && !values64 && !values32) return FGB_ERR_ARG;
  const int64_t slices = fgb_sell_slots(n) / kSellC;
  sell_fill_d15_kernel<<<grid_for(slices * 32, 256, kNumSMs * 16), 256, 0, as_stream(stream)>>>(
      slices, slice_ptr, perm, indptr, indices, values64, values32, col0, col16, val64, val32);
  return launch_status();
}

int32_t fgb_permute(int32_t dtype, int64_t n, const int32_t* order, const void* src, void* dst, int32_t scatter,
                    void* stream) {
  if (n <= 0 || !order || !src || !dst || src == dst) return FGB_ERR_ARG;
  cudaStream_t st = as_stream(stream);
  if (dtype == FGB_F64)
    permute_kernel<double><<<grid_rows(n), kThreads, 0, st>>>(n, order, static_cast<const double*>(src),
                                                               static_cast<double*>(dst), scatter);
  else if (dtype == FGB_F32)
    permute_kernel<float><<<grid_rows(n), kThreads, 0, st>>>(n, order, static_cast<const float*>(src),
                                                              static_cast<float*>(dst), scatter);
  else
    return FGB_ERR_ARG;
  return launch_status();
}

}  // extern "C"
