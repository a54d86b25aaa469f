// Node-triple SELL copy for vector problems with three interleaved components.
//
// Why: with dof = 3 node + comp, every nonzero of a row lies in a run of three
// consecutive columns 3c..3c+2 (the coupling of two nodes is a 3x3 block), so
// one 4-byte column serves three values: the FP32 SpMV streams 16 bytes per
// three entries instead of 24, and the three gathers of a triple hit one or
// two lines.  Rows of Dirichlet dofs keep a partial triple (their unit
// diagonal) with zeros in the other two values.
//
// Construction: triple counts per row (columns ascending), their scan as the
// row pointer given to the SELL plan (rows sorted by triple count inside
// 256-row windows), then the fill: a lane per slot zeroes its slice row and
// writes every entry into its triple.

#include "fgb_common.cuh"
#include "sell_rows.cuh"

namespace fgb {

// triples of every row: runs of entries with the same column / 3
__global__ void b3_counts(int64_t n, const int64_t* __restrict__ indptr, const int32_t* __restrict__ indices,
                          int32_t* __restrict__ cnt) {
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    int m = 0;
    int32_t cur = -1;
    for (int64_t e = indptr[i]; e < indptr[i + 1]; ++e) {
      const int32_t c3 = indices[e] / 3;
      if (c3 != cur) {
        ++m;
        cur = c3;
      }
    }
    cnt[i] = m;
  }
}

// Lane per slot: the slot's slice row, every triple zeroed (its column the
// first column of the row's node, or 0 for padding slots), then the row's
// entries written into their triples in column order.
__global__ void sell_fill_b3_kernel(int64_t n_slices, const int64_t* __restrict__ slice_ptr,
                                    const int32_t* __restrict__ perm, const int64_t* __restrict__ indptr,
                                    const int32_t* __restrict__ indices, const double* __restrict__ v64,
                                    const float* __restrict__ v32, int32_t* __restrict__ scol,
                                    double* __restrict__ s64, float* __restrict__ s32) {
  const int lane = threadIdx.x & 31;
  const int64_t warp = (blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x) >> 5;
  const int64_t nwarps = (static_cast<int64_t>(gridDim.x) * blockDim.x) >> 5;
  for (int64_t s = warp; s < n_slices; s += nwarps) {
    const int64_t base = slice_ptr[s];
    const int w = static_cast<int>((slice_ptr[s + 1] - base) / kSellC);
    const int32_t row = perm[s * kSellC + lane];
    const int32_t pad = row >= 0 ? (row / 3) * 3 : 0;
    for (int k = 0; k < w; ++k) {
      const int64_t pos = base + sell_pos(lane, k);
      scol[pos] = pad;
      for (int j = 0; j < 3; ++j) {
        if (s64) s64[3 * pos + j] = 0.0;
        if (s32) s32[3 * pos + j] = 0.0f;
      }
    }
    if (row < 0) continue;
    int k = -1;
    int32_t cur = -1;
    for (int64_t e = indptr[row]; e < indptr[row + 1]; ++e) {
      const int32_t c = indices[e];
      if (c / 3 != cur) {
        cur = c / 3;
        ++k;
      }
      if (k >= w) break;  // cannot happen: the plan's width covers the triple count
      const int64_t pos = base + sell_pos(lane, k);
      scol[pos] = 3 * cur;
      const int j = c - 3 * cur;
      if (s64) s64[3 * pos + j] = v64 ? v64[e] : static_cast<double>(v32[e]);
      if (s32) s32[3 * pos + j] = v32 ? v32[e] : static_cast<float>(v64[e]);
    }
  }
}

}  // namespace fgb

using namespace fgb;

extern "C" {

int32_t fgb_sell_b3_indptr(int64_t n, const int64_t* indptr, const int32_t* indices, int64_t* triple_indptr,
                           void* workspace, size_t workspace_bytes, void* stream) {
  if (n <= 0 || n % 3 != 0 || !indptr || !indices || !triple_indptr) return FGB_ERR_ARG;
  if (n >= (int64_t(1) << 31)) return FGB_ERR_CAPACITY;
  if (!workspace || workspace_bytes < fgb_sell_d16_workspace_bytes(n)) return FGB_ERR_WORKSPACE;
  cudaStream_t st = as_stream(stream);
  Carver cv(workspace, workspace_bytes);
  int32_t* cnt = cv.take<int32_t>(n);
  void* scan_ws = cv.base + cv.off;
  const size_t scan_bytes = workspace_bytes - cv.off;
  if (!cv.ok) return FGB_ERR_WORKSPACE;
  b3_counts<<<grid_for(n, 256, kNumSMs * 16), 256, 0, st>>>(n, indptr, indices, cnt);
  return exclusive_scan_i32_to_i64(cnt, n, triple_indptr, scan_ws, scan_bytes, st);
}

int32_t fgb_sell_fill_b3(int64_t n, const int64_t* indptr, const int32_t* indices, const double* values64,
                         const float* values32, const int32_t* perm, const int64_t* slice_ptr, int32_t* col,
                         double* val64, float* val32, void* stream) {
  if (n <= 0 || n % 3 != 0 || !indptr || !indices || !perm || !slice_ptr || !col) return FGB_ERR_ARG;
  if ((val64 || val32) && !values64 && !values32) return FGB_ERR_ARG;
  const int64_t slices = fgb_sell_slots(n) / kSellC;
  sell_fill_b3_kernel<<<grid_for(slices * 32, 256, kNumSMs * 16), 256, 0, as_stream(stream)>>>(
      slices, slice_ptr, perm, indptr, indices, values64, values32, col, val64, val32);
  return launch_status();
}

}  // extern "C"
