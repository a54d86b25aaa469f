// Split of a block-diagonal CSR (many independent systems assembled as one:
// system s owns rows and columns [row_off[s], row_off[s + 1])) into the
// systems' own CSRs.  The entries stay where they are (every system's
// indices and values are a contiguous range of the union's arrays); the
// columns are rebased in place to the system's numbering, and every system
// gets its own row pointer (n_s + 1 entries, starting at 0) in indptr_out,
// system s at offset row_off[s] + s.  No FEALPy counterpart: FEALPy assembles
// one system per BilinearForm; this serves the batched assembly of many.

#include "fgb_common.cuh"

namespace fgb {

// the system owning row i: last s with row_off[s] <= i (binary search)
__device__ __forceinline__ int system_of_row(int64_t i, const int64_t* __restrict__ row_off, int n_sys) {
  int lo = 0, hi = n_sys - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (row_off[mid] <= i) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// indptr_out[row_off[s] + s + k] = indptr[row_off[s] + k] - indptr[row_off[s]],
// k = 0 .. n_s; one thread per output entry
__global__ void split_indptr_kernel(int n_sys, const int64_t* __restrict__ row_off,
                                    const int64_t* __restrict__ indptr, int64_t* __restrict__ indptr_out,
                                    int64_t n_out) {
  for (int64_t t = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; t < n_out;
       t += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    // output entry t belongs to the system s with row_off[s] + s <= t
    int lo = 0, hi = n_sys - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (row_off[mid] + mid <= t) lo = mid;
      else hi = mid - 1;
    }
    const int64_t k = t - (row_off[lo] + lo);
    indptr_out[t] = indptr[row_off[lo] + k] - indptr[row_off[lo]];
  }
}

// columns of row i minus the first column of its system; a column outside
// the system's range is a pattern error (the union is not block diagonal)
__global__ void split_indices_kernel(int64_t n, int n_sys, const int64_t* __restrict__ row_off,
                                     const int64_t* __restrict__ indptr, int32_t* __restrict__ indices,
                                     int32_t* status) {
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int s = system_of_row(i, row_off, n_sys);
    const int64_t lo = row_off[s], hi = row_off[s + 1];
    for (int64_t e = indptr[i]; e < indptr[i + 1]; ++e) {
      const int64_t c = indices[e];
      if (c < lo || c >= hi) {
        set_status(status, FGB_ERR_PATTERN);
        continue;
      }
      indices[e] = static_cast<int32_t>(c - lo);
    }
  }
}

}  // namespace fgb

using namespace fgb;

extern "C" {

int32_t fgb_csr_split_blocks(int32_t n_sys, const int64_t* row_off, const int64_t* indptr, int32_t* indices,
                             int64_t* indptr_out, int64_t n_rows, int32_t* status, void* stream) {
  if (n_sys <= 0 || n_rows < 0 || !row_off || !indptr || !indices || !indptr_out || !status) return FGB_ERR_ARG;
  cudaStream_t st = as_stream(stream);
  const int64_t n_out = n_rows + n_sys;
  split_indptr_kernel<<<grid_for(n_out, 256, kNumSMs * 8), 256, 0, st>>>(n_sys, row_off, indptr, indptr_out, n_out);
  if (n_rows > 0)
    split_indices_kernel<<<grid_for(n_rows, 256, kNumSMs * 8), 256, 0, st>>>(n_rows, n_sys, row_off, indptr, indices,
                                                                          status);
  return launch_status();
}

}  // extern "C"
