// spmv.cuh -- CSR sparse matrix * vector on sm_103a.
//
// Warp-tile kernel: each warp owns 32 consecutive rows.  The tile's slice of
// colidx / values is contiguous in CSR, so the warp stages it into shared
// memory with coalesced 16-byte loads, then every lane walks its own row out
// of shared memory, gathering x (L2-resident) and accumulating with FMA in
// column order.  Rows longer than the staging buffer fall back to direct
// loads for that tile.  An optional epilogue fuses the Lanczos dot product
// <v2, y> into the same pass.
#pragma once

#include "ham.cuh"
#include "vec.cuh"

namespace qd {

constexpr int kSpmvWarps = 4;  // warps per block
constexpr int kSpmvThreads = kSpmvWarps * 32;
// staged entries per warp tile: the block's staging fits in 46 KB of static shared memory
template <typename MV>
constexpr int spmv_span() {
  return (46 * 1024) / (kSpmvWarps * (int)(sizeof(int32_t) + sizeof(MV)));
}

template <typename MV, typename VV>
struct SpmvArgs {
  int64_t dim;
  const int64_t* rowptr;
  const int32_t* colidx;
  const MV* vals;
  const VV* x;
  VV* y;
  double scale;        // y = scale * (H x)
  const VV* dotv;      // if non-null: accumulate <dotv, y> into red
  GridRed<VV> red;
  VV* dot_out;         // final <dotv, y> (thread 0 of the last block)
  const int* stop;     // if non-null and *stop != 0 and *stop < step: do nothing
  int step;
};

template <typename T>
__device__ __forceinline__ void stage_copy(T* dst, const T* src, int n, int lane) {
  for (int i = lane; i < n; i += 32) dst[i] = src[i];
}

template <typename MV, typename VV>
__global__ void __launch_bounds__(kSpmvThreads) spmv_tile_kernel(SpmvArgs<MV, VV> A) {
  constexpr int kSpan = spmv_span<MV>();
  __shared__ int32_t s_col[kSpmvWarps][kSpan];
  __shared__ MV s_val[kSpmvWarps][kSpan];
  if (A.stop) {
    const int st = *A.stop;
    if (st != 0 && st < A.step) return;  // whole grid returns together
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t ntiles = (A.dim + 31) >> 5;
  const int64_t gw = (int64_t)blockIdx.x * kSpmvWarps + warp;
  const int64_t nw = (int64_t)gridDim.x * kSpmvWarps;
  VV dotacc = vzero(VV{});
  for (int64_t tile = gw; tile < ntiles; tile += nw) {
    const int64_t r = (tile << 5) + lane;
    const bool live = r < A.dim;
    const int64_t rb = live ? A.rowptr[r] : 0;
    const int64_t re = live ? A.rowptr[r + 1] : 0;
    const int64_t last_row = min((tile << 5) + 32, A.dim);
    const int64_t k0 = A.rowptr[tile << 5];
    const int64_t k1 = A.rowptr[last_row];
    const int64_t span = k1 - k0;
    VV acc = vzero(VV{});
    if (span <= kSpan) {
      stage_copy(s_col[warp], A.colidx + k0, (int)span, lane);
      stage_copy(s_val[warp], A.vals + k0, (int)span, lane);
      __syncwarp();
      const int b = (int)(rb - k0), e = (int)(re - k0);
      for (int k = b; k < e; ++k) acc = vfma(s_val[warp][k], ld_ro(A.x + s_col[warp][k]), acc);
      __syncwarp();
    } else {
      for (int64_t k = rb; k < re; ++k) acc = vfma(A.vals[k], ld_ro(A.x + A.colidx[k]), acc);
    }
    if (live) {
      const VV yv = vscale(A.scale, acc);
      A.y[r] = yv;
      if (A.dotv) dotacc = vdotfma(A.dotv[r], yv, dotacc);
    }
  }
  if (A.dotv) grid_sum(dotacc, A.red, A.dot_out);
}

}  // namespace qd
