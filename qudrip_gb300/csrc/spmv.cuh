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

constexpr int kMaxGrid = 65536;  // upper bound on blocks of any reduction kernel

// CSR product kernels (qd_ham::spmv_variant; qd_ham_time_spmv accepts them as `spmv`)
enum SpmvVariant {
  kSpmvTile = 100,      // warp tile, lane per row, staged in shared memory
  kSpmvBalanced = 101,  // warp tile, equal nnz per lane
  kSpmvVector2 = 102,   // 2 lanes per row
  kSpmvVector4 = 103,
  kSpmvVector8 = 104,
  kSpmvScalar = 105,    // thread per row
  kSpmvRow4 = 106,      // thread per row, 4 loads in flight
  kSpmvRow8 = 107,      // thread per row, 8 loads in flight
  kSpmvRow4Stream = 108,  // as 106 with evict-first matrix loads
  kSpmvRow8Stream = 109,  // as 107 with evict-first matrix loads
  kSpmvRowExact = 110,  // thread per row, groups of 4 loads, exact-count tail
  kSpmvRowSorted = 111, // as 110, rows taken in length order within 256-row windows
  kSpmvLast = 111,
  kSpmvFx = 120,        // uniform-coupling form, exact fixed-point sums (fxsum.cuh)
  kSpmvFxSlots = 121,   // as 120 with the columns computed on the fly (fxslots.cu)
  kSpmvFxBlock = 122,   // as 120 on the block layout of the sector, no column read (fxblock.cu)
};

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
  const double* scale_dev;      // if non-null, the scale is read from the device
  const double* dot_scale_dev;  // if non-null, the final dot is multiplied by *dot_scale_dev
  const int32_t* row_order;     // row permutation for the length-sorted kernel
};

template <typename MV, typename VV>
__device__ __forceinline__ double spmv_scale(const SpmvArgs<MV, VV>& A) {
  return A.scale_dev ? *A.scale_dev : A.scale;
}

template <typename MV, typename VV>
__device__ __forceinline__ void spmv_finish_dot(const SpmvArgs<MV, VV>& A, VV dotacc) {
  if (grid_sum(dotacc, A.red, A.dot_out) && threadIdx.x == 0 && A.dot_scale_dev)
    *A.dot_out = vscale(*A.dot_scale_dev, *A.dot_out);
}

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
      const VV yv = vscale(spmv_scale(A), acc);
      A.y[r] = yv;
      if (A.dotv) dotacc = vdotfma(A.dotv[r], yv, dotacc);
    }
  }
  if (A.dotv) spmv_finish_dot(A, dotacc);
}

}  // namespace qd

namespace qd {

// ---------------------------------------------------------------------------
// Balanced warp tile: the tile's nnz are split into 32 equal contiguous
// chunks (one per lane, an odd chunk length so shared-memory reads are free
// of bank conflicts), so every lane issues the same number of FMAs whatever
// the row lengths.  Rows cut by a chunk boundary are finished by the lane
// that holds their first entry, adding the later pieces in lane order.
// Staging uses 16-byte vector loads from the (padded) CSR arrays.
template <typename MV, typename VV>
__global__ void __launch_bounds__(kSpmvThreads) spmv_balanced_kernel(SpmvArgs<MV, VV> A) {
  constexpr int kVecV = 16 / (int)sizeof(MV);  // values per 16-byte load
  constexpr int kSpan = ((40 * 1024) / (kSpmvWarps * (int)(sizeof(int32_t) + sizeof(MV))) - 8) / 16 * 16;
  __shared__ __align__(16) int32_t s_col[kSpmvWarps][kSpan + 8];
  __shared__ __align__(16) MV s_val[kSpmvWarps][kSpan + 8];
  __shared__ int s_rp[kSpmvWarps][33];
  __shared__ VV s_head[kSpmvWarps][32];
  __shared__ int s_headrow[kSpmvWarps][32];
  __shared__ VV s_y[kSpmvWarps][32];
  if (A.stop) {
    const int st = *A.stop;
    if (st != 0 && st < A.step) return;
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t ntiles = (A.dim + 31) >> 5;
  const int64_t nw = (int64_t)gridDim.x * kSpmvWarps;
  VV dotacc = vzero(VV{});
  int* rp = s_rp[warp];
  for (int64_t tile = (int64_t)blockIdx.x * kSpmvWarps + warp; tile < ntiles; tile += nw) {
    const int64_t r0 = tile << 5;
    const int nrows = (int)min((int64_t)32, A.dim - r0);
    const int64_t kb = A.rowptr[r0];
    if (lane < nrows) rp[lane] = (int)(A.rowptr[r0 + lane] - kb);
    if (lane == 0) rp[nrows] = (int)(A.rowptr[r0 + nrows] - kb);
    s_y[warp][lane] = vzero(VV{});
    s_headrow[warp][lane] = -1;
    __syncwarp();
    const int span = rp[nrows];
    if (span > kSpan) {
      // long rows: lane per row straight from global memory
      if (lane < nrows) {
        VV acc = vzero(VV{});
        for (int64_t k = kb + rp[lane]; k < kb + rp[lane + 1]; ++k)
          acc = vfma(A.vals[k], ld_ro(A.x + A.colidx[k]), acc);
        s_y[warp][lane] = acc;
      }
    } else {
      // stage with 16-byte loads from aligned starts
      const int64_t kv = kb & ~(int64_t)(kVecV - 1);
      const int offv = (int)(kb - kv);
      const int nv = (offv + span + kVecV - 1) / kVecV;
      const int4* gv = reinterpret_cast<const int4*>(A.vals + kv);
      int4* sv = reinterpret_cast<int4*>(s_val[warp]);
      for (int i = lane; i < nv; i += 32) sv[i] = __ldg(gv + i);
      const int64_t kc = kb & ~(int64_t)3;
      const int offc = (int)(kb - kc);
      const int nc = (offc + span + 3) / 4;
      const int4* gc = reinterpret_cast<const int4*>(A.colidx + kc);
      int4* sc = reinterpret_cast<int4*>(s_col[warp]);
      for (int i = lane; i < nc; i += 32) sc[i] = __ldg(gc + i);
      __syncwarp();
      int q = (span + 31) >> 5;
      q |= 1;
      const int a = min(lane * q, span), b = min(a + q, span);
      if (a < b) {
        // row containing entry a: last j with rp[j] <= a
        int lo = 0, hi = nrows - 1;
        while (lo < hi) {
          const int mid = (lo + hi + 1) >> 1;
          if (rp[mid] <= a) lo = mid;
          else hi = mid - 1;
        }
        int j = lo;
        int next = rp[j + 1];
        const bool head_cont = rp[j] < a;  // row j began in an earlier lane
        bool first = true;
        VV acc = vzero(VV{});
        const MV* sval = s_val[warp] + offv;
        const int32_t* scol = s_col[warp] + offc;
        for (int k = a; k < b; ++k) {
          while (k == next) {  // row j ends before k
            if (first && head_cont) {
              s_head[warp][lane] = acc;
              s_headrow[warp][lane] = j;
            } else {
              s_y[warp][j] = acc;  // complete inside this lane
            }
            first = false;
            acc = vzero(VV{});
            ++j;
            next = rp[j + 1];
          }
          acc = vfma(sval[k], ld_ro(A.x + scol[k]), acc);
        }
        // last row touched: complete, a head piece, or continues into later lanes
        if (first && head_cont) {
          s_head[warp][lane] = acc;
          s_headrow[warp][lane] = j;
        } else if (next <= b) {
          s_y[warp][j] = acc;
        } else {
          // this lane owns row j, which continues past b: keep the piece
          s_y[warp][j] = acc;
        }
      }
      __syncwarp();
      // owners of rows cut at their chunk end add the later pieces in lane order
      if (a < b) {
        int lo = 0, hi = nrows - 1;
        const int last = b - 1;
        while (lo < hi) {
          const int mid = (lo + hi + 1) >> 1;
          if (rp[mid] <= last) lo = mid;
          else hi = mid - 1;
        }
        const int j = lo;
        if (rp[j] >= a && rp[j + 1] > b) {
          VV acc = s_y[warp][j];
          for (int l = lane + 1; l < 32 && s_headrow[warp][l] == j; ++l) acc = vadd(acc, s_head[warp][l]);
          s_y[warp][j] = acc;
        }
      }
    }
    __syncwarp();
    if (lane < nrows) {
      const int64_t r = r0 + lane;
      const VV yv = vscale(spmv_scale(A), s_y[warp][lane]);
      A.y[r] = yv;
      if (A.dotv) dotacc = vdotfma(A.dotv[r], yv, dotacc);
    }
    __syncwarp();
  }
  if (A.dotv) spmv_finish_dot(A, dotacc);
}

// ---------------------------------------------------------------------------
// G lanes per row ("vector CSR"): each group strides its row, then a
// shuffle reduction.
template <typename MV, typename VV, int G>
__global__ void __launch_bounds__(256) spmv_vector_kernel(SpmvArgs<MV, VV> A) {
  if (A.stop) {
    const int st = *A.stop;
    if (st != 0 && st < A.step) return;
  }
  const int64_t gt = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int sub = threadIdx.x & (G - 1);
  const int64_t ngroups = ((int64_t)gridDim.x * blockDim.x) / G;
  VV dotacc = vzero(VV{});
  // every thread iterates the same number of times so the shuffles stay converged
  const int64_t iters = (A.dim + ngroups - 1) / ngroups;
  for (int64_t it = 0; it < iters; ++it) {
    const int64_t r = gt / G + it * ngroups;
    VV acc = vzero(VV{});
    if (r < A.dim) {
      const int64_t e = A.rowptr[r + 1];
      for (int64_t k = A.rowptr[r] + sub; k < e; k += G) acc = vfma(A.vals[k], ld_ro(A.x + A.colidx[k]), acc);
    }
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1) acc = vadd(acc, shfl_xor(acc, o));
    if (r < A.dim && sub == 0) {
      const VV yv = vscale(spmv_scale(A), acc);
      A.y[r] = yv;
      if (A.dotv) dotacc = vdotfma(A.dotv[r], yv, dotacc);
    }
  }
  if (A.dotv) spmv_finish_dot(A, dotacc);
}

}  // namespace qd

namespace qd {

__device__ __forceinline__ double ld_stream(const double* p) { return __ldcs(p); }
__device__ __forceinline__ float ld_stream(const float* p) { return __ldcs(p); }
__device__ __forceinline__ int32_t ld_stream(const int32_t* p) { return __ldcs(p); }
__device__ __forceinline__ cplx ld_stream(const cplx* p) {
  const double2 d = __ldcs(reinterpret_cast<const double2*>(p));
  return mkc(d.x, d.y);
}
__device__ __forceinline__ double ld_plain(const double* p) { return __ldg(p); }
__device__ __forceinline__ float ld_plain(const float* p) { return __ldg(p); }
__device__ __forceinline__ int32_t ld_plain(const int32_t* p) { return __ldg(p); }
__device__ __forceinline__ cplx ld_plain(const cplx* p) { return ld_ro(p); }

// Thread per row with U independent (column, value, x) loads in flight per
// iteration; FMAs stay in column order.  STREAM marks the matrix loads
// evict-first so the gathered vector keeps its place in L1/L2.
template <typename MV, typename VV, int U, bool STREAM>
__global__ void __launch_bounds__(256) spmv_rowunroll_kernel(SpmvArgs<MV, VV> A) {
  if (A.stop) {
    const int st = *A.stop;
    if (st != 0 && st < A.step) return;
  }
  VV dotacc = vzero(VV{});
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < A.dim; r += stride) {
    const int64_t b = A.rowptr[r], e = A.rowptr[r + 1];
    VV acc = vzero(VV{});
    for (int64_t k = b; k < e; k += U) {
      int32_t c[U];
      MV v[U];
      VV xv[U];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const bool ok = k + u < e;
        c[u] = ok ? (STREAM ? ld_stream(A.colidx + k + u) : ld_plain(A.colidx + k + u)) : 0;
        v[u] = ok ? (STREAM ? ld_stream(A.vals + k + u) : ld_plain(A.vals + k + u)) : MV{};
      }
#pragma unroll
      for (int u = 0; u < U; ++u) xv[u] = (k + u < e) ? ld_ro(A.x + c[u]) : vzero(VV{});
#pragma unroll
      for (int u = 0; u < U; ++u)
        if (k + u < e) acc = vfma(v[u], xv[u], acc);
    }
    const VV yv = vscale(spmv_scale(A), acc);
    A.y[r] = yv;
    if (A.dotv) dotacc = vdotfma(A.dotv[r], yv, dotacc);
  }
  if (A.dotv) spmv_finish_dot(A, dotacc);
}

}  // namespace qd

namespace qd {

// Thread per row: groups of four (column, value, x) loads in flight, then an
// exact-count tail, so no FMA slot is spent on predicated-off entries.
template <typename MV, typename VV>
__global__ void __launch_bounds__(256) spmv_rowexact_kernel(SpmvArgs<MV, VV> A) {
  if (A.stop) {
    const int st = *A.stop;
    if (st != 0 && st < A.step) return;
  }
  VV dotacc = vzero(VV{});
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < A.dim; r += stride) {
    const int64_t b = A.rowptr[r], e = A.rowptr[r + 1];
    VV acc = vzero(VV{});
    int64_t k = b;
    for (; k + 4 <= e; k += 4) {
      int32_t c[4];
      MV v[4];
      VV xv[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        c[u] = ld_plain(A.colidx + k + u);
        v[u] = ld_plain(A.vals + k + u);
      }
#pragma unroll
      for (int u = 0; u < 4; ++u) xv[u] = ld_ro(A.x + c[u]);
#pragma unroll
      for (int u = 0; u < 4; ++u) acc = vfma(v[u], xv[u], acc);
    }
    for (; k < e; ++k) acc = vfma(ld_plain(A.vals + k), ld_ro(A.x + ld_plain(A.colidx + k)), acc);
    const VV yv = vscale(spmv_scale(A), acc);
    A.y[r] = yv;
    if (A.dotv) dotacc = vdotfma(A.dotv[r], yv, dotacc);
  }
  if (A.dotv) spmv_finish_dot(A, dotacc);
}

// As spmv_rowexact_kernel, but the i-th thread of the grid takes row
// row_order[i]: rows are sorted by length inside windows of 256, so the lanes
// of a warp issue nearly the same number of FMAs (less idle FP64 issue).
template <typename MV, typename VV>
__global__ void __launch_bounds__(256) spmv_rowsorted_kernel(SpmvArgs<MV, VV> A) {
  if (A.stop) {
    const int st = *A.stop;
    if (st != 0 && st < A.step) return;
  }
  VV dotacc = vzero(VV{});
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < A.dim; i += stride) {
    const int64_t r = A.row_order[i];
    const int64_t b = A.rowptr[r], e = A.rowptr[r + 1];
    VV acc = vzero(VV{});
    int64_t k = b;
    for (; k + 4 <= e; k += 4) {
      int32_t c[4];
      MV v[4];
      VV xv[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        c[u] = ld_plain(A.colidx + k + u);
        v[u] = ld_plain(A.vals + k + u);
      }
#pragma unroll
      for (int u = 0; u < 4; ++u) xv[u] = ld_ro(A.x + c[u]);
#pragma unroll
      for (int u = 0; u < 4; ++u) acc = vfma(v[u], xv[u], acc);
    }
    for (; k < e; ++k) acc = vfma(ld_plain(A.vals + k), ld_ro(A.x + ld_plain(A.colidx + k)), acc);
    const VV yv = vscale(spmv_scale(A), acc);
    A.y[r] = yv;
    if (A.dotv) dotacc = vdotfma(A.dotv[r], yv, dotacc);
  }
  if (A.dotv) spmv_finish_dot(A, dotacc);
}

}  // namespace qd

namespace qd {

inline int spmv_grid(Ctx* ctx, int64_t dim) {
  const int64_t tiles = (dim + 31) / 32;
  const int64_t want = ceil_div(tiles, kSpmvWarps);
  return (int)std::max<int64_t>(1, std::min<int64_t>(want, (int64_t)ctx->num_sms * 16));
}

// ---------------------------------------------------------------- launches
template <typename MV, typename VV>
inline void launch_spmv(Ctx* ctx, const qd_ham* H, const MV* vals, const VV* x, VV* y, double scale, const VV* dotv,
                 GridRed<VV> red, VV* dot_out, const int* stop, int step, int variant,
                 const double* scale_dev = nullptr, const double* dot_scale_dev = nullptr) {
  SpmvArgs<MV, VV> A;
  A.dim = H->dim;
  A.rowptr = H->rowptr.p;
  A.colidx = H->colidx.p;
  A.vals = vals;
  A.x = x;
  A.y = y;
  A.scale = scale;
  A.dotv = dotv;
  A.red = red;
  A.dot_out = dot_out;
  A.stop = stop;
  A.step = step;
  A.scale_dev = scale_dev;
  A.dot_scale_dev = dot_scale_dev;
  A.row_order = H->row_order.p;
  if (variant < 0) variant = H->spmv_variant;
  // every grid is capped so the block partials of a fused dot fit in kMaxGrid slots
  const unsigned vg = (unsigned)std::max<int64_t>(
      1, std::min<int64_t>(ceil_div(H->dim, 256 / 4), (int64_t)ctx->num_sms * 8));
  const unsigned rg = (unsigned)std::max<int64_t>(1, std::min<int64_t>(ceil_div(H->dim, 256), (int64_t)kMaxGrid));
  const unsigned tg = (unsigned)spmv_grid(ctx, H->dim);
  QD_REQUIRE(vg <= (unsigned)kMaxGrid && rg <= (unsigned)kMaxGrid && tg <= (unsigned)kMaxGrid, QD_ERR_UNSUPPORTED,
             "reduction grid exceeds its partials buffer");
  switch (variant) {
    case kSpmvTile: spmv_tile_kernel<MV, VV><<<tg, kSpmvThreads, 0, ctx->stream>>>(A); break;
    case kSpmvBalanced: spmv_balanced_kernel<MV, VV><<<tg, kSpmvThreads, 0, ctx->stream>>>(A); break;
    case kSpmvVector2: spmv_vector_kernel<MV, VV, 2><<<vg, 256, 0, ctx->stream>>>(A); break;
    case kSpmvVector4: spmv_vector_kernel<MV, VV, 4><<<vg, 256, 0, ctx->stream>>>(A); break;
    case kSpmvVector8: spmv_vector_kernel<MV, VV, 8><<<vg, 256, 0, ctx->stream>>>(A); break;
    case kSpmvRow4: spmv_rowunroll_kernel<MV, VV, 4, false><<<rg, 256, 0, ctx->stream>>>(A); break;
    case kSpmvRow8: spmv_rowunroll_kernel<MV, VV, 8, false><<<rg, 256, 0, ctx->stream>>>(A); break;
    case kSpmvRow4Stream: spmv_rowunroll_kernel<MV, VV, 4, true><<<rg, 256, 0, ctx->stream>>>(A); break;
    case kSpmvRow8Stream: spmv_rowunroll_kernel<MV, VV, 8, true><<<rg, 256, 0, ctx->stream>>>(A); break;
    case kSpmvRowExact: spmv_rowexact_kernel<MV, VV><<<rg, 256, 0, ctx->stream>>>(A); break;
    case kSpmvRowSorted:
      QD_REQUIRE(H->row_order.p != nullptr, QD_ERR_INVALID, "length-sorted kernel without a row order");
      spmv_rowsorted_kernel<MV, VV><<<rg, 256, 0, ctx->stream>>>(A);
      break;
    default: spmv_vector_kernel<MV, VV, 1><<<vg, 256, 0, ctx->stream>>>(A); break;
  }
  QD_CHECK_LAUNCH();
  QD_LAUNCHED(ctx);
}

}  // namespace qd
