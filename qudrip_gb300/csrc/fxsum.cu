// fxsum.cu -- building the uniform-coupling form and its product (fxsum.cuh).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "fxstep.cuh"
#include "fxsum.cuh"
#include "ham.cuh"
#include "krylov.cuh"
#include "scan.cuh"
#include "spmv.cuh"
#include "vec.cuh"

namespace qd {

constexpr unsigned long long kNoValue = ~0ull;

// The first nonzero off-diagonal value any row meets (its bits).
__global__ void fx_probe_kernel(int64_t n, const int64_t* rowptr, const int32_t* colidx, const double* vals,
                                unsigned long long* cand) {
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
    for (int64_t k = rowptr[r]; k < rowptr[r + 1]; ++k) {
      const double v = vals[k];
      if (colidx[k] != (int32_t)r && v != 0.0) {
        atomicCAS(cand, kNoValue, (unsigned long long)__double_as_longlong(v));
        break;
      }
    }
  }
}

// Per row: off-diagonal count, diagonal value, |row| sum; flags any
// off-diagonal value other than c.
__global__ void fx_count_kernel(int64_t n, const int64_t* rowptr, const int32_t* colidx, const double* vals, double c,
                                int64_t* counts, double* diag, int* mismatch, unsigned long long* rowmax,
                                int* diag_nonzero) {
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
    int64_t cnt = 0;
    double d = 0.0, abs_sum = 0.0;
    for (int64_t k = rowptr[r]; k < rowptr[r + 1]; ++k) {
      const double v = vals[k];
      if (colidx[k] == (int32_t)r) {
        d = v;
      } else if (v != 0.0) {
        if (v != c) *mismatch = 1;
        ++cnt;
        abs_sum += fabs(v);
      }
    }
    abs_sum += fabs(d);
    counts[r] = cnt;
    diag[r] = d;
    if (d != 0.0) *diag_nonzero = 1;
    atomicMax(rowmax, (unsigned long long)__double_as_longlong(abs_sum));
  }
}

// Columns of row r in gather order: by the highest bit in which the column's
// state differs from the row's state, highest first (ties by column).  Rows
// next to each other share their high bits, so the entries of a warp's 32
// rows that flip high bits line up lane by lane and land on consecutive X
// values: the first gathers of a warp coalesce, and the ones that flip low
// bits fall near the warp's own rows.  The row sum is an exact integer sum,
// so the order does not change any result.
__device__ __forceinline__ int fx_order_key(uint64_t s, const uint64_t* basis, int32_t c) {
  return 63 - __clzll((long long)(s ^ basis[c]));
}

__global__ void fx_fill_kernel(int64_t n, const int64_t* rowptr, const int32_t* colidx, const double* vals,
                               const int64_t* off, const uint64_t* basis, int32_t* rowptr32, int32_t* colidx_fx) {
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r <= n; r += (int64_t)gridDim.x * blockDim.x) {
    rowptr32[r] = (int32_t)off[r];
    if (r == n) break;
    const int64_t o0 = off[r];
    int64_t o = o0;
    for (int64_t k = rowptr[r]; k < rowptr[r + 1]; ++k)
      if (colidx[k] != (int32_t)r && vals[k] != 0.0) colidx_fx[o++] = colidx[k];
    const uint64_t s = basis[r];
    for (int64_t i = o0 + 1; i < o; ++i) {  // insertion sort: rows hold at most 128 columns
      const int32_t c = colidx_fx[i];
      const int kc = fx_order_key(s, basis, c);
      int64_t j = i - 1;
      while (j >= o0) {
        const int32_t p = colidx_fx[j];
        const int kp = fx_order_key(s, basis, p);
        if (kp > kc || (kp == kc && p < c)) break;
        colidx_fx[j + 1] = p;
        --j;
      }
      colidx_fx[j + 1] = c;
    }
  }
}

static int fx_grid(Ctx* ctx, int64_t n) {
  return (int)std::max<int64_t>(1, std::min<int64_t>(ceil_div(n, 256), (int64_t)ctx->num_sms * 8));
}

static void build_sell(Ctx* ctx, FxForm& f, int64_t n);

bool ham_build_fx(qd_ham* H) {
  if (H->fx_state != 0) return H->fx_state > 0;
  H->fx_state = -1;
  if (!(H->flags & QD_HAM_REAL) || H->dim < 1 || H->dim >= (1ll << 31)) return false;
  Ctx* ctx = H->ctx;
  const int64_t n = H->dim;
  DBuf<unsigned long long> cand(2);
  DBuf<int> mismatch(1);
  QD_CUDA(cudaMemsetAsync(cand.p, 0xff, sizeof(unsigned long long), ctx->stream));
  QD_CUDA(cudaMemsetAsync(cand.p + 1, 0, sizeof(unsigned long long), ctx->stream));
  QD_CUDA(cudaMemsetAsync(mismatch.p, 0, sizeof(int), ctx->stream));
  DBuf<int> dnz(1);
  QD_CUDA(cudaMemsetAsync(dnz.p, 0, sizeof(int), ctx->stream));
  fx_probe_kernel<<<fx_grid(ctx, n), 256, 0, ctx->stream>>>(n, H->rowptr.p, H->colidx.p, H->vals_r.p, cand.p);
  QD_CHECK_LAUNCH();
  QD_LAUNCHED(ctx);
  unsigned long long cbits = kNoValue;
  QD_CUDA(cudaMemcpyAsync(&cbits, cand.p, 8, cudaMemcpyDeviceToHost, ctx->stream));
  QD_CUDA(cudaStreamSynchronize(ctx->stream));
  double c = 0.0;
  if (cbits != kNoValue) std::memcpy(&c, &cbits, 8);
  std::unique_ptr<FxForm> fx(new FxForm());
  DBuf<int64_t> counts(n + 1), off(n + 1);
  fx->diag.alloc(n);
  fx_count_kernel<<<fx_grid(ctx, n), 256, 0, ctx->stream>>>(n, H->rowptr.p, H->colidx.p, H->vals_r.p, c, counts.p,
                                                            fx->diag.p, mismatch.p, cand.p + 1, dnz.p);
  QD_CHECK_LAUNCH();
  QD_LAUNCHED(ctx);
  QD_CUDA(cudaMemsetAsync(counts.p + n, 0, sizeof(int64_t), ctx->stream));
  exclusive_scan_i64(ctx, counts.p, off.p, n + 1);
  int mm = 0;
  unsigned long long rbits = 0;
  int64_t total = 0;
  QD_CUDA(cudaMemcpyAsync(&mm, mismatch.p, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  QD_CUDA(cudaMemcpyAsync(&rbits, cand.p + 1, 8, cudaMemcpyDeviceToHost, ctx->stream));
  QD_CUDA(cudaMemcpyAsync(&total, off.p + n, sizeof(int64_t), cudaMemcpyDeviceToHost, ctx->stream));
  int diag_nz = 1;
  QD_CUDA(cudaMemcpyAsync(&diag_nz, dnz.p, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  QD_CUDA(cudaStreamSynchronize(ctx->stream));
  fx->diag_zero = diag_nz == 0;
  if (mm || total >= (1ll << 31) || H->max_row_nnz > 128) return false;
  double rowmax = 0.0;
  std::memcpy(&rowmax, &rbits, 8);
  if (!std::isfinite(rowmax)) return false;
  const double bound = std::max(1.0, rowmax);
  const int eb = (int)std::ceil(std::log2(bound)) + 1;  // one bit of margin
  fx->F = 119 - eb;
  fx->c = c;
  fx->nnz = total;
  fx->rowptr.alloc(n + 1);
  fx->colidx.alloc(std::max<int64_t>(total, 1) + 16);
  QD_CUDA(cudaMemsetAsync(fx->colidx.p, 0, fx->colidx.bytes(), ctx->stream));
  fx_fill_kernel<<<fx_grid(ctx, n + 1), 256, 0, ctx->stream>>>(n, H->rowptr.p, H->colidx.p, H->vals_r.p, off.p,
                                                               H->sec->basis.p,
                                                               fx->rowptr.p, fx->colidx.p);
  QD_CHECK_LAUNCH();
  QD_LAUNCHED(ctx);
  QD_CUDA(cudaStreamSynchronize(ctx->stream));
  build_sell(ctx, *fx, n);
  H->fx = std::move(fx);
  H->fx_state = 1;
  // QD_FX_BLOCK=1 makes the block layout (code 122) the default where the sector and the
  // terms give it; otherwise the stored columns stay (the autotuner may still pick 122)
  const char* blk_env = std::getenv("QD_FX_BLOCK");
  if (blk_env && std::strcmp(blk_env, "1") == 0 && ham_build_fx_block(H)) H->fx->use_blk = true;
  return true;
}

// ---------------------------------------------------------------- product
// Column layout of the product: the rows in slices of 32 (a warp's rows),
// entry k of row 32 s + l at sell_off[s] + 128 (k / 4) + 4 l + k % 4, so
// that lane l loads four of its columns with one 16-byte load and the warp's
// 32 loads are one contiguous 512-byte run; a slice is as wide as its longest
// row, rounded up to 4 (26 % padding at L = 24), and sell_len holds each
// row's own count, so padding is never gathered.  Within a row the columns
// keep their gather order.

// Sum of the row's fixed-point gathers: four columns per 16-byte load, four
// predicated gathers in flight, and the next group's columns loaded before
// the current group's gathers.  The first group is loaded before the row's
// count is known: a row with no columns reads four padding entries (the
// column array carries 128 entries of tail padding, zeros).
__device__ __forceinline__ __int128 sell_row_sum(const int4* __restrict__ c4, int e, const __int128* __restrict__ X) {
  __int128 s = 0;
  int4 cc = __ldcs(c4);
#pragma unroll 1
  for (int k = 0; k < e; k += 4) {
    int4 nc = cc;
    if (k + 4 < e) nc = __ldcs(c4 + 8 * (k + 4));  // group k / 4 starts 32 int4 further on
    __int128 x0 = X[cc.x], x1 = 0, x2 = 0, x3 = 0;
    if (k + 1 < e) x1 = X[cc.y];
    if (k + 2 < e) x2 = X[cc.z];
    if (k + 3 < e) x3 = X[cc.w];
    s += (x0 + x1) + (x2 + x3);
    cc = nc;
  }
  return s;
}

__device__ __forceinline__ const int4* sell_row(const int64_t* __restrict__ soff, const int32_t* __restrict__ scol,
                                                int64_t r) {
  return reinterpret_cast<const int4*>(scol + __ldg(soff + (r >> 5))) + (r & 31);
}

// w_r = s * (d_r x_r + c 2^-F sum_k X_k), one FP64 rounding of the sum.
__global__ void __launch_bounds__(256) spmv_fx_kernel(int64_t n, const int64_t* __restrict__ soff,
                                                      const int32_t* __restrict__ scol,
                                                      const uint8_t* __restrict__ slen,
                                                      const double* __restrict__ diag,
                                                      const double* __restrict__ x, const __int128* __restrict__ X,
                                                      double* __restrict__ y, double cF, const double* scale_dev,
                                                      const int* stop, int step) {
  if (stop) {
    const int st = *stop;
    if (st != 0 && st < step) return;
  }
  const double sc = scale_dev ? *scale_dev : 1.0;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += stride) {
    const __int128 acc = sell_row_sum(sell_row(soff, scol, r), __ldcs(slen + r), X);
    y[r] = sc * fma(cF, (double)acc, __ldcs(diag + r) * __ldg(x + r));
  }
}

// The product fused with the Lanczos step's three inner products (K1 + K2):
// w = s1 H V1 with V1 = x, then d1 = <V2, w>, d2 = <V1, w>, d3 = <V1, V2>,
// beta = s2 d1 and alpha = s1 (d2 - beta s2 d3), as lz_dots_kernel forms
// them.  V1[r] is already loaded for the diagonal term and the FP64 pipe is
// idle while the fixed-point gathers run, so the dots cost one extra 8-byte
// read per row.  Grid-stride rows on a resident grid, one block reduction per
// block, two-level grid reduction of the three sums.  Everything but the
// gathered fixed-point vector is loaded and stored with evict-first hints so
// that the 16-byte-per-row vector X stays in L2 for the gathers.
template <bool kHas2>
__global__ void __launch_bounds__(256, 6) spmv_fx_dots_kernel(
    int64_t n, const int64_t* __restrict__ soff, const int32_t* __restrict__ scol, const uint8_t* __restrict__ slen,
    const double* __restrict__ diag, const double* __restrict__ x, const __int128* __restrict__ X,
    const double* __restrict__ V2, double* __restrict__ y, double cF, const double* s1, const double* s2,
    const int* stop, int step, double* beta, double* alpha, Tri<double>* dots, GridRed<Tri<double>> red) {
  if (stop) {
    const int st = *stop;
    if (st != 0 && st < step) return;
  }
  const double sc = *s1;
  Tri<double> acc = vzero(Tri<double>{});
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += stride) {
    const __int128 s = sell_row_sum(sell_row(soff, scol, r), __ldcs(slen + r), X);
    const double xr = __ldcs(x + r);
    const double w = sc * fma(cF, (double)s, __ldcs(diag + r) * xr);
    __stcs(y + r, w);
    acc.b = fma(xr, w, acc.b);
    if (kHas2) {
      const double v2 = __ldcs(V2 + r);
      acc.a = fma(v2, w, acc.a);
      acc.c = fma(xr, v2, acc.c);
    }
  }
  if (grid_sum_ordered(acc, red, dots) && threadIdx.x == 0) {
    const Tri<double> d = *dots;
    const double bt = kHas2 ? (*s2) * d.a : 0.0;
    double t = d.b;
    if (kHas2) t = fma(-(bt * (*s2)), d.c, t);
    *beta = bt;
    *alpha = (*s1) * t;
  }
}

__global__ void sell_width_kernel(int64_t n, const int32_t* rowptr, int64_t* width, uint8_t* len) {
  const int64_t nsl = (n + 31) / 32;
  for (int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; s < nsl; s += (int64_t)gridDim.x * blockDim.x) {
    int w = 0;
    for (int64_t r = s * 32; r < std::min<int64_t>(n, s * 32 + 32); ++r) {
      const int l = rowptr[r + 1] - rowptr[r];
      len[r] = (uint8_t)l;
      w = max(w, l);
    }
    width[s] = (int64_t)((w + 3) / 4) * 128;  // groups of 4 entries per lane
  }
}

__global__ void sell_fill_kernel(int64_t n, const int32_t* rowptr, const int32_t* colidx, const int64_t* off,
                                 int32_t* scol) {
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
    const int64_t base = off[r >> 5] + 4 * (r & 31);
    for (int k = rowptr[r]; k < rowptr[r + 1]; ++k) {
      const int j = k - rowptr[r];
      scol[base + 128 * (int64_t)(j >> 2) + (j & 3)] = colidx[k];
    }
  }
}

// The slice layout from the row-ordered columns (rows hold at most 128 of them).
static void build_sell(Ctx* ctx, FxForm& f, int64_t n) {
  const int64_t nsl = (n + 31) / 32;
  f.sell_off.alloc(nsl + 1);
  f.sell_len.alloc(n + 32);
  DBuf<int64_t> width(nsl + 1);
  QD_CUDA(cudaMemsetAsync(width.p, 0, (nsl + 1) * 8, ctx->stream));
  sell_width_kernel<<<fx_grid(ctx, nsl), 256, 0, ctx->stream>>>(n, f.rowptr.p, width.p, f.sell_len.p);
  QD_CHECK_LAUNCH();
  QD_LAUNCHED(ctx);
  exclusive_scan_i64(ctx, width.p, f.sell_off.p, nsl + 1);
  int64_t total = 0;
  QD_CUDA(cudaMemcpyAsync(&total, f.sell_off.p + nsl, 8, cudaMemcpyDeviceToHost, ctx->stream));
  QD_CUDA(cudaStreamSynchronize(ctx->stream));
  f.sell_cols = total;
  f.sell_col.alloc(total + 128);
  QD_CUDA(cudaMemsetAsync(f.sell_col.p, 0, (total + 128) * 4, ctx->stream));
  sell_fill_kernel<<<fx_grid(ctx, n), 256, 0, ctx->stream>>>(n, f.rowptr.p, f.colidx.p, f.sell_off.p, f.sell_col.p);
  QD_CHECK_LAUNCH();
  QD_LAUNCHED(ctx);
  QD_CUDA(cudaStreamSynchronize(ctx->stream));
}

static int fx_dots_grid(Ctx* ctx, int64_t n) {
  static thread_local int per_sm = 0;
  if (!per_sm) {
    int a = 0, b = 0;
    QD_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a, spmv_fx_dots_kernel<true>, 256, 0));
    QD_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, spmv_fx_dots_kernel<false>, 256, 0));
    per_sm = std::max(1, std::min(a, b));
  }
  return (int)std::max<int64_t>(1, std::min<int64_t>(ceil_div(n, 256), (int64_t)ctx->num_sms * per_sm));
}

void launch_fx_dots(Ctx* ctx, const qd_ham* H, const FxForm& f, const double* x, const __int128* X,
                    const double* V2, double* y, const double* s1, const double* s2, const int* stop, int step,
                    double* beta, double* alpha, Tri<double>* dots, GridRed<Tri<double>> red) {
  const double cF = std::ldexp(f.c, -f.F);
  const int g = fx_dots_grid(ctx, H->dim);
  QD_REQUIRE(g <= kMaxGrid, QD_ERR_UNSUPPORTED, "reduction grid exceeds its partials buffer");
  if (f.blk_state > 0 && f.use_blk) {  // same grid: the same reduction tree as below
    launch_fx_block_dots(ctx, H, f, x, X, V2, y, s1, s2, stop, step, beta, alpha, dots, red, g);
    return;
  }
  if (f.slots_state > 0 && f.use_slots) {  // same grid: the same reduction tree as below
    launch_fx_slots_dots(ctx, H, f, x, X, V2, y, s1, s2, stop, step, beta, alpha, dots, red, g);
    return;
  }
  if (V2)
    spmv_fx_dots_kernel<true><<<g, 256, 0, ctx->stream>>>(H->dim, f.sell_off.p, f.sell_col.p, f.sell_len.p, f.diag.p,
                                                           x, X, V2, y, cF, s1, s2, stop, step, beta, alpha, dots,
                                                           red);
  else
    spmv_fx_dots_kernel<false><<<g, 256, 0, ctx->stream>>>(H->dim, f.sell_off.p, f.sell_col.p, f.sell_len.p, f.diag.p,
                                                            x, X, x, y, cF, s1, s1, stop, step, beta, alpha, dots,
                                                            red);
  QD_CHECK_LAUNCH();
  QD_LAUNCHED(ctx);
}

// Rows of the stored-column form for the one-launch step (fxstep.cuh).
struct SellRows {
  const int64_t* soff;
  const int32_t* scol;
  const uint8_t* slen;
  const __int128* X;
  __device__ const SellRows& bind(unsigned char*) const { return *this; }
  __device__ __int128 row_sum(int64_t r) const { return sell_row_sum(sell_row(soff, scol, r), __ldcs(slen + r), X); }
};

bool launch_fx_step(Ctx* ctx, const qd_ham* H, const FxForm& f, FxStepArgs a) {
  a.n = H->dim;
  a.diag = f.diag_zero ? nullptr : f.diag.p;  // no diagonal (e.g. the XY chain): nothing to read
  a.cF = std::ldexp(f.c, -f.F);
  a.F = f.F;
  const int g = fx_dots_grid(ctx, H->dim);
  bool ok = false;
  if (g <= kMaxGrid) {
    if (f.blk_state > 0 && f.use_blk)
      ok = launch_fx_block_step(ctx, H, f, a, g);
    else if (f.slots_state > 0 && f.use_slots)
      ok = launch_fx_slots_step(ctx, H, f, a, g);
    else
      ok = fx_step_launch(ctx, SellRows{f.sell_off.p, f.sell_col.p, f.sell_len.p, a.X}, a, g, 0);
  }
  f.step_fused = ok ? 1 : -1;
  return ok;
}

// <psi|H psi> for a psi whose imaginary part is 0 (State::eval, state.hpp:33-43, on a
// real ground state): (H psi)_r = c sum_k psi_k + d_r psi_r over the row's
// sliced columns, the gathered values summed in FP64 in the row's column order,
// and psi_r (H psi)_r summed over the grid in one pass.  Only the real halves of
// the gathered entries are read.  A row whose own psi_r carries an imaginary
// part sets *has_imag; the caller then takes the complex CSR product, so every
// entry is checked (each is some row's own).
__global__ void __launch_bounds__(256) fx_eval_real_kernel(int64_t n, const int64_t* __restrict__ soff,
                                                           const int32_t* __restrict__ scol,
                                                           const uint8_t* __restrict__ slen,
                                                           const double* __restrict__ diag, double c,
                                                           const cplx* __restrict__ psi, GridRed<double> red,
                                                           double* out, int* has_imag) {
  const double* pre = reinterpret_cast<const double*>(psi);  // psi[k].re at pre[2 k]
  double acc = 0.0;
  bool im = false;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += stride) {
    const int4* c4 = sell_row(soff, scol, r);
    const int e = __ldcs(slen + r);
    double s = 0.0;
    int4 cc = __ldcs(c4);
#pragma unroll 1
    for (int k = 0; k < e; k += 4) {
      int4 nc = cc;
      if (k + 4 < e) nc = __ldcs(c4 + 8 * (k + 4));
      double x0 = __ldg(pre + 2 * (int64_t)cc.x), x1 = 0.0, x2 = 0.0, x3 = 0.0;
      if (k + 1 < e) x1 = __ldg(pre + 2 * (int64_t)cc.y);
      if (k + 2 < e) x2 = __ldg(pre + 2 * (int64_t)cc.z);
      if (k + 3 < e) x3 = __ldg(pre + 2 * (int64_t)cc.w);
      s += (x0 + x1) + (x2 + x3);
      cc = nc;
    }
    const double2 p = __ldcs(reinterpret_cast<const double2*>(psi + r));
    im |= (p.y != 0.0);
    acc = fma(p.x, fma(c, s, __ldcs(diag + r) * p.x), acc);
  }
  if (im) *has_imag = 1;
  grid_sum(acc, red, out);
}

bool fx_eval_real(Ctx* ctx, const qd_ham* H, const FxForm& f, const cplx* psi, GridRed<double> red, double* out_dev,
                  int* flag_dev, double* value) {
  QD_CUDA(cudaMemsetAsync(flag_dev, 0, sizeof(int), ctx->stream));
  fx_eval_real_kernel<<<fx_dots_grid(ctx, H->dim), 256, 0, ctx->stream>>>(
      H->dim, f.sell_off.p, f.sell_col.p, f.sell_len.p, f.diag.p, f.c, psi, red, out_dev, flag_dev);
  QD_CHECK_LAUNCH();
  QD_LAUNCHED(ctx);
  struct {
    double v;
    int flag;
  } h{};
  QD_CUDA(cudaMemcpyAsync(&h.v, out_dev, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  QD_CUDA(cudaMemcpyAsync(&h.flag, flag_dev, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  QD_CUDA(cudaStreamSynchronize(ctx->stream));
  *value = h.v;
  return h.flag == 0;
}

// X = fixed-point copy of x (v_0 of a Lanczos run).
__global__ void fx_shadow_kernel(int64_t n, const double* x, __int128* X, int F, int* ovf) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    X[i] = fx_from_double(x[i], F, ovf);
}

void launch_fx(Ctx* ctx, const qd_ham* H, const FxForm& f, const double* x, const __int128* X, double* y,
               const double* scale_dev, const int* stop, int step) {
  if (f.blk_state > 0 && f.use_blk && !scale_dev && !stop) {  // the plain product (timing)
    launch_fx_block(ctx, H, f, x, X, y);
    return;
  }
  if (f.slots_state > 0 && f.use_slots) {
    launch_fx_slots(ctx, H, f, x, X, y, scale_dev, stop, step);
    return;
  }
  const double cF = std::ldexp(f.c, -f.F);
  spmv_fx_kernel<<<(unsigned)std::max<int64_t>(1, ceil_div(H->dim, 256)), 256, 0, ctx->stream>>>(
      H->dim, f.sell_off.p, f.sell_col.p, f.sell_len.p, f.diag.p, x, X, y, cF, scale_dev, stop, step);
  QD_CHECK_LAUNCH();
  QD_LAUNCHED(ctx);
}

void launch_fx_shadow(Ctx* ctx, int64_t n, const double* x, __int128* X, int F, int* ovf) {
  fx_shadow_kernel<<<fx_grid(ctx, n), 256, 0, ctx->stream>>>(n, x, X, F, ovf);
  QD_CHECK_LAUNCH();
  QD_LAUNCHED(ctx);
}

}  // namespace qd
