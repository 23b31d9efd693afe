// krylov.cu -- SpMV entry points, psi.eval, and the Lanczos ground state.
//
// Lanczos (Arnoldi::ArnoldiSolver<T, herm=1>, sparse_algorithm.hpp:395-425,
// 458-473, 514-585).  Step k = 1..kry_dim, with v1 = v_{k-1}, v2 = v_{k-2}:
//   K1  w = H v1                                  (the product alone)
//   K2  beta_k = <v2, w>, alpha_k = <v1, w - beta_k v2>   (one read of w, v1, v2)
//   K3  v_k = (w - beta_k v2) - alpha_k v1,  n_k = ||v_k||,  stop if n_k < 1e-10
// This is the reference's local orthogonalisation against the two previous
// vectors (no full reorthogonalisation), with its two subtractions in its
// order; alpha is expanded as <v1, w> - beta <v1, v2> so that w is read once
// and never rewritten.  The basis is stored unnormalised with 1 / n_k on the
// device.  The scalars stay on the device, so the whole recurrence is one
// CUDA graph with no host round trip; a breakdown sets a device flag that
// turns the remaining steps into no-ops.  The tridiagonal matrix
// tridiag(Re alpha, n) is solved on the host and the Ritz vector
// psi = sum_k y_k v_k is formed from the stored basis -- the values the
// reference's second Lanczos pass (getState<1>) regenerates, obtained without
// repeating the kry_dim products.
#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "fxstep.cuh"
#include "krylov.cuh"
#include "spmv.cuh"
#include "tridiag.cuh"

namespace qd {

constexpr int kVecThreads = 256;

static int vec_grid(Ctx* ctx, int64_t n) {
  const int64_t want = ceil_div(n, kVecThreads);
  return (int)std::max<int64_t>(1, std::min<int64_t>(want, (int64_t)ctx->num_sms * 8));
}


// ---------------------------------------------------------------- kernels
__device__ __forceinline__ bool stopped(const int* stop, int step) {
  if (!stop) return false;
  const int st = *stop;
  return st != 0 && st < step;
}

// The basis is stored unnormalised: V[k] = n_k v_k, with s_k = 1 / n_k kept on
// the device (s_0 = 1).  Every consumer folds s into its scalars, so no pass
// is spent rescaling a vector.  The two vector passes of a step read 16 bytes
// per load (two reals, or one complex) with two loads per operand in flight.
constexpr int kLzThreads = 256;
constexpr int kLzBlocksPerSm = 4;

static int lz_grid(Ctx* ctx, int64_t packs) {
  const int64_t want = ceil_div(packs, 2 * kLzThreads);
  return (int)std::max<int64_t>(1, std::min<int64_t>(want, (int64_t)ctx->num_sms * kLzBlocksPerSm));
}

// 16-byte packs: two reals or one complex element.
template <typename VV>
struct LzPack;
template <>
struct LzPack<double> {
  using T = double2;
  static constexpr int kPer = 2;
  __device__ static T load(const double* p, int64_t i) { return reinterpret_cast<const double2*>(p)[i]; }
  __device__ static T load_last(const double* p, int64_t i) { return __ldcs(reinterpret_cast<const double2*>(p) + i); }
  __device__ static void store(double* p, int64_t i, T v) { reinterpret_cast<double2*>(p)[i] = v; }
  __device__ static void store_stream(double* p, int64_t i, T v) { __stcs(reinterpret_cast<double2*>(p) + i, v); }
  __device__ static double dot(T a, T b, double acc) { return fma(a.y, b.y, fma(a.x, b.x, acc)); }
  __device__ static double nrm(T a, double acc) { return fma(a.y, a.y, fma(a.x, a.x, acc)); }
  __device__ static T submul(T x, double a, T y) { return make_double2(fma(-a, y.x, x.x), fma(-a, y.y, x.y)); }
  __device__ static void shadow(__int128* X, int64_t p, T v, int F, int* ovf) {
    X[2 * p] = fx_from_double(v.x, F, ovf);
    X[2 * p + 1] = fx_from_double(v.y, F, ovf);
  }
};
template <>
struct LzPack<cplx> {
  using T = cplx;
  static constexpr int kPer = 1;
  __device__ static T load(const cplx* p, int64_t i) { return p[i]; }
  __device__ static T load_last(const cplx* p, int64_t i) {
    const double2 d = __ldcs(reinterpret_cast<const double2*>(p) + i);
    return mkc(d.x, d.y);
  }
  __device__ static void store(cplx* p, int64_t i, T v) { p[i] = v; }
  __device__ static void store_stream(cplx* p, int64_t i, T v) { p[i] = v; }
  __device__ static cplx dot(T a, T b, cplx acc) { return vdotfma(a, b, acc); }
  __device__ static double nrm(T a, double acc) { return acc + vnorm2(a); }
  __device__ static T submul(T x, cplx a, T y) { return vsubmul(x, a, y); }
  __device__ static void shadow(__int128*, int64_t, T, int, int*) {}
};

__device__ __forceinline__ void shadow_one(__int128* X, int64_t i, double v, int F, int* ovf) {
  X[i] = fx_from_double(v, F, ovf);
}
__device__ __forceinline__ void shadow_one(__int128*, int64_t, cplx, int, int*) {}

// K2: the three inner products of step k from one read of w, V1, V2:
//   d1 = <V2, w>,  d2 = <V1, w>,  d3 = <V1, V2>
//   beta  = s2 d1                   = <v2, w>
//   alpha = s1 (d2 - beta s2 d3)    = <v1, w - beta v2>
// alpha is the reference's <v1, w> taken after w -= beta v2
// (sparse_algorithm.hpp:405-415), expanded so that w is read once and not
// written.  For k = 1 there is no V2 and beta = 0.
template <typename VV, bool kHas2>
__global__ void __launch_bounds__(kLzThreads, kLzBlocksPerSm)
    lz_dots_kernel(int64_t n, const int* stop, int step, const VV* __restrict__ w, const VV* __restrict__ V1,
                   const VV* __restrict__ V2, const double* s1, const double* s2, VV* beta, VV* alpha,
                   Tri<VV>* dots, GridRed<Tri<VV>> red) {
  if (stopped(stop, step)) return;
  using P = LzPack<VV>;
  const int64_t np = n / P::kPer;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  Tri<VV> acc0 = vzero(Tri<VV>{});
  int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  for (; p + stride < np; p += 2 * stride) {
    const typename P::T w0 = P::load(w, p), w1 = P::load(w, p + stride);
    const typename P::T a0 = P::load(V1, p), a1 = P::load(V1, p + stride);
    acc0.b = P::dot(a1, w1, P::dot(a0, w0, acc0.b));
    if (kHas2) {
      const typename P::T b0 = P::load(V2, p), b1 = P::load(V2, p + stride);
      acc0.a = P::dot(b1, w1, P::dot(b0, w0, acc0.a));
      acc0.c = P::dot(a1, b1, P::dot(a0, b0, acc0.c));
    }
  }
  if (p < np) {
    const typename P::T w0 = P::load(w, p), a0 = P::load(V1, p);
    acc0.b = P::dot(a0, w0, acc0.b);
    if (kHas2) {
      const typename P::T b0 = P::load(V2, p);
      acc0.a = P::dot(b0, w0, acc0.a);
      acc0.c = P::dot(a0, b0, acc0.c);
    }
  }
  if (P::kPer == 2 && (n & 1) && blockIdx.x == 0 && threadIdx.x == 0) {  // odd real length: last element
    acc0.b = vdotfma(V1[n - 1], w[n - 1], acc0.b);
    if (kHas2) {
      acc0.a = vdotfma(V2[n - 1], w[n - 1], acc0.a);
      acc0.c = vdotfma(V1[n - 1], V2[n - 1], acc0.c);
    }
  }
  if (grid_sum(acc0, red, dots) && threadIdx.x == 0) {
    const Tri<VV> d = *dots;
    const VV b = kHas2 ? vscale(*s2, d.a) : vzero(VV{});
    VV t = d.b;
    if (kHas2) t = vsubmul(t, vscale(*s2, b), d.c);
    *beta = b;
    *alpha = vscale(*s1, t);
  }
}

// K3: V[k] = (w - (beta s2) V2) - (alpha s1) V1   (the reference's two
// subtractions in its order);  n_k = ||V[k]||, s_k = 1 / n_k, stop if n_k < 1e-10.
// kShadow: also write the fixed-point copy X of V[k] that the next product
// gathers (with evict-first stores of V[k], so that X stays in L2), and raise
// *ovf once if an element left the fixed-point range.
template <typename VV, bool kHas2, bool kShadow>
__global__ void __launch_bounds__(kLzThreads, kLzBlocksPerSm)
    lz_update_kernel(int64_t n, int* stop, int step, const VV* __restrict__ w, const VV* __restrict__ V1,
                     const VV* __restrict__ V2, const double* s1, const double* s2, const VV* alpha,
                     const VV* beta, VV* __restrict__ Vk, double* nrm2, double* nrm, double* sk,
                     GridRed<double> red, __int128* Xk, int F, int* ovf) {
  if (stopped(stop, step)) return;
  using P = LzPack<VV>;
  const VV a = vscale(*s1, *alpha);
  const VV b = kHas2 ? vscale(*s2, *beta) : vzero(VV{});
  const int64_t np = n / P::kPer;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  double acc0 = 0.0, acc1 = 0.0;
  int out = 0;
  int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  for (; p + stride < np; p += 2 * stride) {
    typename P::T o0 = P::load_last(w, p), o1 = P::load_last(w, p + stride);
    const typename P::T a0 = P::load(V1, p), a1 = P::load(V1, p + stride);
    if (kHas2) {
      const typename P::T b0 = P::load_last(V2, p), b1 = P::load_last(V2, p + stride);
      o0 = P::submul(o0, b, b0);
      o1 = P::submul(o1, b, b1);
    }
    o0 = P::submul(o0, a, a0);
    o1 = P::submul(o1, a, a1);
    if (kShadow) {
      P::store_stream(Vk, p, o0);
      P::store_stream(Vk, p + stride, o1);
      P::shadow(Xk, p, o0, F, &out);
      P::shadow(Xk, p + stride, o1, F, &out);
    } else {
      P::store(Vk, p, o0);
      P::store(Vk, p + stride, o1);
    }
    acc0 = P::nrm(o0, acc0);
    acc1 = P::nrm(o1, acc1);
  }
  if (p < np) {
    typename P::T o0 = P::load_last(w, p);
    if (kHas2) o0 = P::submul(o0, b, P::load_last(V2, p));
    o0 = P::submul(o0, a, P::load(V1, p));
    P::store(Vk, p, o0);
    if (kShadow) P::shadow(Xk, p, o0, F, &out);
    acc0 = P::nrm(o0, acc0);
  }
  if (P::kPer == 2 && (n & 1) && blockIdx.x == 0 && threadIdx.x == 0) {
    VV o = w[n - 1];
    if (kHas2) o = vsubmul(o, b, V2[n - 1]);
    o = vsubmul(o, a, V1[n - 1]);
    Vk[n - 1] = o;
    if (kShadow) shadow_one(Xk, n - 1, o, F, &out);
    acc0 += vnorm2(o);
  }
  if (kShadow && out) *ovf = 1;
  double n2 = 0.0;
  if (grid_sum(acc0 + acc1, red, nrm2, &n2) && threadIdx.x == 0) {
    const double nr = sqrt(n2);
    *nrm = nr;
    *sk = 1.0 / nr;
    if (nr < 1e-10 && stop && *stop == 0) *stop = step;  // sparse_algorithm.hpp:421
  }
}

// One Lanczos step's two vector passes (after K1 has written w = s1 H V1).
template <typename VV>
static void lz_vector_passes(Ctx* ctx, int64_t n, int* stop, int step, const VV* w, const VV* V1, const VV* V2,
                             const double* s1, const double* s2, VV* beta, VV* alpha, Tri<VV>* dots, VV* Vk,
                             double* nrm2, double* nrm, double* sk, GridRed<Tri<VV>> rt, GridRed<double> rd,
                             __int128* Xk = nullptr, int F = 0, int* ovf = nullptr, bool dots_done = false) {
  const int g = lz_grid(ctx, n / LzPack<VV>::kPer + 1);
  if (V2) {
    if (!dots_done) {
      lz_dots_kernel<VV, true><<<g, kLzThreads, 0, ctx->stream>>>(n, stop, step, w, V1, V2, s1, s2, beta, alpha,
                                                                  dots, rt);
      QD_CHECK_LAUNCH();
      QD_LAUNCHED(ctx);
    }
    if (Xk)
      lz_update_kernel<VV, true, true><<<g, kLzThreads, 0, ctx->stream>>>(n, stop, step, w, V1, V2, s1, s2, alpha,
                                                                          beta, Vk, nrm2, nrm, sk, rd, Xk, F, ovf);
    else
      lz_update_kernel<VV, true, false><<<g, kLzThreads, 0, ctx->stream>>>(n, stop, step, w, V1, V2, s1, s2, alpha,
                                                                           beta, Vk, nrm2, nrm, sk, rd, Xk, F, ovf);
  } else {
    if (!dots_done) {
      lz_dots_kernel<VV, false><<<g, kLzThreads, 0, ctx->stream>>>(n, stop, step, w, V1, V1, s1, s1, beta, alpha,
                                                                   dots, rt);
      QD_CHECK_LAUNCH();
      QD_LAUNCHED(ctx);
    }
    if (Xk)
      lz_update_kernel<VV, false, true><<<g, kLzThreads, 0, ctx->stream>>>(n, stop, step, w, V1, V1, s1, s1, alpha,
                                                                           beta, Vk, nrm2, nrm, sk, rd, Xk, F, ovf);
    else
      lz_update_kernel<VV, false, false><<<g, kLzThreads, 0, ctx->stream>>>(n, stop, step, w, V1, V1, s1, s1,
                                                                            alpha, beta, Vk, nrm2, nrm, sk, rd, Xk,
                                                                            F, ovf);
  }
  QD_CHECK_LAUNCH();
  QD_LAUNCHED(ctx);
}

// ||psi||^2 of a complex column, and whether its imaginary part vanishes.
__global__ void __launch_bounds__(kVecThreads) colnorm_kernel(int64_t n, const cplx* psi, double* nrm2,
                                                              GridRed<double> red, int* has_imag) {
  double acc = 0.0;
  bool im = false;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const cplx p = psi[i];
    acc = fma(p.re, p.re, fma(p.im, p.im, acc));
    im |= (p.im != 0.0);
  }
  if (im) atomicOr(has_imag, 1);
  grid_sum(acc, red, nrm2);
}

__device__ __forceinline__ void store_from(double& dst, cplx v) { dst = v.re; }
__device__ __forceinline__ void store_from(cplx& dst, cplx v) { dst = v; }

// v0 = psi / ||psi||  (initKrylov, sparse_algorithm.hpp:514-519)
template <typename VV>
__global__ void __launch_bounds__(kVecThreads) init_v0_kernel(int64_t n, const cplx* psi, const double* nrm2,
                                                              VV* v0) {
  const double inv = 1.0 / sqrt(*nrm2);
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const cplx p = psi[i];
    store_from(v0[i], mkc(p.re * inv, p.im * inv));
  }
}

__device__ __forceinline__ cplx to_c(double v) { return mkc(v, 0.0); }
__device__ __forceinline__ cplx to_c(cplx v) { return v; }

// psi = sum_{k < act} y_k V[k], accumulated in k order per element.
template <typename VV>
__global__ void __launch_bounds__(kVecThreads) ritz_kernel(int64_t n, const VV* V, int64_t ld, const double* y,
                                                           int act, cplx* psi) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    VV acc = vscale(y[0], V[i]);
    for (int k = 1; k < act; ++k) acc = vfma(y[k], V[(int64_t)k * ld + i], acc);
    psi[i] = to_c(acc);
  }
}

// <a, b> over complex columns (a^dagger b).
__global__ void __launch_bounds__(kVecThreads) cdot_kernel(int64_t n, const cplx* a, const cplx* b, cplx* out,
                                                           GridRed<cplx> red) {
  cplx acc = mkc(0.0, 0.0);
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    acc = vdotfma(a[i], b[i], acc);
  grid_sum(acc, red, out);
}

Workspace::Workspace(Ctx* c) : ctx(c) {
  partials_d.alloc(kMaxGrid);
  partials_c.alloc(kMaxGrid);
  partials_td.alloc(kMaxGrid);
  partials_tc.alloc(kMaxGrid);
  gpart_td.alloc(kRedMaxGroups);
  gpart_tc.alloc(kRedMaxGroups);
  gpart_d.alloc(kRedMaxGroups);
  gpart_c.alloc(kRedMaxGroups);
  tickets.alloc(8 * (1 + kRedMaxGroups));
  QD_CUDA(cudaMemsetAsync(tickets.p, 0, tickets.bytes(), c->stream));
}

GridRed<double> Workspace::red_d(int slot) {
  return GridRed<double>{partials_d.p, tickets.p + (size_t)slot * (1 + kRedMaxGroups), gpart_d.p};
}
// One-level form (the last block adds every block partial): for grids of a
// few hundred blocks it saves a fence-and-ticket round on the critical tail.
GridRed<double> Workspace::red_d_flat(int slot) {
  return GridRed<double>{partials_d.p, tickets.p + (size_t)slot * (1 + kRedMaxGroups), nullptr};
}
GridRed<cplx> Workspace::red_c(int slot) {
  return GridRed<cplx>{partials_c.p, tickets.p + (size_t)slot * (1 + kRedMaxGroups), gpart_c.p};
}

Workspace& ham_workspace(qd_ham* H) {
  if (!H->ws) H->ws.reset(new Workspace(H->ctx));
  return *H->ws;
}

// y = H x on complex columns.
void ham_apply_c(qd_ham* H, const cplx* x, cplx* y) {
  Workspace& W = ham_workspace(H);
  if (H->flags & QD_HAM_REAL)
    launch_spmv<double, cplx>(H->ctx, H, H->vals_r.p, x, y, 1.0, nullptr, W.red_c(0), nullptr, nullptr, 0, -1);
  else
    launch_spmv<cplx, cplx>(H->ctx, H, H->vals_c.p, x, y, 1.0, nullptr, W.red_c(0), nullptr, nullptr, 0, -1);
}

cplx state_eval(qd_ham* H, const cplx* psi) {
  Ctx* ctx = H->ctx;
  Workspace& W = ham_workspace(H);
  // a real state on an operator whose uniform-coupling form is built (by a solve
  // on it): the sliced columns, no stored values read
  if ((H->flags & QD_HAM_REAL) && H->fx_allowed && H->fx_state > 0 && H->fx) {
    if (!W.eval_real.p) W.eval_real.alloc(1);
    if (!W.eval_flag.p) W.eval_flag.alloc(1);
    double v = 0.0;
    if (fx_eval_real(ctx, H, *H->fx, psi, W.red_d(0), W.eval_real.p, W.eval_flag.p, &v)) return mkc(v, 0.0);
  }
  if (W.eval_y.n < (size_t)H->dim + 1) W.eval_y.alloc(H->dim + 1);
  if (!W.eval_out.p) W.eval_out.alloc(1);
  // psi^dagger (H psi): the product and the dot in one pass
  if (H->flags & QD_HAM_REAL)
    launch_spmv<double, cplx>(ctx, H, H->vals_r.p, psi, W.eval_y.p, 1.0, psi, W.red_c(0), W.eval_out.p, nullptr, 0,
                              -1);
  else
    launch_spmv<cplx, cplx>(ctx, H, H->vals_c.p, psi, W.eval_y.p, 1.0, psi, W.red_c(0), W.eval_out.p, nullptr, 0,
                            -1);
  cplx h;
  QD_CUDA(cudaMemcpyAsync(&h, W.eval_out.p, sizeof(cplx), cudaMemcpyDeviceToHost, ctx->stream));
  QD_CUDA(cudaStreamSynchronize(ctx->stream));
  return h;
}

// <psi|O_i|psi> for a list of operators (McManager::incrAllObs,
// mc_manager.hpp:88-106): every product is fused with its inner product and
// the launches go back to back on one stream, with one copy of all results.
void obs_eval_many(qd_ham* const* obs, int nobs, const cplx* psi, cplx* out_host) {
  Ctx* ctx = obs[0]->ctx;
  const int64_t n = obs[0]->dim;
  DBuf<cplx> tmp(n + 1);
  DBuf<cplx> out(nobs);
  for (int i = 0; i < nobs; ++i) {
    qd_ham* H = obs[i];
    QD_REQUIRE(H->ctx == ctx && H->dim == n, QD_ERR_INVALID, "observable %d: other context or dimension", i);
    Workspace& W = ham_workspace(H);
    if (H->flags & QD_HAM_REAL)
      launch_spmv<double, cplx>(ctx, H, H->vals_r.p, psi, tmp.p, 1.0, psi, W.red_c(0), out.p + i, nullptr, 0, -1);
    else
      launch_spmv<cplx, cplx>(ctx, H, H->vals_c.p, psi, tmp.p, 1.0, psi, W.red_c(0), out.p + i, nullptr, 0, -1);
  }
  QD_CUDA(cudaMemcpyAsync(out_host, out.p, nobs * sizeof(cplx), cudaMemcpyDeviceToHost, ctx->stream));
  QD_CUDA(cudaStreamSynchronize(ctx->stream));
}

// ||psi||^2 on the Hamiltonian's stream.
double state_norm2(qd_ham* H, const cplx* psi) {
  Ctx* ctx = H->ctx;
  Workspace& W = ham_workspace(H);
  DBuf<double> nrm2(1);
  DBuf<int> has_im(1);
  QD_CUDA(cudaMemsetAsync(has_im.p, 0, sizeof(int), ctx->stream));
  colnorm_kernel<<<vec_grid(ctx, H->dim), kVecThreads, 0, ctx->stream>>>(H->dim, psi, nrm2.p, W.red_d(0), has_im.p);
  QD_CHECK_LAUNCH();
  QD_LAUNCHED(ctx);
  double h = 0.0;
  QD_CUDA(cudaMemcpyAsync(&h, nrm2.p, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  QD_CUDA(cudaStreamSynchronize(ctx->stream));
  return h;
}

// psi^dagger psi and psi^dagger H psi with one wait for both (a served result).
void state_norm2_eval(qd_ham* H, const cplx* psi, double* n2, cplx* e) {
  Ctx* ctx = H->ctx;
  Workspace& W = ham_workspace(H);
  DBuf<char> out(64);
  DBuf<cplx> tmp(H->dim + 1);
  double* nrm2 = reinterpret_cast<double*>(out.p);
  int* has_im = reinterpret_cast<int*>(out.p + 8);
  cplx* hv = reinterpret_cast<cplx*>(out.p + 16);
  QD_CUDA(cudaMemsetAsync(has_im, 0, sizeof(int), ctx->stream));
  colnorm_kernel<<<vec_grid(ctx, H->dim), kVecThreads, 0, ctx->stream>>>(H->dim, psi, nrm2, W.red_d(0), has_im);
  QD_CHECK_LAUNCH();
  QD_LAUNCHED(ctx);
  if (H->flags & QD_HAM_REAL)
    launch_spmv<double, cplx>(ctx, H, H->vals_r.p, psi, tmp.p, 1.0, psi, W.red_c(0), hv, nullptr, 0, -1);
  else
    launch_spmv<cplx, cplx>(ctx, H, H->vals_c.p, psi, tmp.p, 1.0, psi, W.red_c(0), hv, nullptr, 0, -1);
  char host[32];
  QD_CUDA(cudaMemcpyAsync(host, out.p, sizeof(host), cudaMemcpyDeviceToHost, ctx->stream));
  QD_CUDA(cudaStreamSynchronize(ctx->stream));
  std::memcpy(n2, host, sizeof(double));
  std::memcpy(e, host + 16, sizeof(cplx));
}

// The product the real Lanczos path launches, timed back to back.
// The one-launch step of the uniform-coupling form is the default;
// QD_LANCZOS_STEP=split keeps the product and the update in two launches.
// (read per run; a captured recurrence keeps the form it was captured with)
static bool fx_one_launch_step() {
  const char* e = std::getenv("QD_LANCZOS_STEP");
  return !(e && std::strcmp(e, "split") == 0);
}

// Test control of the one-launch step's bounded grid barrier:
// QD_STEP_WAIT_OUT=<polls> (1 .. 2^20) keeps the publishing block from
// publishing alpha and beta and lets every block give up after <polls> polls, so each step's
// wait runs out and the solve returns QD_ERR_TIMEOUT with the kernel finished.
// Read per solve; 0 when unset.
static unsigned step_wait_out_polls() {
  const char* e = std::getenv("QD_STEP_WAIT_OUT");
  if (!e) return 0;
  const long v = std::strtol(e, nullptr, 10);
  return v > 0 ? (unsigned)std::min<long>(v, 1L << 20) : 0u;
}

// The epoch to 0 and every mailbox entry to kMboxEmpty (once per Lanczos run,
// so that a run does not depend on what earlier runs left).
__global__ void step_mbox_reset_kernel(unsigned* epoch, double* mbox) {
  for (int i = threadIdx.x; i < kMboxDoubles; i += blockDim.x) mbox[i] = __longlong_as_double(kMboxEmpty);
  if (threadIdx.x == 0) *epoch = 0u;
}

// Overflow flag of a fixed-point run (nonzero: rerun on the FP64 product);
// a bounded device wait that ran out is an error.
static int fx_flags(Ctx* ctx, const int* flags) {
  int f[2] = {0, 0};
  QD_CUDA(cudaMemcpyAsync(f, flags, sizeof(f), cudaMemcpyDeviceToHost, ctx->stream));
  QD_CUDA(cudaStreamSynchronize(ctx->stream));
  QD_REQUIRE(!f[1], QD_ERR_TIMEOUT, "a Lanczos step's blocks did not meet within the wait limit");
  return f[0];
}

void time_spmv(qd_ham* H, int spmv, int iters, double* avg_ms, double* bytes_per_launch) {
  Ctx* ctx = H->ctx;
  Workspace& W = ham_workspace(H);
  const int64_t n = H->dim;
  const bool real = (H->flags & QD_HAM_REAL) != 0;
  const size_t vb = real ? sizeof(double) : sizeof(cplx);
  DBuf<char> x((n + 32) * vb), y((n + 32) * vb);
  QD_CUDA(cudaMemsetAsync(x.p, 0, x.bytes(), ctx->stream));
  // diagnostic codes: 2000 + kernel = product with the fused Lanczos dot;
  // 3001 / 3002 = the Lanczos vector kernels K2 / K3 alone (real path)
  const int mode = spmv >= 3000 ? 3 : (spmv >= 2000 ? 2 : 1);
  const int code = spmv % 1000;
  const int variant = (mode == 2) ? spmv - 2000 : ((spmv >= kSpmvTile && mode == 1) ? spmv : -1);
  DBuf<char> z((n + 32) * vb), t((n + 32) * vb), scal(128);
  QD_CUDA(cudaMemsetAsync(z.p, 0, z.bytes(), ctx->stream));
  QD_CUDA(cudaMemsetAsync(scal.p, 0, 128, ctx->stream));
  const double one = 1.0;
  QD_CUDA(cudaMemcpyAsync(scal.p, &one, sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
  const double* s1 = (const double*)scal.p;
  const bool mf = (spmv == QD_SPMV_MATRIX_FREE);
  if (mf) ham_build_matrix_free(H);
  // code 1: what the matrix-free Lanczos path launches (the slot form with its dots where it applies)
  const bool mfx = mf && real && H->fx_allowed && ham_build_mf_fx(H);
  // code 0: the product the real Lanczos path launches (the fixed-point form when it applies)
  const bool fxcode = spmv == kSpmvFx || spmv == kSpmvFxSlots || spmv == kSpmvFxBlock;
  const bool fx = real && (fxcode || (spmv == QD_SPMV_CSR && H->fx_allowed)) && ham_build_fx(H);
  QD_REQUIRE(!fxcode || fx, QD_ERR_UNSUPPORTED, "the fixed-point form does not apply to this operator");
  QD_REQUIRE(spmv != kSpmvFxSlots || ham_build_fx_slots(H), QD_ERR_UNSUPPORTED,
             "the columns of this operator cannot be computed on the fly (code 121)");
  QD_REQUIRE(spmv != kSpmvFxBlock || ham_build_fx_block(H), QD_ERR_UNSUPPORTED,
             "this sector or operator has no block layout (code 122)");
  struct SlotChoice {  // 120 / 121 / 122 pick the column source for this timing only
    FxForm* f;
    bool saved, saved_blk;
    ~SlotChoice() {
      if (f) {
        f->use_slots = saved;
        f->use_blk = saved_blk;
      }
    }
  } choice{fx ? H->fx.get() : nullptr, fx ? H->fx->use_slots : true, fx ? H->fx->use_blk : false};
  if (fx && fxcode) {
    H->fx->use_slots = (spmv == kSpmvFxSlots);
    H->fx->use_blk = (spmv == kSpmvFxBlock);
  }
  const bool slots = fx && H->fx->use_slots && H->fx->slots_state > 0;
  const bool blk = fx && H->fx->use_blk && H->fx->blk_state > 0;
  DBuf<__int128> X((fx || mfx) ? n + 32 : 1);
  if (fx || mfx) QD_CUDA(cudaMemsetAsync(X.p, 0, X.bytes(), ctx->stream));
  // what the Lanczos recurrence launches on the uniform-coupling form: the
  // whole step in one launch (product, dots, update, fixed-point copy, norm)
  const FxForm* step_form = mfx ? H->mfx.get() : ((fx && spmv == QD_SPMV_CSR) ? H->fx.get() : nullptr);
  if (!fx_one_launch_step()) step_form = nullptr;
  DBuf<__int128> X2(step_form ? n + 32 : 1);
  DBuf<unsigned> ep(4);
  DBuf<double> mb(kMboxDoubles);
  DBuf<int> flags(2);
  step_mbox_reset_kernel<<<1, 128, 0, ctx->stream>>>(ep.p, mb.p);
  QD_CHECK_LAUNCH();
  QD_CUDA(cudaMemsetAsync(flags.p, 0, 2 * sizeof(int), ctx->stream));
  bool stepped = false;
  auto launch = [&]() {
    if (step_form) {
      double* d = (double*)scal.p;
      FxStepArgs a{};
      a.x = (const double*)x.p;
      a.X = X.p;
      a.V2 = (const double*)z.p;
      a.s1 = s1;
      a.s2 = s1;
      a.beta = d + 1;
      a.alpha = d + 2;
      a.dots = reinterpret_cast<Tri<double>*>(d + 6);
      a.red = W.red_tri<double>(2);
      a.epoch = ep.p;
      a.mbox = mb.p;
      a.Vk = (double*)t.p;
      a.nrm2 = d + 3;
      a.nrm = d + 4;
      a.sk = d + 5;
      a.rd = W.red_d_flat(3);
      a.Xk = X2.p;
      a.ovf = flags.p;
      stepped = launch_fx_step(ctx, H, *step_form, a);
      if (stepped) return;
    }
    if (mfx) {
      double* d = (double*)scal.p;
      launch_fx_dots(ctx, H, *H->mfx, (const double*)x.p, X.p, (const double*)z.p, (double*)y.p, s1, s1, nullptr,
                     0, d + 1, d + 2, reinterpret_cast<Tri<double>*>(d + 6), W.red_tri<double>(2));
      return;
    }
    if (fx && spmv == QD_SPMV_CSR) {  // what the recurrence launches: the product fused with its dots
      double* d = (double*)scal.p;
      launch_fx_dots(ctx, H, *H->fx, (const double*)x.p, X.p, (const double*)z.p, (double*)y.p, s1, s1, nullptr, 0,
                     d + 1, d + 2, reinterpret_cast<Tri<double>*>(d + 6), W.red_tri<double>(2));
      return;
    }
    if (fx) {
      launch_fx(ctx, H, *H->fx, (const double*)x.p, X.p, (double*)y.p, nullptr, nullptr, 0);
      return;
    }
    if (mf) {
      if (H->mf_real && real)
        launch_mf<double>(ctx, H, (const double*)x.p, (double*)y.p, 1.0, nullptr, nullptr, 0);
      else
        launch_mf<cplx>(ctx, H, (const cplx*)x.p, (cplx*)y.p, 1.0, nullptr, nullptr, 0);
      return;
    }
    if (mode == 3) {
      QD_REQUIRE(real, QD_ERR_UNSUPPORTED, "vector-kernel timing is for real Hamiltonians");
      double* d = (double*)scal.p;
      const int g = lz_grid(ctx, n / 2 + 1);
      if (code == 1)
        lz_dots_kernel<double, true><<<g, kLzThreads, 0, ctx->stream>>>(
            n, nullptr, 0, (const double*)y.p, (const double*)x.p, (const double*)z.p, s1, s1, d + 1, d + 2,
            reinterpret_cast<Tri<double>*>(d + 6), W.red_tri<double>(2));
      else
        lz_update_kernel<double, true, false><<<g, kLzThreads, 0, ctx->stream>>>(
            n, nullptr, 0, (const double*)y.p, (const double*)x.p, (const double*)z.p, s1, s1, d + 1, d + 2,
            (double*)t.p, d + 3, d + 4, d + 5, W.red_d(3), nullptr, 0, nullptr);
      QD_CHECK_LAUNCH();
      QD_LAUNCHED(ctx);
      return;
    }
    const bool dot = (mode == 2);
    if (real)
      launch_spmv<double, double>(ctx, H, H->vals_r.p, (const double*)x.p, (double*)y.p, 1.0,
                                  dot ? (const double*)z.p : nullptr, W.red_d(1), dot ? (double*)scal.p + 6 : nullptr,
                                  nullptr, 0, variant, dot ? s1 : nullptr, dot ? s1 : nullptr);
    else
      launch_spmv<cplx, cplx>(ctx, H, H->vals_c.p, (const cplx*)x.p, (cplx*)y.p, 1.0,
                              dot ? (const cplx*)z.p : nullptr, W.red_c(1), dot ? (cplx*)scal.p + 2 : nullptr,
                              nullptr, 0, variant, dot ? s1 : nullptr, dot ? s1 : nullptr);
  };
  for (int i = 0; i < 3; ++i) launch();
  QD_CUDA(cudaEventRecord(ctx->events[14], ctx->stream));
  for (int i = 0; i < iters; ++i) launch();
  QD_CUDA(cudaEventRecord(ctx->events[15], ctx->stream));
  QD_CUDA(cudaEventSynchronize(ctx->events[15]));
  float ms = 0.f;
  QD_CUDA(cudaEventElapsedTime(&ms, ctx->events[14], ctx->events[15]));
  *avg_ms = (double)ms / iters;
  const double mvb = real ? 8.0 : 16.0;
  *bytes_per_launch = (double)H->nnz * (mvb + 4.0) + (double)(n + 1) * 8.0 + (double)n * 2.0 * (double)vb;
  if (mf)  // basis word, diagonal, x[r], y[r] per row (the gathered x comes from L2)
    *bytes_per_launch = (double)n * (8.0 + (H->mf_real ? 8.0 : 16.0) + 2.0 * (double)vb);
  if (mfx)  // 32-bit state, diagonal, x, its fixed-point copy once, y, v2
    *bytes_per_launch = (double)n * (4.0 + 8.0 + 8.0 + 16.0 + 8.0 + 8.0);
  if (fx)  // slice columns (padding included), slice offsets, row counts, diagonal, x, its fixed-point copy, y
           // (+ v2 for the fused dots)
    *bytes_per_launch = (double)H->fx->sell_cols * 4.0 + (double)((n + 31) / 32 + 1) * 8.0 + (double)n +
                        (double)n * (8.0 + 8.0 + 16.0 + 8.0 + (spmv == QD_SPMV_CSR ? 8.0 : 0.0));
  if (slots || blk)  // 32-bit state, diagonal, x, its fixed-point copy once, y (+ v2)
    *bytes_per_launch = (double)n * (4.0 + 8.0 + 8.0 + 16.0 + 8.0 + (spmv == QD_SPMV_CSR ? 8.0 : 0.0));
  if (stepped)  // one Lanczos step: w stays on chip; v_k and its fixed-point copy are written
    *bytes_per_launch += (double)n * (8.0 + 16.0 - 8.0);
  int fl[2] = {0, 0};
  QD_CUDA(cudaMemcpyAsync(fl, flags.p, sizeof(fl), cudaMemcpyDeviceToHost, ctx->stream));
  QD_CUDA(cudaStreamSynchronize(ctx->stream));
  QD_REQUIRE(!fl[1], QD_ERR_TIMEOUT, "a timed step's blocks did not meet within the wait limit");
}

// ---------------------------------------------------------------- Lanczos
template <typename MV, typename VV>
// fxk: 0 the product alone (CSR or matrix-free), then K2; 1 the uniform-
// coupling form with fixed-point sums fused with the step's inner products.
static void lanczos_run(qd_ham* H, const MV* vals, LanczosBuffers<VV>& B, int k_first, int k_last, Workspace& W,
                        bool mf, int fxk = 0, const FxForm* form = nullptr) {
  Ctx* ctx = H->ctx;
  const int64_t n = H->dim;
  // requests of the serving loop share the device with other lanes' kernels,
  // and a cooperative launch waits for room for its whole grid: they keep the
  // two-launch step
  const bool one_launch = fxk == 1 && fx_one_launch_step() && !H->one_shot;
  if (fxk == 1 && !one_launch) form->step_fused = -1;
  // the step's epoch and mailbox start every run empty
  if (one_launch) {
    step_mbox_reset_kernel<<<1, 128, 0, ctx->stream>>>(B.epoch.p, B.mbox.p);
    QD_CHECK_LAUNCH();
    QD_LAUNCHED(ctx);
  }
  for (int k = k_first; k <= k_last; ++k) {
    const VV* V1 = B.V.p + (int64_t)(k - 1) * B.ld;
    const VV* V2 = (k >= 2) ? B.V.p + (int64_t)(k - 2) * B.ld : nullptr;
    VV* Vk = B.V.p + (int64_t)k * B.ld;
    const double* s1 = B.scl.p + (k - 1);
    const double* s2 = (k >= 2) ? B.scl.p + (k - 2) : nullptr;
    // K1: w = s1 * H V1 (CSR, fixed-point uniform-coupling form, or matrix-free)
    __int128* Xprev = (fxk == 1) ? B.X.p + (int64_t)((k - 1) & 1) * B.ld : nullptr;
    __int128* Xnext = (fxk == 1) ? B.X.p + (int64_t)(k & 1) * B.ld : nullptr;
    if constexpr (std::is_same<VV, double>::value) {
      if (one_launch) {  // the whole step in one launch (fxstep.cuh)
        FxStepArgs a{};
        a.x = V1;
        a.X = Xprev;
        a.V2 = V2;
        a.s1 = s1;
        a.s2 = s2;
        a.stop = B.stop.p;
        a.step = k;
        a.beta = B.beta.p + k;
        a.alpha = B.alpha.p + k;
        a.dots = B.dots.p + k;
        a.red = W.red_tri<double>(2);
        a.epoch = B.epoch.p;
        a.mbox = B.mbox.p;
        a.Vk = Vk;
        a.nrm2 = B.nrm2.p + k;
        a.nrm = B.nrm.p + k;
        a.sk = B.scl.p + k;
        a.rd = W.red_d_flat(3);
        a.Xk = Xnext;
        a.ovf = B.ovf.p;
        a.spin_limit = step_wait_out_polls();
        a.hold_publish = a.spin_limit != 0;
        if (launch_fx_step(ctx, H, *form, a)) continue;
      }
      if (fxk == 1)  // product fused with the step's inner products, then the update
        launch_fx_dots(ctx, H, *form, V1, Xprev, V2, B.w.p, s1, s2, B.stop.p, k, B.beta.p + k, B.alpha.p + k,
                       B.dots.p + k,
                       W.red_tri<double>(2));
    }
    if (fxk == 0) {
      if (mf)
        launch_mf<VV>(ctx, H, V1, B.w.p, 1.0, s1, B.stop.p, k);
      else
        launch_spmv<MV, VV>(ctx, H, vals, V1, B.w.p, 1.0, nullptr, W.red_c_or_d<VV>(1), nullptr, B.stop.p, k, -1,
                            s1, nullptr);
    }
    // K2, K3 (K3 also writes the fixed-point copy of v_k for the next product)
    lz_vector_passes<VV>(ctx, n, B.stop.p, k, B.w.p, V1, V2, s1, s2, B.beta.p + k, B.alpha.p + k, B.dots.p + k, Vk,
                         B.nrm2.p + k, B.nrm.p + k, B.scl.p + k, W.red_tri<VV>(2), W.red_d_flat(3), Xnext,
                         fxk == 1 ? form->F : 0, fxk == 1 ? B.ovf.p : nullptr, fxk != 0);
  }
}

template <typename VV>
static LanczosBuffers<VV>& buffers_for(Workspace& W, int64_t n, int kdim);

template <>
LanczosBuffers<double>& buffers_for<double>(Workspace& W, int64_t n, int kdim) {
  W.lz_d.ensure(n, kdim);
  return W.lz_d;
}
template <>
LanczosBuffers<cplx>& buffers_for<cplx>(Workspace& W, int64_t n, int kdim) {
  W.lz_c.ensure(n, kdim);
  return W.lz_c;
}

template <typename MV, typename VV>
static void lanczos_finish(qd_ham* H, cplx* psi, const double* psi_nrm2, const qd_lanczos_opts& o,
                           LanczosBuffers<VV>& B, Workspace& W, const MV* vals, bool mf, int fxk,
                           const FxForm* form, double* evals_out, qd_lanczos_result* res);

template <typename MV, typename VV>
static void lanczos_ground_impl(qd_ham* H, cplx* psi, const double* psi_nrm2, const qd_lanczos_opts& o,
                                double* evals_out, qd_lanczos_result* res) {
  Ctx* ctx = H->ctx;
  const int64_t n = H->dim;
  const int kdim = o.krylov_dim;
  Workspace& W = ham_workspace(H);
  LanczosBuffers<VV>& B = buffers_for<VV>(W, n, kdim);
  const MV* vals = nullptr;
  if constexpr (std::is_same<MV, double>::value) vals = H->vals_r.p;
  else vals = H->vals_c.p;
  const int vg = vec_grid(ctx, n);
  QD_CUDA(cudaMemsetAsync(B.stop.p, 0, sizeof(int), ctx->stream));
  const double one = 1.0;
  QD_CUDA(cudaMemcpyAsync(B.scl.p, &one, sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
  init_v0_kernel<VV><<<vg, kVecThreads, 0, ctx->stream>>>(n, psi, psi_nrm2, B.V.p);
  QD_CHECK_LAUNCH();
  QD_LAUNCHED(ctx);

  const bool timing = std::getenv("QD_TIMING") != nullptr;
  const auto host_t0 = std::chrono::steady_clock::now();
  if (timing) QD_CUDA(cudaEventRecord(ctx->events[12], ctx->stream));
  const bool mf = (o.spmv == QD_SPMV_MATRIX_FREE);
  // fxk 1: the fixed-point uniform-coupling form fused with the dots (fxsum.cuh): the stored-matrix
  // form on the CSR path, the form built from the terms alone on the matrix-free path
  int fxk = 0;
  const FxForm* form = nullptr;
  if constexpr (std::is_same<VV, double>::value) {
    if (!mf && H->fx_allowed && ham_build_fx(H)) form = H->fx.get();
    if (mf && H->fx_allowed && ham_build_mf_fx(H)) form = H->mfx.get();
  }
  fxk = form ? 1 : 0;
  const bool fx = fxk == 1;
  const int fxF = fx ? form->F : 0;
  const bool one_launch = fx && fx_one_launch_step() && !H->one_shot;
  // the column source of the fixed-point form is part of what a captured recurrence launches
  const int src = !fx ? 0 : ((form->blk_state > 0 && form->use_blk) ? 2 : ((form->slots_state > 0 && form->use_slots) ? 1 : 0));
  const int kind = (mf ? 1 : 0) + 2 * fxk + (one_launch ? 4 : 0) + ((one_launch && step_wait_out_polls()) ? 8 : 0) +
                   16 * src;
  if (B.kind != kind) {
    B.drop_graph();
    B.kind = kind;
  }
  if (fx) {
    B.ensure_fx(ctx->stream);
    QD_CUDA(cudaMemsetAsync(B.ovf.p, 0, 2 * sizeof(int), ctx->stream));
    if constexpr (std::is_same<VV, double>::value) launch_fx_shadow(ctx, n, B.V.p, B.X.p, fxF, B.ovf.p);
  }
  const int steps = (o.add_dim > 0 && o.add_dim < kdim) ? o.add_dim : kdim;  // add_dim of an incremental start
  if (steps == kdim && !H->one_shot)
    B.run_graph(ctx, [&]() { lanczos_run<MV, VV>(H, vals, B, 1, kdim, W, mf, fxk, form); });
  else
    lanczos_run<MV, VV>(H, vals, B, 1, steps, W, mf, fxk, form);
  B.done = steps;
  W.lz_vv = std::is_same<VV, double>::value ? 1 : 2;
  W.lz_mv = std::is_same<MV, double>::value ? 1 : 2;
  W.lz_mf = mf;
  W.lz_fxk = fxk;
  if (fx) {
    const int ov = fx_flags(ctx, B.ovf.p);
    if (ov) {  // a vector left the fixed-point range: redo the solve on the FP64 CSR product
      H->fx_allowed = false;
      lanczos_ground_impl<MV, VV>(H, psi, psi_nrm2, o, evals_out, res);
      H->fx_allowed = true;
      return;
    }
  }
  if (timing) QD_CUDA(cudaEventRecord(ctx->events[13], ctx->stream));
  lanczos_finish<MV, VV>(H, psi, psi_nrm2, o, B, W, vals, mf, fxk, form, evals_out, res);
  if (timing) {
    float g = 0.f;
    QD_CUDA(cudaEventElapsedTime(&g, ctx->events[12], ctx->events[13]));
    const double host_ms =
        std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - host_t0).count();
    std::fprintf(stderr, "[qd timing] lanczos n=%lld k=%d: recurrence %.3f ms (%.1f us/step), whole solve %.3f ms\n",
                 (long long)n, kdim, g, 1e3 * g / kdim, host_ms);
  }
}

// Eigen-decomposition of the tridiagonal matrix of the B.done steps run so
// far and the Ritz vector of its lowest level, written to psi.
template <typename MV, typename VV>
static void lanczos_finish(qd_ham* H, cplx* psi, const double* psi_nrm2, const qd_lanczos_opts& o,
                           LanczosBuffers<VV>& B, Workspace& W, const MV* vals, bool mf, int fxk,
                           const FxForm* form, double* evals_out, qd_lanczos_result* res) {
  Ctx* ctx = H->ctx;
  const int64_t n = H->dim;
  const int kdim = B.done;
  const bool fx = fxk == 1;
  const int fxF = fx ? form->F : 0;
  const int vg = vec_grid(ctx, n);
  int matvecs = kdim;

  std::vector<VV> alpha(kdim + 1);
  std::vector<double> nrm(kdim + 1);
  int stop = 0;
  QD_CUDA(cudaMemcpyAsync(alpha.data(), B.alpha.p, (kdim + 1) * sizeof(VV), cudaMemcpyDeviceToHost, ctx->stream));
  QD_CUDA(cudaMemcpyAsync(nrm.data(), B.nrm.p, (kdim + 1) * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  QD_CUDA(cudaMemcpyAsync(&stop, B.stop.p, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  QD_CUDA(cudaStreamSynchronize(ctx->stream));
  if (stop) matvecs = stop;
  const int act = stop ? stop - 1 : kdim;  // expandBasis<1> return value
  QD_REQUIRE(act >= 1, QD_ERR_BREAKDOWN, "Lanczos broke down at the first step (start vector in an "
             "invariant subspace of dimension 1)");
  std::vector<double> d(act), e(act), z(act), ev(act);
  for (int i = 0; i < act; ++i) {
    d[i] = real_part(alpha[i + 1]);
    e[i] = (i + 1 < act) ? nrm[i + 1] : 0.0;
  }
  QD_REQUIRE(tridiag_lowest<double>(act, d.data(), e.data(), ev.data(), z.data()) == 0, QD_ERR_INVALID,
             "tridiagonal eigensolver did not converge");
  d = ev;
  if (o.ritz == QD_RITZ_SECOND_PASS) {
    // getState<1> regenerates v_1..v_act with the same kernels (same bits);
    // run it for the reference's work pattern (act more products).
    init_v0_kernel<VV><<<vg, kVecThreads, 0, ctx->stream>>>(n, psi, psi_nrm2, B.V.p);
    QD_CHECK_LAUNCH();
    QD_LAUNCHED(ctx);
    QD_CUDA(cudaMemsetAsync(B.stop.p, 0, sizeof(int), ctx->stream));
    if (fx) {
      QD_CUDA(cudaMemsetAsync(B.ovf.p, 0, 2 * sizeof(int), ctx->stream));
      if constexpr (std::is_same<VV, double>::value) launch_fx_shadow(ctx, n, B.V.p, B.X.p, fxF, B.ovf.p);
    }
    lanczos_run<MV, VV>(H, vals, B, 1, act, W, mf, fxk, form);
    if (fx) fx_flags(ctx, B.ovf.p);
    matvecs += act;
  }
  // psi = sum_k y_k v_k = sum_k (y_k s_k) V[k]
  std::vector<double> scl(kdim + 1), yk(act);
  QD_CUDA(cudaMemcpyAsync(scl.data(), B.scl.p, (kdim + 1) * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  QD_CUDA(cudaStreamSynchronize(ctx->stream));
  for (int i = 0; i < act; ++i) yk[i] = z[i] * scl[i];
  QD_CUDA(cudaMemcpyAsync(B.y.p, yk.data(), act * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
  ritz_kernel<VV><<<vg, kVecThreads, 0, ctx->stream>>>(n, B.V.p, B.ld, B.y.p, act, psi);
  QD_CHECK_LAUNCH();
  QD_LAUNCHED(ctx);
  QD_CUDA(cudaStreamSynchronize(ctx->stream));
  if (evals_out) std::memcpy(evals_out, d.data(), act * sizeof(double));
  res->act_dim = act;
  res->breakdown = stop ? 1 : 0;
  res->matvecs = matvecs;
  res->ritz_value = d[0];
  res->err = std::fabs(d[0]);
}

// updateKrylovRepr with add_dim (sparse_algorithm.hpp:521-546): the recurrence
// of the last solve on this operator continues for add_dim more steps (up to
// its krylov_dim) from the stored basis, and the Ritz vector of the grown
// space is written to psi.
template <typename MV, typename VV>
static void lanczos_extend_impl(qd_ham* H, cplx* psi, const qd_lanczos_opts& o, double* evals_out,
                                qd_lanczos_result* res) {
  Ctx* ctx = H->ctx;
  Workspace& W = ham_workspace(H);
  LanczosBuffers<VV>& B = buffers_for<VV>(W, H->dim, o.krylov_dim);
  const MV* vals = nullptr;
  if constexpr (std::is_same<MV, double>::value) vals = H->vals_r.p;
  else vals = H->vals_c.p;
  int stop = 0;
  QD_CUDA(cudaMemcpyAsync(&stop, B.stop.p, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  QD_CUDA(cudaStreamSynchronize(ctx->stream));
  const int add = (o.add_dim > 0) ? std::min(o.add_dim, B.kdim - B.done) : B.kdim - B.done;
  const FxForm* form = W.lz_fxk == 1 ? (W.lz_mf ? H->mfx.get() : H->fx.get()) : nullptr;
  if (!stop && add > 0) {
    lanczos_run<MV, VV>(H, vals, B, B.done + 1, B.done + add, W, W.lz_mf, W.lz_fxk, form);
    B.done += add;
  }
  if (W.lz_fxk == 1) {
    const int ov = fx_flags(ctx, B.ovf.p);
    QD_REQUIRE(!ov, QD_ERR_OVERFLOW, "a Lanczos vector left the fixed-point range; restart the solve");
  }
  qd_lanczos_opts o2 = o;
  o2.ritz = QD_RITZ_STORED_BASIS;
  lanczos_finish<MV, VV>(H, psi, nullptr, o2, B, W, vals, W.lz_mf, W.lz_fxk, form, evals_out, res);
}

void lanczos_extend(qd_ham* H, cplx* psi, const qd_lanczos_opts& o, double* evals_out, qd_lanczos_result* res) {
  Workspace& W = ham_workspace(H);
  QD_REQUIRE(W.lz_vv != 0, QD_ERR_INVALID, "no Lanczos solve on this operator to continue");
  const bool dbl = (W.lz_vv == 1);
  LanczosBuffers<double>& Bd = W.lz_d;
  LanczosBuffers<cplx>& Bc = W.lz_c;
  const int kd = dbl ? Bd.kdim : Bc.kdim;
  QD_REQUIRE(o.krylov_dim == kd, QD_ERR_INVALID, "krylov_dim %d differs from the running solve's %d", o.krylov_dim,
             kd);
  QD_REQUIRE((o.spmv == QD_SPMV_MATRIX_FREE) == (W.lz_mf != 0), QD_ERR_INVALID,
             "the product kind differs from the running solve's");
  if (dbl)
    lanczos_extend_impl<double, double>(H, psi, o, evals_out, res);
  else if (W.lz_mv == 1)
    lanczos_extend_impl<double, cplx>(H, psi, o, evals_out, res);
  else
    lanczos_extend_impl<cplx, cplx>(H, psi, o, evals_out, res);
}

void lanczos_ground(qd_ham* H, cplx* psi, const qd_lanczos_opts& o, double* evals_out, qd_lanczos_result* res) {
  Ctx* ctx = H->ctx;
  const int64_t n = H->dim;
  QD_REQUIRE(o.krylov_dim >= 1 && o.krylov_dim <= 4096, QD_ERR_INVALID, "krylov_dim must be in 1..4096");
  QD_REQUIRE(n >= 1, QD_ERR_INVALID, "empty sector");
  Workspace& W = ham_workspace(H);
  // ||psi||^2 and whether the start vector is real (buffers kept in the workspace)
  if (!W.start_nrm2.p) W.start_nrm2.alloc(1);
  if (!W.start_has_im.p) W.start_has_im.alloc(1);
  DBuf<double>& nrm2 = W.start_nrm2;
  DBuf<int>& has_im = W.start_has_im;
  QD_CUDA(cudaMemsetAsync(has_im.p, 0, sizeof(int), ctx->stream));
  colnorm_kernel<<<vec_grid(ctx, n), kVecThreads, 0, ctx->stream>>>(n, psi, nrm2.p, W.red_d(0), has_im.p);
  QD_CHECK_LAUNCH();
  QD_LAUNCHED(ctx);
  int him = 0;
  double hn = 0.0;
  QD_CUDA(cudaMemcpyAsync(&him, has_im.p, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  QD_CUDA(cudaMemcpyAsync(&hn, nrm2.p, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  QD_CUDA(cudaStreamSynchronize(ctx->stream));
  QD_REQUIRE(hn > 0.0 && std::isfinite(hn), QD_ERR_INVALID, "start vector has zero or non-finite norm");
  if (o.spmv == QD_SPMV_MATRIX_FREE) ham_build_matrix_free(H);
  const bool real_h = (o.spmv == QD_SPMV_MATRIX_FREE) ? H->mf_real : (H->flags & QD_HAM_REAL) != 0;
  if (real_h && !him)
    lanczos_ground_impl<double, double>(H, psi, nrm2.p, o, evals_out, res);
  else if (real_h)
    lanczos_ground_impl<double, cplx>(H, psi, nrm2.p, o, evals_out, res);
  else
    lanczos_ground_impl<cplx, cplx>(H, psi, nrm2.p, o, evals_out, res);
}

// ---------------------------------------------------------------- Hermitian::LanczosSolver
// Hermitian::LanczosSolver::getGroundState (sparse_algorithm.hpp:287-301):
// getKrylovReprAd (:72-122) keeps two vectors v, w and alternates which one
// is rebuilt; step i takes x (the newest vector) and p (the one before):
//   a_i = <x, H x>,  p = H x - a_i x - sqrt(nn_{i-1}) p,  nn_i = ||p||^2,
//   p /= sqrt(nn_i),  and stops once nn_i <= 1e-10 (qudrip.hpp:18).
// The reference forms H x twice per step (once inside <x, H x>, once for the
// update); here one product serves both, with the inner product fused into
// it.  The lowest eigenvector z of tridiag(Re a, sqrt nn) is then expanded
// by getKrylovGS (:206-238): a second pass regenerates the same vectors with
// the same kernels (same bits) and accumulates psi = sum_i z_i x_i, so only
// three vectors of the space are ever held.
__device__ __forceinline__ double as_vv(double b, double) { return b; }
__device__ __forceinline__ cplx as_vv(double b, cplx) { return mkc(b, 0.0); }

__device__ __forceinline__ bool hstopped(const int* stop, int step) {
  const int st = *stop;
  return st != 0 && step >= st;
}

template <typename VV>
__global__ void __launch_bounds__(kVecThreads) herm_update_kernel(int64_t n, int* stop, int step, const VV* h,
                                                                  const VV* x, VV* p, const VV* a,
                                                                  const double* nn_prev, double* nn_out,
                                                                  GridRed<double> red) {
  if (hstopped(stop, step)) return;
  const VV ai = *a;
  const double b = nn_prev ? sqrt(*nn_prev) : 0.0;
  double acc = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    VV o = vsubmul(h[i], ai, x[i]);
    if (nn_prev) o = vsubmul(o, as_vv(b, VV{}), p[i]);
    p[i] = o;
    acc += vnorm2(o);
  }
  if (grid_sum(acc, red, nn_out) && threadIdx.x == 0) {
    if (!(*nn_out > 1e-10)) *stop = step + 1;
  }
}

template <typename VV>
__global__ void __launch_bounds__(kVecThreads) herm_scale_kernel(int64_t n, const int* stop, int step, VV* p,
                                                                 const double* nn) {
  if (hstopped(stop, step)) return;
  const double inv = 1.0 / sqrt(*nn);
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    p[i] = vscale(inv, p[i]);
}

template <typename VV>
__global__ void __launch_bounds__(kVecThreads) herm_accum_kernel(int64_t n, double z, const VV* x, cplx* psi,
                                                                 int first) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const cplx xi = to_c(x[i]);
    psi[i] = first ? mkc(z * xi.re, z * xi.im) : mkc(fma(z, xi.re, psi[i].re), fma(z, xi.im, psi[i].im));
  }
}

template <typename MV, typename VV>
static void herm_lanczos_impl(qd_ham* H, cplx* psi, const double* psi_nrm2, int kdim, double* evals_out,
                              qd_lanczos_result* res) {
  Ctx* ctx = H->ctx;
  const int64_t n = H->dim;
  Workspace& W = ham_workspace(H);
  const MV* vals = nullptr;
  if constexpr (std::is_same<MV, double>::value) vals = H->vals_r.p;
  else vals = H->vals_c.p;
  const int vg = vec_grid(ctx, n);
  DBuf<VV> v(n), w(n), h(n), a(kdim + 2);
  DBuf<double> nn(kdim + 2);
  DBuf<int> stop(1);
  DBuf<cplx> start(n);
  QD_CUDA(cudaMemcpyAsync(start.p, psi, n * sizeof(cplx), cudaMemcpyDeviceToDevice, ctx->stream));
  int64_t matvecs = 0;
  // one pass: steps 0..kdim-1 (accumulating psi += z_i x_i when z is given)
  auto pass = [&](const std::vector<double>* z, int K) {
    QD_CUDA(cudaMemsetAsync(stop.p, 0, sizeof(int), ctx->stream));
    init_v0_kernel<VV><<<vg, kVecThreads, 0, ctx->stream>>>(n, start.p, psi_nrm2, v.p);
    QD_CHECK_LAUNCH();
    QD_LAUNCHED(ctx);
    const int steps = z ? K : kdim + 1;  // a_0 and kdim more (the reference's idx runs 1..kdim)
    for (int i = 0; i < steps; ++i) {
      VV* x = (i % 2 == 0) ? v.p : w.p;
      VV* pp = (i % 2 == 0) ? w.p : v.p;
      if (z) {
        herm_accum_kernel<VV><<<vg, kVecThreads, 0, ctx->stream>>>(n, (*z)[i], x, psi, i == 0);
        QD_CHECK_LAUNCH();
        QD_LAUNCHED(ctx);
        if (i == K - 1) break;
      }
      launch_spmv<MV, VV>(ctx, H, vals, x, h.p, 1.0, x, W.red_c_or_d<VV>(1), a.p + i, stop.p, i + 1, -1);
      ++matvecs;
      herm_update_kernel<VV><<<vg, kVecThreads, 0, ctx->stream>>>(n, stop.p, i, h.p, x, pp, a.p + i,
                                                                  i ? nn.p + i - 1 : nullptr, nn.p + i, W.red_d(3));
      QD_CHECK_LAUNCH();
      QD_LAUNCHED(ctx);
      herm_scale_kernel<VV><<<vg, kVecThreads, 0, ctx->stream>>>(n, stop.p, i, pp, nn.p + i);
      QD_CHECK_LAUNCH();
      QD_LAUNCHED(ctx);
    }
  };
  pass(nullptr, 0);
  std::vector<VV> ha(kdim + 2);
  std::vector<double> hnn(kdim + 2);
  int st = 0;
  QD_CUDA(cudaMemcpyAsync(ha.data(), a.p, (kdim + 2) * sizeof(VV), cudaMemcpyDeviceToHost, ctx->stream));
  QD_CUDA(cudaMemcpyAsync(hnn.data(), nn.p, (kdim + 2) * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  QD_CUDA(cudaMemcpyAsync(&st, stop.p, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  QD_CUDA(cudaStreamSynchronize(ctx->stream));
  const int K = st ? st : kdim + 1;
  std::vector<double> d(K), e(K), ev(K), z(K);
  for (int i = 0; i < K; ++i) {
    d[i] = real_part(ha[i]);
    e[i] = (i + 1 < K) ? std::sqrt(hnn[i]) : 0.0;
  }
  QD_REQUIRE(tridiag_lowest<double>(K, d.data(), e.data(), ev.data(), z.data()) == 0, QD_ERR_INVALID,
             "tridiagonal eigensolver did not converge");
  pass(&z, K);
  QD_CUDA(cudaStreamSynchronize(ctx->stream));
  if (evals_out) std::memcpy(evals_out, ev.data(), K * sizeof(double));
  res->act_dim = K;
  res->breakdown = st ? 1 : 0;
  (void)matvecs;
  res->matvecs = 2 * K - 1;  // K products in the first pass, K - 1 in the second
  res->ritz_value = ev[0];
  res->err = std::sqrt(hnn[K - 1]);
}

void hermitian_lanczos_ground(qd_ham* H, cplx* psi, int kdim, double* evals_out, qd_lanczos_result* res) {
  Ctx* ctx = H->ctx;
  const int64_t n = H->dim;
  QD_REQUIRE(kdim >= 1 && kdim <= 4096, QD_ERR_INVALID, "krylov_dim must be in 1..4096");
  QD_REQUIRE(H->flags & QD_HAM_HERMITIAN, QD_ERR_NOT_HERMITIAN, "Hermitian::LanczosSolver needs a Hermitian operator");
  Workspace& W = ham_workspace(H);
  DBuf<double> nrm2(1);
  DBuf<int> has_im(1);
  QD_CUDA(cudaMemsetAsync(has_im.p, 0, sizeof(int), ctx->stream));
  colnorm_kernel<<<vec_grid(ctx, n), kVecThreads, 0, ctx->stream>>>(n, psi, nrm2.p, W.red_d(0), has_im.p);
  QD_CHECK_LAUNCH();
  QD_LAUNCHED(ctx);
  int him = 0;
  double hn = 0.0;
  QD_CUDA(cudaMemcpyAsync(&him, has_im.p, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  QD_CUDA(cudaMemcpyAsync(&hn, nrm2.p, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  QD_CUDA(cudaStreamSynchronize(ctx->stream));
  QD_REQUIRE(hn > 0.0 && std::isfinite(hn), QD_ERR_INVALID, "start vector has zero or non-finite norm");
  const bool real_h = (H->flags & QD_HAM_REAL) != 0;
  if (real_h && !him)
    herm_lanczos_impl<double, double>(H, psi, nrm2.p, kdim, evals_out, res);
  else if (real_h)
    herm_lanczos_impl<double, cplx>(H, psi, nrm2.p, kdim, evals_out, res);
  else
    herm_lanczos_impl<cplx, cplx>(H, psi, nrm2.p, kdim, evals_out, res);
}

// ---------------------------------------------------------------- Hermitian Krylov exponential
// psi_out = V exp(-i h T) e_0 with the Lanczos basis V of psi_in and its
// tridiagonal projection T: for Hermitian H the Arnoldi projection of
// ArnoldiSolver<T,0>::evolve (sparse_algorithm.hpp:548-562) is tridiagonal,
// so the three-term recurrence reaches the same Krylov space with 2 vector
// passes per product instead of a Gram-Schmidt sweep over the whole basis.
// m - 1 products as the reference's expandBasis<0>; a breakdown at step s
// keeps s basis vectors (the expandBasis<0> count, sparse_algorithm.hpp:
// 387-390).  exp(-i h T) e_0 = Q exp(-i h Lambda) Q^T e_0 from the QL
// eigen-decomposition of T.  The output has the input norm dropped.
// exp(-i h T) e_0 for T = tridiag(Re alpha_1.., n_1..) of dimension act on
// one warp (lane j holds component j): Taylor series with scaling (N. J.
// Higham and A. H. Al-Mohy, SIAM J. Sci. Comput. 33 (2011) 488-511), each
// term a tridiagonal product through shuffles, cut once a term falls below
// 1e-17 of the sum.  Writes y_j = c_j s_j (the stored basis is unnormalised)
// and act; adds act to *matvecs.
__global__ void __launch_bounds__(32) texp_kernel(int kdim, double h, const cplx* alpha, const double* nrm,
                                                  const double* scl, const int* stop, cplx* y, int* act_out,
                                                  long long* matvecs) {
  const int lane = threadIdx.x;
  const int st = *stop;
  const int act = st ? st : kdim;
  const bool on = lane < act;
  const double d = on ? alpha[lane + 1].re : 0.0;
  const double e = (lane + 1 < act) ? nrm[lane + 1] : 0.0;  // T(lane, lane+1)
  double em = __shfl_up_sync(0xffffffffu, e, 1);           // T(lane, lane-1)
  if (lane == 0) em = 0.0;
  double rowsum = fabs(d) + e + em;
  for (int o = 16; o > 0; o >>= 1) rowsum = fmax(rowsum, __shfl_xor_sync(0xffffffffu, rowsum, o));
  const int steps = max(1, (int)ceil(rowsum * fabs(h) / 0.5));
  const double hs = h / steps;
  double yr = (lane == 0) ? 1.0 : 0.0, yi = 0.0;
  for (int sstep = 0; sstep < steps; ++sstep) {
    double tr = yr, ti = yi;
    for (int p = 1; p <= 60; ++p) {
      const double tr_dn = __shfl_down_sync(0xffffffffu, tr, 1), ti_dn = __shfl_down_sync(0xffffffffu, ti, 1);
      const double tr_up = __shfl_up_sync(0xffffffffu, tr, 1), ti_up = __shfl_up_sync(0xffffffffu, ti, 1);
      double kr = d * tr + e * tr_dn + (lane ? em * tr_up : 0.0);
      double ki = d * ti + e * ti_dn + (lane ? em * ti_up : 0.0);
      if (!on) kr = ki = 0.0;
      const double f = hs / p;  // t <- (-i f) K t
      tr = f * ki;
      ti = -f * kr;
      yr += tr;
      yi += ti;
      double tn = tr * tr + ti * ti, yn = yr * yr + yi * yi;
      for (int o = 16; o > 0; o >>= 1) {
        tn += __shfl_xor_sync(0xffffffffu, tn, o);
        yn += __shfl_xor_sync(0xffffffffu, yn, o);
      }
      if (tn <= 1e-34 * yn) break;
    }
  }
  if (on) y[lane] = mkc(yr * scl[lane], yi * scl[lane]);
  if (lane == 0) {
    *act_out = act;
    if (matvecs) *matvecs += act;
  }
}

// psi = sum_{k < *act} y_k V[k]
__global__ void __launch_bounds__(kVecThreads) combine_dev_kernel(int64_t n, const cplx* V, int64_t ld, const cplx* y,
                                                                  const int* act_dev, cplx* psi) {
  const int act = *act_dev;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    cplx acc = vfma(y[0], V[i], mkc(0.0, 0.0));
    for (int k = 1; k < act; ++k) acc = vfma(y[k], V[(int64_t)k * ld + i], acc);
    psi[i] = acc;
  }
}

// One Krylov step psi <- V exp(-i h T) e_0 on the device, as one CUDA graph
// (norm, v_0, the m - 1 Lanczos steps, the small exponential, the
// combination): no host round trip, so nsteps steps are nsteps graph launches.
struct EvolveGraph {
  cudaGraphExec_t exec = nullptr;
  const cplx* psi = nullptr;
  double h = 0.0;
  int m = 0, mv_kind = 0;
  int64_t kernels = 0;
  DBuf<double> nrm2;
  DBuf<int> has_im, act;
  DBuf<cplx> y;
  DBuf<long long> matvecs;
  ~EvolveGraph() {
    if (exec) cudaGraphExecDestroy(exec);
  }
};

void EvolveGraphDeleter::operator()(EvolveGraph* g) const { delete g; }

template <typename MV>
static void lanczos_evolve_steps(qd_ham* H, cplx* psi, double h, int m, int nsteps, int* act_out,
                                 int64_t* matvecs_out) {
  Ctx* ctx = H->ctx;
  const int64_t n = H->dim;
  const int kdim = m - 1;
  Workspace& W = ham_workspace(H);
  LanczosBuffers<cplx>& B = buffers_for<cplx>(W, n, kdim);
  const MV* vals = nullptr;
  if constexpr (std::is_same<MV, double>::value) vals = H->vals_r.p;
  else vals = H->vals_c.p;
  const int mv_kind = std::is_same<MV, double>::value ? 1 : 2;
  W.lz_vv = 0;  // the Lanczos buffers are reused here: no ground-state run left to continue
  if (!W.evolve) W.evolve.reset(new EvolveGraph());
  EvolveGraph& G = *W.evolve;
  if (!G.nrm2.p) {
    G.nrm2.alloc(1);
    G.has_im.alloc(1);
    G.act.alloc(1);
    G.y.alloc(64);
    G.matvecs.alloc(1);
  }
  const double one = 1.0;
  QD_CUDA(cudaMemcpyAsync(B.scl.p, &one, sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
  QD_CUDA(cudaMemsetAsync(G.matvecs.p, 0, sizeof(long long), ctx->stream));
  if (B.kind != 0) {
    B.drop_graph();
    B.kind = 0;
  }
  const int vg = vec_grid(ctx, n);
  // one Krylov step: psi <- exp(-ih H) psi through the short recurrence
  auto step = [&]() {
    QD_CUDA(cudaMemsetAsync(B.stop.p, 0, sizeof(int), ctx->stream));
    colnorm_kernel<<<vg, kVecThreads, 0, ctx->stream>>>(n, psi, G.nrm2.p, W.red_d(0), G.has_im.p);
    QD_CHECK_LAUNCH();
    QD_LAUNCHED(ctx);
    init_v0_kernel<cplx><<<vg, kVecThreads, 0, ctx->stream>>>(n, psi, G.nrm2.p, B.V.p);
    QD_CHECK_LAUNCH();
    QD_LAUNCHED(ctx);
    lanczos_run<MV, cplx>(H, vals, B, 1, kdim, W, false);
    texp_kernel<<<1, 32, 0, ctx->stream>>>(kdim, h, B.alpha.p, B.nrm.p, B.scl.p, B.stop.p, G.y.p, G.act.p,
                                           G.matvecs.p);
    QD_CHECK_LAUNCH();
    QD_LAUNCHED(ctx);
    combine_dev_kernel<<<vg, kVecThreads, 0, ctx->stream>>>(n, B.V.p, B.ld, G.y.p, G.act.p, psi);
    QD_CHECK_LAUNCH();
    QD_LAUNCHED(ctx);
  };
  if (H->one_shot) {  // solved once: capturing a graph would cost more than it saves
    for (int s = 0; s < nsteps; ++s) step();
  } else if (!G.exec || G.psi != psi || G.h != h || G.m != m || G.mv_kind != mv_kind) {
    if (G.exec) cudaGraphExecDestroy(G.exec);
    G.exec = nullptr;
    cudaGraph_t g = nullptr;
    const int64_t before = ctx->launches;
    QD_CUDA(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
    try {
      step();
    } catch (...) {
      cudaStreamEndCapture(ctx->stream, &g);
      if (g) cudaGraphDestroy(g);
      ctx->launches = before;
      throw;
    }
    QD_CUDA(cudaStreamEndCapture(ctx->stream, &g));
    G.kernels = ctx->launches - before;
    ctx->launches = before;
    const cudaError_t e = cudaGraphInstantiate(&G.exec, g, 0);
    cudaGraphDestroy(g);
    QD_CUDA(e);
    G.psi = psi;
    G.h = h;
    G.m = m;
    G.mv_kind = mv_kind;
  }
  if (!H->one_shot)
    for (int s = 0; s < nsteps; ++s) {
      QD_CUDA(cudaGraphLaunch(G.exec, ctx->stream));
      ctx->launches += G.kernels;
    }
  int act = 0;
  long long mv = 0;
  QD_CUDA(cudaMemcpyAsync(&act, G.act.p, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  QD_CUDA(cudaMemcpyAsync(&mv, G.matvecs.p, sizeof(long long), cudaMemcpyDeviceToHost, ctx->stream));
  QD_CUDA(cudaStreamSynchronize(ctx->stream));
  if (act_out) *act_out = act;
  if (matvecs_out) *matvecs_out = mv;
}

void lanczos_evolve(qd_ham* H, const cplx* psi_in, cplx* psi_out, double h, int m, int nsteps, int* act_out,
                    int64_t* matvecs_out) {
  Ctx* ctx = H->ctx;
  const int64_t n = H->dim;
  QD_REQUIRE(m >= 2 && m <= 33, QD_ERR_INVALID, "Krylov dimension must be in 2..33");
  QD_REQUIRE(nsteps >= 1, QD_ERR_INVALID, "nsteps must be positive");
  QD_REQUIRE(H->flags & QD_HAM_HERMITIAN, QD_ERR_NOT_HERMITIAN,
             "the short-recurrence Krylov exponential needs a Hermitian operator");
  Workspace& W = ham_workspace(H);
  {
    DBuf<double> nrm2(1);
    DBuf<int> has_im(1);
    QD_CUDA(cudaMemsetAsync(has_im.p, 0, sizeof(int), ctx->stream));
    colnorm_kernel<<<vec_grid(ctx, n), kVecThreads, 0, ctx->stream>>>(n, psi_in, nrm2.p, W.red_d(0), has_im.p);
    QD_CHECK_LAUNCH();
    QD_LAUNCHED(ctx);
    double hn = 0.0;
    QD_CUDA(cudaMemcpyAsync(&hn, nrm2.p, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    QD_CUDA(cudaStreamSynchronize(ctx->stream));
    QD_REQUIRE(hn > 0.0 && std::isfinite(hn), QD_ERR_INVALID, "input state has zero or non-finite norm");
  }
  if (psi_out != psi_in)
    QD_CUDA(cudaMemcpyAsync(psi_out, psi_in, n * sizeof(cplx), cudaMemcpyDeviceToDevice, ctx->stream));
  if (H->flags & QD_HAM_REAL)
    lanczos_evolve_steps<double>(H, psi_out, h, m, nsteps, act_out, matvecs_out);
  else
    lanczos_evolve_steps<cplx>(H, psi_out, h, m, nsteps, act_out, matvecs_out);
}

}  // namespace qd
