// kbatch.cu -- many Krylov real-time steps y_b = exp(-i H h) x_b at once.
//
// The reference's ArnoldiSolver<T,0>::evolve (sparse_algorithm.hpp:548-562)
// for a batch of vectors sharing one Hamiltonian, in one persistent launch:
// a CTA takes the next vector from an atomic counter and runs the whole
// Arnoldi process for it in FP64 (m-1 products, Gram-Schmidt twice against
// its own basis, breakdown at norm < 1e-10, the expandBasis<0> dimension
// rule), keeps the Hessenberg matrix in shared memory, and evaluates
// exp(-i h K) e_0 on the device by a truncated Taylor series with scaling
// (N. J. Higham and A. H. Al-Mohy, SIAM J. Sci. Comput. 33 (2011) 488-511),
// then writes y = V exp(-i h K) e_0 normalised as the reference leaves it
// (the input norm dropped).  Used to tabulate the no-jump propagator of the
// trajectory loop and for time-evolution requests of the request loop.
#include <algorithm>
#include <cstring>

#include "kbatch.cuh"
#include "krylov.cuh"

namespace qd {

constexpr int kKbThreads = 256;
constexpr int kKbMaxM = 32;

struct KbScratch {
  cplx K[kKbMaxM][kKbMaxM];  // K[j][i]: projection of H v_i on v_j
  cplx h[kKbMaxM];
  cplx y[kKbMaxM], t[kKbMaxM], u[kKbMaxM];
  double red[kKbThreads / 32];
  double redi[kKbThreads / 32];
  double bcast, bcasti;
  int act, idx;
};

__device__ cplx kb_block_sum(cplx v, KbScratch& S) {
  double re = warp_sum0(v.re), im = warp_sum0(v.im);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) {
    S.red[warp] = re;
    S.redi[warp] = im;
  }
  __syncthreads();
  if (warp == 0) {
    double a = (lane < kKbThreads / 32) ? S.red[lane] : 0.0;
    double b = (lane < kKbThreads / 32) ? S.redi[lane] : 0.0;
    a = warp_sum0(a);
    b = warp_sum0(b);
    if (lane == 0) {
      S.bcast = a;
      S.bcasti = b;
    }
  }
  __syncthreads();
  return mkc(S.bcast, S.bcasti);
}

template <typename MV>
__device__ void kb_spmv(const KbArgs& A, const MV* vals, const cplx* __restrict__ x, cplx* __restrict__ y) {
  for (int64_t r = threadIdx.x; r < A.dim; r += blockDim.x) {
    cplx acc = mkc(0.0, 0.0);
    for (int64_t k = A.rowptr[r]; k < A.rowptr[r + 1]; ++k) acc = vfma(vals[k], x[A.colidx[k]], acc);
    y[r] = acc;
  }
}

template <typename MV>
__global__ void __launch_bounds__(kKbThreads) kbatch_kernel(KbArgs A, const MV* vals) {
  __shared__ KbScratch S;
  const int m = A.m;
  const int64_t n = A.dim;
  cplx* V = A.work + (size_t)blockIdx.x * (size_t)(m + 1) * A.ld;
  for (;;) {
    if (threadIdx.x == 0) S.idx = (int)atomicAdd(A.counter, 1u);
    __syncthreads();
    const int b = S.idx;
    __syncthreads();
    if (b >= A.nvec) return;
    // input column b: either X[:, b] or the unit vector e_b (propagator tabulation)
    double n2 = 0.0;
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) {
      const cplx xi = A.X ? A.X[(size_t)b * A.ldx + i] : mkc(i == b ? 1.0 : 0.0, 0.0);
      V[i] = xi;
      n2 += vnorm2(xi);
    }
    n2 = kb_block_sum(mkc(n2, 0.0), S).re;
    const double inv0 = 1.0 / sqrt(n2);
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) V[i] = vscale(inv0, V[i]);
    for (int q = threadIdx.x; q < kKbMaxM * kKbMaxM; q += blockDim.x) (&S.K[0][0])[q] = mkc(0.0, 0.0);
    __syncthreads();
    int act = m - 1;
    for (int idx = 1; idx <= m - 1; ++idx) {
      const cplx* vprev = V + (size_t)(idx - 1) * A.ld;
      cplx* w = V + (size_t)idx * A.ld;
      kb_spmv<MV>(A, vals, vprev, w);
      __syncthreads();
      for (int pass = 0; pass < 2; ++pass) {
        // projections on v_0 .. v_{idx-1}, one warp per basis vector
        const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
        for (int j = warp; j < idx; j += kKbThreads / 32) {
          const cplx* vj = V + (size_t)j * A.ld;
          cplx acc = mkc(0.0, 0.0);
          for (int64_t i = lane; i < n; i += 32) acc = vdotfma(vj[i], w[i], acc);
          acc = warp_sum0(acc);
          if (lane == 0) S.h[j] = acc;
        }
        __syncthreads();
        for (int64_t i = threadIdx.x; i < n; i += blockDim.x) {
          cplx wi = w[i];
          for (int j = 0; j < idx; ++j) wi = vsubmul(wi, S.h[j], V[(size_t)j * A.ld + i]);
          w[i] = wi;
        }
        if (threadIdx.x < idx) S.K[threadIdx.x][idx - 1] = vadd(S.K[threadIdx.x][idx - 1], S.h[threadIdx.x]);
        __syncthreads();
      }
      double nn = 0.0;
      for (int64_t i = threadIdx.x; i < n; i += blockDim.x) nn += vnorm2(w[i]);
      const double nr = sqrt(kb_block_sum(mkc(nn, 0.0), S).re);
      const double inv = 1.0 / nr;
      for (int64_t i = threadIdx.x; i < n; i += blockDim.x) w[i] = vscale(inv, w[i]);
      if (threadIdx.x == 0 && idx < kKbMaxM) S.K[idx][idx - 1] = mkc(nr, 0.0);
      __syncthreads();
      if (nr < 1e-10) {  // expandBasis<0>: the breaking step counts (sparse_algorithm.hpp:387-390)
        act = idx;
        break;
      }
    }
    // y = exp(-i h K[:act,:act]) e_0 by Taylor series with scaling (one warp)
    if (threadIdx.x < 32) {
      const int lane = threadIdx.x;
      double colmax = 0.0;
      for (int c = 0; c < act; ++c) {
        double s = 0.0;
        for (int r = 0; r < act; ++r) s += sqrt(vnorm2(S.K[r][c]));
        colmax = fmax(colmax, s);
      }
      const double nrm1 = colmax * fabs(A.h);
      const int steps = max(1, (int)ceil(nrm1 / 0.5));
      const double hs = A.h / steps;
      if (lane < act) S.y[lane] = mkc(lane == 0 ? 1.0 : 0.0, 0.0);
      __syncwarp();
      for (int st = 0; st < steps; ++st) {
        if (lane < act) {
          S.t[lane] = S.y[lane];
        }
        __syncwarp();
        for (int p = 1; p <= 40; ++p) {
          // u = (-i hs / p) K t
          cplx acc = mkc(0.0, 0.0);
          if (lane < act)
            for (int c = 0; c < act; ++c) acc = vfma(S.K[lane][c], S.t[c], acc);
          const double f = hs / p;
          const cplx u = mkc(f * acc.im, -f * acc.re);  // (-i f) * acc
          __syncwarp();
          double tn = (lane < act) ? vnorm2(u) : 0.0;
          double yn = (lane < act) ? vnorm2(S.y[lane]) : 0.0;
          if (lane < act) {
            S.t[lane] = u;
            S.y[lane] = vadd(S.y[lane], u);
          }
          tn = warp_sum(tn);
          yn = warp_sum(yn);
          __syncwarp();
          if (tn <= 1e-34 * yn) break;  // term below 1e-17 of the sum
        }
      }
    }
    __syncthreads();
    // y_out = sum_j y_j v_j
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) {
      cplx acc = mkc(0.0, 0.0);
      for (int j = 0; j < act; ++j) acc = vfma(S.y[j], V[(size_t)j * A.ld + i], acc);
      if (A.Y64) A.Y64[(size_t)b * A.ldy + i] = acc;
      if (A.Y32) A.Y32[(size_t)b * A.ldy + i] = make_float2((float)acc.re, (float)acc.im);
    }
    if (threadIdx.x == 0 && A.act_out) A.act_out[b] = act;
    __syncthreads();
  }
}

void krylov_batch(qd_ham* H, const cplx* X, int64_t ldx, int nvec, double h, int m, cplx* Y64, float2* Y32,
                  int64_t ldy, int* act_out) {
  Ctx* ctx = H->ctx;
  QD_REQUIRE(m >= 2 && m <= kKbMaxM, QD_ERR_UNSUPPORTED, "Krylov dimension m must be in 2..%d", kKbMaxM);
  QD_REQUIRE(nvec >= 1, QD_ERR_INVALID, "no vectors");
  KbArgs A;
  std::memset(&A, 0, sizeof(A));
  A.dim = H->dim;
  A.rowptr = H->rowptr.p;
  A.colidx = H->colidx.p;
  A.m = m;
  A.h = h;
  A.X = X;
  A.ldx = ldx;
  A.nvec = nvec;
  A.Y64 = Y64;
  A.Y32 = Y32;
  A.ldy = ldy;
  A.ld = (H->dim + 31) / 32 * 32;
  const int grid = std::min(nvec, 2 * ctx->num_sms);
  DBuf<cplx> work((size_t)grid * (m + 1) * A.ld);
  DBuf<unsigned> counter(1);
  DBuf<int> acts(nvec);
  QD_CUDA(cudaMemsetAsync(counter.p, 0, sizeof(unsigned), ctx->stream));
  A.work = work.p;
  A.counter = counter.p;
  A.act_out = acts.p;
  if (H->flags & QD_HAM_REAL)
    kbatch_kernel<double><<<grid, kKbThreads, 0, ctx->stream>>>(A, H->vals_r.p);
  else
    kbatch_kernel<cplx><<<grid, kKbThreads, 0, ctx->stream>>>(A, H->vals_c.p);
  QD_CHECK_LAUNCH();
  QD_LAUNCHED(ctx);
  if (act_out) QD_CUDA(cudaMemcpyAsync(act_out, acts.p, nvec * sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  QD_CUDA(cudaStreamSynchronize(ctx->stream));
}

}  // namespace qd
