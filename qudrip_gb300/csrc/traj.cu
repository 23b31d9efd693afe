// traj.cu -- quantum-jump trajectory ensembles (the jump loop of
// programs/hubbard_diss.cpp:439-482 with lindblad_weight :520-529,
// QJ_operator :514-517 and bsearch :565-577) for diagonal jump operators
// L_j = sqrt(gamma) n_{bit_j}.
//
// Per step and trajectory, as the reference does:
//   weights w_j = <psi| n_j^dagger n_j |psi>, wtot = sum_j w_j;
//   if u1 < gamma * wtot * dt: jump into channel bsearch(cumulative w / wtot, u2),
//       psi <- n_j psi / ||n_j psi||;
//   else psi <- exp(-i H_eff dt) psi / ||.||;
//   record the observables <psi| n_a n_b |psi>.
// GB300 form:
//   * the no-jump generator H_eff = H - (i/2) gamma sum_j n_j is the same for
//     every trajectory and every step (the reference's per-step shift
//     +(i/2) gamma wtot I only rescales the state, and the reference
//     renormalises right after), so exp(-i H_eff dt) is tabulated once,
//     column by column, by the batched Krylov kernel (m vectors, FP64
//     projection, kbatch.cu) and stored as complex64;
//   * each step advances all trajectories with one complex GEMM
//     (cuBLAS, FP32 accumulation emulated on the tensor cores) and one kernel
//     that takes the jump decisions (Philox4x32-10 keyed by seed, trajectory
//     and step, replayable on the CPU), applies jumps and computes weights,
//     norms and observables of the new states in one pass (FP32 sums);
//   * states are complex64 and kept up to a known scale: the norm is carried
//     to the next step instead of an extra normalisation pass.
#include <cublas_v2.h>

#include <algorithm>
#include <cstring>
#include <vector>

#include "kbatch.cuh"
#include "krylov.cuh"
#include "philox.cuh"
#include "traj.cuh"

namespace qd {

constexpr int kTrajThreads = 256;

struct TrajArgs {
  int64_t n;
  int64_t ld;            // leading dimension of the state block
  int ntraj;
  int nchan;
  int nobs;
  int step;
  double gamma, dt;
  uint64_t seed;
  const uint64_t* basis;
  float2* psi;           // current states (n x ntraj), overwritten with the next ones
  const float2* psi_new; // U psi
  float* w;              // per trajectory: nchan weights + norm^2 (stride kTrajMaxChan + 1)
  float* obs;            // (step) x nobs x ntraj, normalised observables
  int* jumps;            // per trajectory jump count
  const int* chan_bits;
  const uint64_t* obs_mask;  // observable k: state contributes when (s & mask_k) == mask_k
};

__global__ void __launch_bounds__(kTrajThreads) traj_step_kernel(TrajArgs A) {
  __shared__ float s_red[kTrajThreads / 32][kTrajMaxChan + 1 + kTrajMaxObs];
  __shared__ int s_jump;      // -1: evolve, else channel
  __shared__ float s_scale;
  const int b = blockIdx.x;
  if (b >= A.ntraj) return;
  float* wb = A.w + (size_t)b * (kTrajMaxChan + 1);
  if (A.step > 0 && threadIdx.x == 0) {
    // decision from the previous state's weights (unnormalised, norm^2 in wb[kTrajMaxChan])
    const double nrm2 = wb[kTrajMaxChan];
    double cum[kTrajMaxChan + 1];
    cum[0] = 0.0;
    for (int j = 0; j < A.nchan; ++j) cum[j + 1] = cum[j] + (double)wb[j] / nrm2;
    const double wtot = cum[A.nchan];
    double u1, u2;
    philox_uniform2(A.seed, (uint32_t)b, (uint32_t)A.step, u1, u2);
    int jump = -1;
    if (u1 < A.gamma * wtot * A.dt && wtot > 0.0) {
      // bsearch (hubbard_diss.cpp:565-577) on the cumulative weights normalised by wtot
      int is = 0, ie = A.nchan + 1;
      while (ie - is > 1) {
        const int mid = is + (ie - is) / 2;
        if (u2 < cum[mid] / wtot) ie = mid;
        else is = mid;
      }
      jump = min(is, A.nchan - 1);
    }
    s_jump = jump;
    // scale so the new state has unit norm: jump -> 1/||n_j psi||, evolve -> 1/||psi||
    s_scale = (jump >= 0) ? (float)(1.0 / sqrt((double)wb[jump])) : (float)(1.0 / sqrt(nrm2));
    if (jump >= 0) A.jumps[b] += 1;
  }
  if (A.step == 0 && threadIdx.x == 0) {
    s_jump = -2;  // initial state: moments only
    s_scale = 1.0f;
  }
  __syncthreads();
  const int jump = s_jump;
  const float sc = s_scale;
  const uint64_t jmask = (jump >= 0) ? (1ull << A.chan_bits[jump]) : 0ull;
  float acc[kTrajMaxChan + 1 + kTrajMaxObs];
#pragma unroll
  for (int q = 0; q < kTrajMaxChan + 1 + kTrajMaxObs; ++q) acc[q] = 0.f;
  float2* col = A.psi + (size_t)b * A.ld;
  const float2* ncol = A.psi_new + (size_t)b * A.ld;
  for (int64_t s = threadIdx.x; s < A.n; s += blockDim.x) {
    const uint64_t st = A.basis[s];
    float2 x;
    if (jump == -2) {
      x = col[s];
    } else if (jump >= 0) {
      x = (st & jmask) ? col[s] : make_float2(0.f, 0.f);
      x.x *= sc;
      x.y *= sc;
    } else {
      x = ncol[s];
      x.x *= sc;
      x.y *= sc;
    }
    if (jump != -2) col[s] = x;
    const float p = fmaf(x.x, x.x, x.y * x.y);
#pragma unroll
    for (int j = 0; j < kTrajMaxChan; ++j)
      if (j < A.nchan && ((st >> A.chan_bits[j]) & 1ull)) acc[j] += p;
    acc[kTrajMaxChan] += p;
#pragma unroll
    for (int k = 0; k < kTrajMaxObs; ++k)
      if (k < A.nobs && (st & A.obs_mask[k]) == A.obs_mask[k]) acc[kTrajMaxChan + 1 + k] += p;
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int q = 0; q < kTrajMaxChan + 1 + kTrajMaxObs; ++q) {
    float v = acc[q];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) s_red[warp][q] = v;
  }
  __syncthreads();
  if (threadIdx.x < kTrajMaxChan + 1 + kTrajMaxObs) {
    const int q = threadIdx.x;
    double t = 0.0;
    for (int w = 0; w < kTrajThreads / 32; ++w) t += s_red[w][q];
    s_red[0][q] = (float)t;
  }
  __syncthreads();
  if (threadIdx.x <= kTrajMaxChan) wb[threadIdx.x] = s_red[0][threadIdx.x];
  if (threadIdx.x < A.nobs) {
    const float nrm2 = s_red[0][kTrajMaxChan];
    A.obs[((size_t)A.step * A.nobs + threadIdx.x) * A.ntraj + b] = s_red[0][kTrajMaxChan + 1 + threadIdx.x] / nrm2;
  }
}

// mean and standard error over trajectories (fixed order, FP64)
__global__ void traj_reduce_kernel(const float* obs, int ntraj, int nrows, double* mean, double* stderr_) {
  const int row = blockIdx.x * blockDim.x + threadIdx.x;
  if (row >= nrows) return;
  double s = 0.0, s2 = 0.0;
  for (int b = 0; b < ntraj; ++b) {
    const double v = obs[(size_t)row * ntraj + b];
    s += v;
    s2 += v * v;
  }
  const double m = s / ntraj;
  mean[row] = m;
  stderr_[row] = (ntraj > 1) ? sqrt(fmax(s2 / ntraj - m * m, 0.0) / (ntraj - 1)) : 0.0;
}

__global__ void init_states_kernel(float2* psi, int64_t n, int64_t ld, int ntraj, const cplx* psi0, double inv) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int b = blockIdx.y;
  if (i >= n || b >= ntraj) return;
  const cplx v = psi0[i];
  psi[(size_t)b * ld + i] = make_float2((float)(v.re * inv), (float)(v.im * inv));
}

#define QD_CUBLAS(call)                                                      \
  do {                                                                       \
    cublasStatus_t s__ = (call);                                             \
    QD_REQUIRE(s__ == CUBLAS_STATUS_SUCCESS, QD_ERR_CUDA, "%s failed: %d", #call, (int)s__); \
  } while (0)

void traj_run(qd_ham* H, const qd_traj_desc& d, const double* psi0_host, double* obs_mean, double* obs_stderr,
              int64_t* jumps_total, double* timings) {
  Ctx* ctx = H->ctx;
  const int64_t n = H->dim;
  QD_REQUIRE(d.ntraj >= 1 && d.nsteps >= 0, QD_ERR_INVALID, "ntraj >= 1 and nsteps >= 0 required");
  QD_REQUIRE(d.nchan >= 1 && d.nchan <= kTrajMaxChan, QD_ERR_UNSUPPORTED, "1..%d jump channels", kTrajMaxChan);
  QD_REQUIRE(d.nobs >= 0 && d.nobs <= kTrajMaxObs, QD_ERR_UNSUPPORTED, "at most %d observables", kTrajMaxObs);
  QD_REQUIRE(d.dt > 0.0 && d.gamma >= 0.0, QD_ERR_INVALID, "dt > 0 and gamma >= 0 required");
  QD_REQUIRE(n <= (int64_t)INT32_MAX, QD_ERR_UNSUPPORTED, "dimension too large");
  for (int j = 0; j < d.nchan; ++j)
    QD_REQUIRE(d.chan_bits[j] >= 0 && d.chan_bits[j] < H->sec->nbits, QD_ERR_INVALID, "channel %d: bad bit", j);
  std::vector<uint64_t> masks(kTrajMaxObs, 0ull);
  for (int k = 0; k < d.nobs; ++k) {
    QD_REQUIRE(d.obs_a[k] >= 0 && d.obs_a[k] < H->sec->nbits && d.obs_b[k] >= 0 && d.obs_b[k] < H->sec->nbits,
               QD_ERR_INVALID, "observable %d: bad bit", k);
    masks[k] = (1ull << d.obs_a[k]) | (1ull << d.obs_b[k]);
  }
  cudaEvent_t e0, e1, e2;
  QD_CUDA(cudaEventCreate(&e0));
  QD_CUDA(cudaEventCreate(&e1));
  QD_CUDA(cudaEventCreate(&e2));
  QD_CUDA(cudaEventRecord(e0, ctx->stream));
  // propagator columns U e_b, complex64, n x n
  DBuf<float2> U((size_t)n * n);
  krylov_batch(H, nullptr, 0, (int)n, d.dt, d.m, nullptr, U.p, n, nullptr);
  QD_CUDA(cudaEventRecord(e1, ctx->stream));
  const int64_t ld = (n + 31) / 32 * 32;
  DBuf<float2> psi((size_t)ld * d.ntraj), psi_new((size_t)ld * d.ntraj);
  QD_CUDA(cudaMemsetAsync(psi.p, 0, psi.bytes(), ctx->stream));
  QD_CUDA(cudaMemsetAsync(psi_new.p, 0, psi_new.bytes(), ctx->stream));
  DBuf<cplx> p0(n);
  QD_CUDA(cudaMemcpyAsync(p0.p, psi0_host, n * sizeof(cplx), cudaMemcpyHostToDevice, ctx->stream));
  double n0 = 0.0;
  for (int64_t i = 0; i < n; ++i) n0 += psi0_host[2 * i] * psi0_host[2 * i] + psi0_host[2 * i + 1] * psi0_host[2 * i + 1];
  QD_REQUIRE(n0 > 0.0, QD_ERR_INVALID, "initial state is zero");
  init_states_kernel<<<dim3((unsigned)ceil_div(n, 256), d.ntraj), 256, 0, ctx->stream>>>(psi.p, n, ld, d.ntraj, p0.p,
                                                                                     1.0 / std::sqrt(n0));
  QD_CHECK_LAUNCH();
  QD_LAUNCHED(ctx);
  DBuf<float> w((size_t)d.ntraj * (kTrajMaxChan + 1));
  DBuf<float> obs((size_t)(d.nsteps + 1) * std::max(d.nobs, 1) * d.ntraj);
  DBuf<int> jumps(d.ntraj);
  DBuf<int> bits(kTrajMaxChan);
  DBuf<uint64_t> omask(kTrajMaxObs);
  QD_CUDA(cudaMemsetAsync(jumps.p, 0, jumps.bytes(), ctx->stream));
  QD_CUDA(cudaMemcpyAsync(bits.p, d.chan_bits, d.nchan * sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
  QD_CUDA(cudaMemcpyAsync(omask.p, masks.data(), kTrajMaxObs * 8, cudaMemcpyHostToDevice, ctx->stream));
  TrajArgs A;
  std::memset(&A, 0, sizeof(A));
  A.n = n;
  A.ld = ld;
  A.ntraj = d.ntraj;
  A.nchan = d.nchan;
  A.nobs = d.nobs;
  A.gamma = d.gamma;
  A.dt = d.dt;
  A.seed = d.seed;
  A.basis = H->sec->basis.p;
  A.psi = psi.p;
  A.psi_new = psi_new.p;
  A.w = w.p;
  A.obs = obs.p;
  A.jumps = jumps.p;
  A.chan_bits = bits.p;
  A.obs_mask = omask.p;
  cublasHandle_t hb = nullptr;
  QD_CUBLAS(cublasCreate(&hb));
  struct HandleGuard {
    cublasHandle_t h;
    ~HandleGuard() {
      if (h) cublasDestroy(h);
    }
  } hg{hb};
  QD_CUBLAS(cublasSetStream(hb, ctx->stream));
  if (cublasSetMathMode(hb, CUBLAS_FP32_EMULATED_BF16X9_MATH) != CUBLAS_STATUS_SUCCESS)
    QD_CUBLAS(cublasSetMathMode(hb, CUBLAS_DEFAULT_MATH));
  const cuComplex one = make_cuComplex(1.f, 0.f), zero = make_cuComplex(0.f, 0.f);
  A.step = 0;
  traj_step_kernel<<<d.ntraj, kTrajThreads, 0, ctx->stream>>>(A);
  QD_CHECK_LAUNCH();
  QD_LAUNCHED(ctx);
  for (int step = 1; step <= d.nsteps; ++step) {
    QD_CUBLAS(cublasCgemm(hb, CUBLAS_OP_N, CUBLAS_OP_N, (int)n, d.ntraj, (int)n, &one,
                          reinterpret_cast<const cuComplex*>(U.p), (int)n,
                          reinterpret_cast<const cuComplex*>(psi.p), (int)ld, &zero,
                          reinterpret_cast<cuComplex*>(psi_new.p), (int)ld));
    A.step = step;
    traj_step_kernel<<<d.ntraj, kTrajThreads, 0, ctx->stream>>>(A);
    QD_CHECK_LAUNCH();
    QD_LAUNCHED(ctx);
  }
  const int nrows = (d.nsteps + 1) * d.nobs;
  if (nrows > 0) {
    DBuf<double> dm(nrows), ds(nrows);
    traj_reduce_kernel<<<(unsigned)ceil_div(nrows, 128), 128, 0, ctx->stream>>>(obs.p, d.ntraj, nrows, dm.p, ds.p);
    QD_CHECK_LAUNCH();
    QD_LAUNCHED(ctx);
    QD_CUDA(cudaMemcpyAsync(obs_mean, dm.p, nrows * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    if (obs_stderr)
      QD_CUDA(cudaMemcpyAsync(obs_stderr, ds.p, nrows * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    QD_CUDA(cudaStreamSynchronize(ctx->stream));
  }
  QD_CUDA(cudaEventRecord(e2, ctx->stream));
  std::vector<int> hj(d.ntraj);
  QD_CUDA(cudaMemcpyAsync(hj.data(), jumps.p, d.ntraj * sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  QD_CUDA(cudaStreamSynchronize(ctx->stream));
  int64_t tot = 0;
  for (int v : hj) tot += v;
  if (jumps_total) *jumps_total = tot;
  if (timings) {
    float a = 0.f, b2 = 0.f;
    cudaEventElapsedTime(&a, e0, e1);
    cudaEventElapsedTime(&b2, e1, e2);
    timings[0] = a;
    timings[1] = b2;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaEventDestroy(e2);
}

}  // namespace qd
