// batch.cu -- many Lanczos ground states in one persistent launch.
//
// The mixed-precision form of the reference's Lanczos (sparse_algorithm.hpp:
// 395-425, 564-585) for a packed work list of independent, uneven instances:
//   * small instances: one CTA owns one instance at a time and takes the next
//     one from an atomic counter;
//   * large instances (dim >= kClusterMinDim): a thread-block cluster of
//     8, 4 or 2 CTAs owns one instance (per call, the largest size at which
//     every large instance of the call is resident at once, else 2: more
//     instances side by side beat wider clusters once the device is full, and
//     an instance's bits depend on this size); each CTA keeps a slice of the rows
//     of every vector, and the inner products are combined through
//     distributed shared memory (each CTA adds the CTAs' partials in rank
//     order, so every CTA holds the same bits) between hardware cluster
//     barriers -- one SM's memory parallelism is far too little for an
//     instance of 10^5 rows;
//   * the lists are sorted by decreasing nnz (longest first);
//   * matrix values and Krylov vectors are FP32 and so is the product;
//   * every inner product keeps FP32 partial sums over at most 64 elements per
//     thread and adds those partials in FP64 (threads, warps, blocks, CTAs);
//   * after the three-term step (the reference's local orthogonalisation
//     against the two previous vectors) the new vector is orthogonalised
//     once more against the whole stored basis (classical Gram-Schmidt);
//   * the tridiagonal matrix (FP64) is solved on the device: eigenvalues by
//     implicit QL, the lowest eigenvector by inverse iteration;
//   * the Ritz vector gets one FP64 refinement: E = psi^T H psi / psi^T psi with
//     the FP64 matrix values and FP64 accumulation.
// No CTA spins on another: the only shared state is the work counter, and the
// CTAs of a cluster meet only at hardware cluster barriers, which the
// hardware schedules together and every CTA of a cluster reaches the same
// number of times (the instance index and every stopping decision are the
// same in all of them).
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <numeric>
#include <vector>

#include <cooperative_groups.h>

#include "batch.cuh"
#include "krylov.cuh"
#include "tridiag.cuh"

namespace cg = cooperative_groups;

namespace qd {

constexpr int kBatchThreads = 512;  // two CTAs per SM
constexpr int kBatchMaxSteps = 256;
constexpr int kChunk = 64;  // FP32 partial sums cover at most this many elements
constexpr int kClusterCtasMax = 8;  // CTAs of a cluster that shares one large instance: 8, 4 or 2 per call
constexpr int64_t kClusterMinDim = 32768;

struct BlockScratch {
  double red[kBatchThreads / 32];
  double bcast;
  double xp[2], bc[2];                    // this CTA's partial of a cluster sum, and the sum
  double hp[2][kBatchMaxSteps + 2];       // this CTA's partials of the Gram-Schmidt coefficients
  double alpha[kBatchMaxSteps + 2];
  double beta[kBatchMaxSteps + 2];
  double y[kBatchMaxSteps + 2];
  double h[kBatchMaxSteps + 2];
  int stop;
  int idx;
};

// The device's nanosecond clock (the instance schedule in out[5], out[6]).
__device__ __forceinline__ unsigned long long batch_clock_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// FP64 sum over the block of per-thread values; every thread gets the result.
__device__ double block_sum_all(double v, BlockScratch& S) {
  v = warp_sum(v);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) S.red[warp] = v;
  __syncthreads();
  if (warp == 0) {
    double t = (lane < (int)(blockDim.x >> 5)) ? S.red[lane] : 0.0;
    t = warp_sum(t);
    if (lane == 0) S.bcast = t;
  }
  __syncthreads();
  return S.bcast;
}

// <a, b> over [lo, hi) with FP32 products and partials over <= kChunk
// elements, FP64 beyond; the block's total in every thread.  lo is a
// multiple of 32 and the vectors start on a 32-element boundary.
__device__ double block_dot(const float* __restrict__ a, const float* __restrict__ b, int64_t lo, int64_t hi,
                            BlockScratch& S) {
  double dacc = 0.0;
  float acc = 0.f;
  int cnt = 0;
  const int64_t q0 = lo >> 2, q1 = hi >> 2;
  const float4* a4 = reinterpret_cast<const float4*>(a);
  const float4* b4 = reinterpret_cast<const float4*>(b);
#pragma unroll 4
  for (int64_t i = q0 + threadIdx.x; i < q1; i += blockDim.x) {
    const float4 x = a4[i], y = b4[i];
    acc = fmaf(x.x, y.x, acc);
    acc = fmaf(x.y, y.y, acc);
    acc = fmaf(x.z, y.z, acc);
    acc = fmaf(x.w, y.w, acc);
    if (++cnt == kChunk / 4) {
      dacc += (double)acc;
      acc = 0.f;
      cnt = 0;
    }
  }
  for (int64_t i = (q1 << 2) + threadIdx.x; i < hi; i += blockDim.x) acc = fmaf(a[i], b[i], acc);
  dacc += (double)acc;
  return block_sum_all(dacc, S);
}

// w -= c * v on [lo, hi)
__device__ void block_axpy(float* __restrict__ w, float c, const float* __restrict__ v, int64_t lo, int64_t hi) {
  const int64_t q0 = lo >> 2, q1 = hi >> 2;
  float4* w4 = reinterpret_cast<float4*>(w);
  const float4* v4 = reinterpret_cast<const float4*>(v);
#pragma unroll 4
  for (int64_t i = q0 + threadIdx.x; i < q1; i += blockDim.x) {
    float4 x = w4[i];
    const float4 y = v4[i];
    x.x = fmaf(-c, y.x, x.x);
    x.y = fmaf(-c, y.y, x.y);
    x.z = fmaf(-c, y.z, x.z);
    x.w = fmaf(-c, y.w, x.w);
    w4[i] = x;
  }
  for (int64_t i = (q1 << 2) + threadIdx.x; i < hi; i += blockDim.x) w[i] = fmaf(-c, v[i], w[i]);
}

// y = H x on rows [lo, hi) (FP32 values, FP32 accumulation), one thread per
// row.  x is a basis vector written earlier in the same launch (by this CTA
// or, for a cluster, by all of its CTAs), so it is read with ordinary loads,
// not the read-only path.
__device__ void block_spmv_f32(const BatchInst& I, const float* x, float* __restrict__ y, int64_t lo, int64_t hi) {
  for (int64_t r = lo + threadIdx.x; r < hi; r += blockDim.x) {
    const int64_t b = I.rowptr[r], e = I.rowptr[r + 1];
    float acc = 0.f;
    int64_t k = b;
    for (; k + 4 <= e; k += 4) {
      const int32_t c0 = I.colidx[k], c1 = I.colidx[k + 1], c2 = I.colidx[k + 2], c3 = I.colidx[k + 3];
      const float v0 = I.vals_f[k], v1 = I.vals_f[k + 1], v2 = I.vals_f[k + 2], v3 = I.vals_f[k + 3];
      const float x0 = x[c0], x1 = x[c1], x2 = x[c2], x3 = x[c3];
      acc = fmaf(v0, x0, acc);
      acc = fmaf(v1, x1, acc);
      acc = fmaf(v2, x2, acc);
      acc = fmaf(v3, x3, acc);
    }
    for (; k < e; ++k) acc = fmaf(I.vals_f[k], x[I.colidx[k]], acc);
    y[r] = acc;
  }
}

// ---------------------------------------------------------------- cluster sums
// A barrier over the instance's CTAs (the block for C == 1).
template <int C>
__device__ __forceinline__ void inst_sync() {
  if constexpr (C > 1) cg::this_cluster().sync();
  else __syncthreads();
}

// The instance total of a block total: every CTA adds the C partials in rank
// order from distributed shared memory.  Double-buffered: a buffer is written
// again only two sums later, after every CTA has passed the barrier between.
template <int C>
__device__ double inst_sum(double block_total, BlockScratch& S, int& buf) {
  if constexpr (C == 1) {
    return block_total;
  } else {
    cg::cluster_group cl = cg::this_cluster();
    if (threadIdx.x == 0) S.xp[buf] = block_total;
    cl.sync();
    if (threadIdx.x == 0) {
      double t = 0.0;
      for (int r = 0; r < C; ++r) t += *cl.map_shared_rank(&S.xp[buf], r);
      S.bc[buf] = t;
    }
    __syncthreads();
    const double t = S.bc[buf];
    buf ^= 1;
    return t;
  }
}

// Lowest eigenpair of tridiag(d, e) (n <= kBatchMaxSteps), one thread:
// eigenvalues by QL, eigenvector by two steps of inverse iteration with
// partial pivoting (the reorthogonalised Lanczos matrix has no spurious copies).
__device__ double device_tridiag_lowest(int n, const double* d_in, const double* e_in, double* y, double* work) {
  double* d = work;
  double* e = work + (kBatchMaxSteps + 2);
  for (int i = 0; i < n; ++i) {
    d[i] = d_in[i];
    e[i] = (i + 1 < n) ? e_in[i] : 0.0;
  }
  tridiag_ql<double>(n, d, e, nullptr, 0);
  const double lam = d[0];
  // (T - sigma I) y = b, sigma just below lam; Gaussian elimination with
  // partial pivoting on the tridiagonal band (three diagonals + fill-in)
  double* dl = work + 2 * (kBatchMaxSteps + 2);
  double* dd = work + 3 * (kBatchMaxSteps + 2);
  double* du = work + 4 * (kBatchMaxSteps + 2);
  double* du2 = work + 5 * (kBatchMaxSteps + 2);
  int* piv = reinterpret_cast<int*>(work + 6 * (kBatchMaxSteps + 2));
  const double scale = fmax(fabs(lam), 1.0);
  const double sigma = lam - 1e-10 * scale;
  for (int i = 0; i < n; ++i) y[i] = 1.0;
  for (int it = 0; it < 3; ++it) {
    for (int i = 0; i < n; ++i) {
      dd[i] = d_in[i] - sigma;
      du[i] = (i + 1 < n) ? e_in[i] : 0.0;
      dl[i] = (i + 1 < n) ? e_in[i] : 0.0;
      du2[i] = 0.0;
    }
    // factor
    for (int i = 0; i < n - 1; ++i) {
      if (fabs(dd[i]) >= fabs(dl[i])) {
        piv[i] = i;
        const double f = (dd[i] != 0.0) ? dl[i] / dd[i] : 0.0;
        dl[i] = f;
        dd[i + 1] -= f * du[i];
      } else {
        piv[i] = i + 1;
        const double f = dd[i] / dl[i];
        dd[i] = dl[i];
        dl[i] = f;
        const double t = du[i];
        du[i] = dd[i + 1];
        dd[i + 1] = t - f * dd[i + 1];
        if (i < n - 2) {
          du2[i] = du[i + 1];
          du[i + 1] = -f * du[i + 1];
        }
      }
    }
    // solve L U x = P b
    for (int i = 0; i < n - 1; ++i) {
      if (piv[i] == i) {
        y[i + 1] -= dl[i] * y[i];
      } else {
        const double t = y[i];
        y[i] = y[i + 1];
        y[i + 1] = t - dl[i] * y[i + 1];
      }
    }
    for (int i = n - 1; i >= 0; --i) {
      double s = y[i];
      if (i + 1 < n) s -= du[i] * y[i + 1];
      if (i + 2 < n) s -= du2[i] * y[i + 2];
      const double p = (dd[i] != 0.0) ? dd[i] : 1e-300;
      y[i] = s / p;
    }
    double nr = 0.0;
    for (int i = 0; i < n; ++i) nr += y[i] * y[i];
    nr = sqrt(nr);
    for (int i = 0; i < n; ++i) y[i] /= nr;
  }
  return lam;
}

template <int C>
__global__ void __launch_bounds__(kBatchThreads, 2) batch_lanczos_kernel(const BatchInst* __restrict__ list, int ninst,
                                                                     unsigned* counter, double* tri_work) {
  __shared__ BlockScratch S;
  int rank = 0;
  if constexpr (C > 1) rank = (int)cg::this_cluster().block_rank();
  int buf = 0, hbuf = 0;
  for (;;) {
    if (rank == 0 && threadIdx.x == 0) S.idx = (int)atomicAdd(counter, 1u);
    inst_sync<C>();
    int idx;
    if constexpr (C > 1) idx = *cg::this_cluster().map_shared_rank(&S.idx, 0);
    else idx = S.idx;
    inst_sync<C>();
    if (idx >= ninst) return;  // the same index in every CTA of the cluster
    const BatchInst I = list[idx];
    const unsigned long long t_start = batch_clock_ns();
    const int64_t n = I.dim;
    // this CTA's rows: a slice of 32-element multiples (the whole vector for C == 1)
    const int64_t per = ((n + C - 1) / C + 31) / 32 * 32;
    const int64_t lo = std::min<int64_t>(n, (int64_t)rank * per), hi = std::min<int64_t>(n, lo + per);
    float* V = I.V;
    float* w = I.w;
    // v_0 = v0 / ||v0||
    const double nrm0 = sqrt(inst_sum<C>(block_dot(I.v0, I.v0, lo, hi, S), S, buf));
    const float inv0 = (float)(1.0 / nrm0);
    for (int64_t i = lo + threadIdx.x; i < hi; i += blockDim.x) V[i] = I.v0[i] * inv0;
    if (threadIdx.x == 0) S.stop = 0;
    inst_sync<C>();
    int act = I.steps;
    for (int k = 1; k <= I.steps; ++k) {
      const float* v1 = V + (int64_t)(k - 1) * I.ld;
      const float* v2 = (k >= 2) ? V + (int64_t)(k - 2) * I.ld : nullptr;
      block_spmv_f32(I, v1, w, lo, hi);
      __syncthreads();
      double bp = 0.0;
      if (v2) {
        bp = inst_sum<C>(block_dot(v2, w, lo, hi, S), S, buf);
        block_axpy(w, (float)bp, v2, lo, hi);
        __syncthreads();
      }
      const double al = inst_sum<C>(block_dot(v1, w, lo, hi, S), S, buf);
      block_axpy(w, (float)al, v1, lo, hi);
      __syncthreads();
      // one full Gram-Schmidt pass against v_0 .. v_{k-1}: a warp per basis vector
      {
        const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
        const int64_t q0 = lo >> 2, q1 = hi >> 2;
        const float4* w4 = reinterpret_cast<const float4*>(w);
        double* part = (C > 1) ? S.hp[hbuf] : S.h;
        for (int j = warp; j < k; j += nw) {
          const float* vj = V + (int64_t)j * I.ld;
          const float4* vj4 = reinterpret_cast<const float4*>(vj);
          double dacc = 0.0;
          float acc = 0.f;
          int cnt = 0;
          int64_t i = q0 + lane;
          for (; i + 96 < q1; i += 128) {  // four float4 pairs in flight per lane
            const float4 x0 = vj4[i], y0 = w4[i], x1 = vj4[i + 32], y1 = w4[i + 32];
            const float4 x2 = vj4[i + 64], y2 = w4[i + 64], x3 = vj4[i + 96], y3 = w4[i + 96];
            acc = fmaf(x0.x, y0.x, acc);
            acc = fmaf(x0.y, y0.y, acc);
            acc = fmaf(x0.z, y0.z, acc);
            acc = fmaf(x0.w, y0.w, acc);
            acc = fmaf(x1.x, y1.x, acc);
            acc = fmaf(x1.y, y1.y, acc);
            acc = fmaf(x1.z, y1.z, acc);
            acc = fmaf(x1.w, y1.w, acc);
            acc = fmaf(x2.x, y2.x, acc);
            acc = fmaf(x2.y, y2.y, acc);
            acc = fmaf(x2.z, y2.z, acc);
            acc = fmaf(x2.w, y2.w, acc);
            acc = fmaf(x3.x, y3.x, acc);
            acc = fmaf(x3.y, y3.y, acc);
            acc = fmaf(x3.z, y3.z, acc);
            acc = fmaf(x3.w, y3.w, acc);
            cnt += 4;
            if (cnt >= kChunk / 4) {
              dacc += (double)acc;
              acc = 0.f;
              cnt = 0;
            }
          }
          for (; i < q1; i += 32) {
            const float4 x = vj4[i], y = w4[i];
            acc = fmaf(x.x, y.x, acc);
            acc = fmaf(x.y, y.y, acc);
            acc = fmaf(x.z, y.z, acc);
            acc = fmaf(x.w, y.w, acc);
            if (++cnt == kChunk / 4) {
              dacc += (double)acc;
              acc = 0.f;
              cnt = 0;
            }
          }
          for (int64_t i = (q1 << 2) + lane; i < hi; i += 32) acc = fmaf(vj[i], w[i], acc);
          dacc += (double)acc;
          dacc = warp_sum(dacc);
          if (lane == 0) part[j] = dacc;
        }
        if constexpr (C > 1) {  // the coefficients of the whole vector, the same bits in every CTA
          cg::cluster_group cl = cg::this_cluster();
          cl.sync();
          for (int j = threadIdx.x; j < k; j += blockDim.x) {
            double t = 0.0;
            for (int r = 0; r < C; ++r) t += *cl.map_shared_rank(&S.hp[hbuf][j], r);
            S.h[j] = t;
          }
          hbuf ^= 1;
        }
        __syncthreads();
        float4* wm4 = reinterpret_cast<float4*>(w);
        const int64_t bs = blockDim.x;
        int64_t i = q0 + threadIdx.x;
        for (; i + bs < q1; i += 2 * bs) {  // two float4 of w per thread: two independent chains
          float4 x = wm4[i], u = wm4[i + bs];
#pragma unroll 4
          for (int j = 0; j < k; ++j) {
            const float c = -(float)S.h[j];
            const float4* vj4 = reinterpret_cast<const float4*>(V + (int64_t)j * I.ld);
            const float4 y = vj4[i], z = vj4[i + bs];
            x.x = fmaf(c, y.x, x.x);
            x.y = fmaf(c, y.y, x.y);
            x.z = fmaf(c, y.z, x.z);
            x.w = fmaf(c, y.w, x.w);
            u.x = fmaf(c, z.x, u.x);
            u.y = fmaf(c, z.y, u.y);
            u.z = fmaf(c, z.z, u.z);
            u.w = fmaf(c, z.w, u.w);
          }
          wm4[i] = x;
          wm4[i + bs] = u;
        }
        for (; i < q1; i += bs) {
          float4 x = wm4[i];
#pragma unroll 4
          for (int j = 0; j < k; ++j) {
            const float c = -(float)S.h[j];
            const float4 y = reinterpret_cast<const float4*>(V + (int64_t)j * I.ld)[i];
            x.x = fmaf(c, y.x, x.x);
            x.y = fmaf(c, y.y, x.y);
            x.z = fmaf(c, y.z, x.z);
            x.w = fmaf(c, y.w, x.w);
          }
          wm4[i] = x;
        }
        for (int64_t i = (q1 << 2) + threadIdx.x; i < hi; i += blockDim.x) {
          float wi = w[i];
          for (int j = 0; j < k; ++j) wi = fmaf(-(float)S.h[j], V[(int64_t)j * I.ld + i], wi);
          w[i] = wi;
        }
        __syncthreads();
      }
      const double nr = sqrt(inst_sum<C>(block_dot(w, w, lo, hi, S), S, buf));
      if (threadIdx.x == 0) {
        S.alpha[k] = al + S.h[k - 1];
        S.beta[k] = nr;
        // breakdown (sparse_algorithm.hpp:421): the reference's 1e-10, or the
        // FP32 resolution of the recurrence, or an exhausted space
        const double scale = fabs(al) + fabs(bp) + (k >= 2 ? S.beta[k - 1] : 0.0);
        if (nr < 1e-10 || nr < 1e-5 * scale || k >= n) S.stop = k;
      }
      __syncthreads();
      if (S.stop) {  // the same decision in every CTA of the cluster
        act = k;     // v_0 .. v_{k-1} span an invariant subspace: T_k is exact
        break;
      }
      const float inv = (float)(1.0 / nr);
      float* vk = V + (int64_t)k * I.ld;
      for (int64_t i = lo + threadIdx.x; i < hi; i += blockDim.x) vk[i] = w[i] * inv;
      inst_sync<C>();  // the next product reads all of v_k
    }
    if (act < 1) act = 1;
    // lowest Ritz pair of tridiag(alpha_1..act, beta_1..act-1), the same in every CTA
    if (threadIdx.x == 0) {
      double* work = tri_work + (size_t)blockIdx.x * 8 * (kBatchMaxSteps + 2);
      const double lam = device_tridiag_lowest(act, S.alpha + 1, S.beta + 1, S.y, work);
      if (rank == 0) {
        I.out[0] = lam;
        I.out[3] = act;
        I.out[4] = S.stop ? 1 : 0;
      }
    }
    __syncthreads();
    // Ritz vector psi = sum_k y_k v_k (FP32 storage)
    for (int64_t i = lo + threadIdx.x; i < hi; i += blockDim.x) {
      float acc = 0.f;
      for (int k = 0; k < act; ++k) acc = fmaf((float)S.y[k], V[(int64_t)k * I.ld + i], acc);
      I.psi[i] = acc;
    }
    inst_sync<C>();  // the refinement reads all of psi
    // FP64 refinement: Rayleigh quotient with the FP64 values
    double num = 0.0, den = 0.0;
    for (int64_t r = lo + threadIdx.x; r < hi; r += blockDim.x) {
      double hr = 0.0;
      for (int64_t e = I.rowptr[r]; e < I.rowptr[r + 1]; ++e) hr = fma(I.vals_d[e], (double)I.psi[I.colidx[e]], hr);
      const double pr = (double)I.psi[r];
      num = fma(pr, hr, num);
      den = fma(pr, pr, den);
    }
    num = inst_sum<C>(block_sum_all(num, S), S, buf);
    den = inst_sum<C>(block_sum_all(den, S), S, buf);
    if (rank == 0 && threadIdx.x == 0) {
      I.out[1] = num / den;
      I.out[2] = den;
      I.out[5] = (double)t_start;
      I.out[6] = (double)batch_clock_ns();
      I.out[7] = (double)C;
    }
    inst_sync<C>();
  }
}

// Launches kernel C over `count` instances of `list` with `grid` CTAs
// (clusters of C CTAs for C > 1).
template <int C>
static void launch_batch(Ctx* ctx, cudaStream_t stream, const BatchInst* list, int count, unsigned* counter,
                         double* tri_work, int grid) {
  if (count <= 0) return;
  if constexpr (C == 1) {
    batch_lanczos_kernel<1><<<grid, kBatchThreads, 0, stream>>>(list, count, counter, tri_work);
  } else {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3(kBatchThreads);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = C;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    QD_CUDA(cudaLaunchKernelEx(&cfg, batch_lanczos_kernel<C>, list, count, counter, tri_work));
  }
  QD_CHECK_LAUNCH();
  QD_LAUNCHED(ctx);
}

// Clusters of C CTAs the device keeps resident at once (0 if none).
template <int C>
static int resident_clusters(Ctx* ctx) {
  static thread_local int cached = -1;
  if (cached >= 0) return cached;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)(C * 2 * ctx->num_sms));
  cfg.blockDim = dim3(kBatchThreads);
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = C;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  int n = 0;
  if (cudaOccupancyMaxActiveClusters(&n, batch_lanczos_kernel<C>, &cfg) != cudaSuccess) {
    cudaGetLastError();
    n = 0;
  }
  cached = n;
  return n;
}

void batch_lanczos(Ctx* ctx, qd_ham* const* hams, const double* const* v0s, int ninst, int steps, double* out) {
  QD_REQUIRE(ninst >= 1, QD_ERR_INVALID, "empty batch");
  QD_REQUIRE(steps >= 1 && steps <= kBatchMaxSteps, QD_ERR_INVALID, "steps must be in 1..%d", kBatchMaxSteps);
  std::vector<int> order(ninst);
  std::iota(order.begin(), order.end(), 0);
  for (int i = 0; i < ninst; ++i) {
    QD_REQUIRE(hams[i] && v0s[i], QD_ERR_INVALID, "instance %d: null argument", i);
    QD_REQUIRE(hams[i]->flags & QD_HAM_REAL, QD_ERR_UNSUPPORTED,
               "instance %d: the batched mixed-precision solver needs a real Hamiltonian", i);
    QD_REQUIRE(hams[i]->ctx == ctx, QD_ERR_INVALID, "instance %d: Hamiltonian of another context", i);
  }
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return hams[a]->nnz > hams[b]->nnz; });
  // large instances (a cluster each) first, each class longest first
  std::stable_partition(order.begin(), order.end(), [&](int a) { return hams[a]->dim >= kClusterMinDim; });
  // one arena for every instance's basis, work vector and Ritz vector
  std::vector<int64_t> off_V(ninst), off_w(ninst), off_psi(ninst);
  int64_t total = 0;
  for (int i = 0; i < ninst; ++i) {
    const int64_t ld = (hams[i]->dim + 31) / 32 * 32;
    off_V[i] = total;
    total += (int64_t)(steps + 1) * ld;
    off_w[i] = total;
    total += ld;
    off_psi[i] = total;
    total += ld;
  }
  DBuf<float> arena(total);
  DBuf<double> dout((size_t)ninst * 8);
  QD_CUDA(cudaMemsetAsync(dout.p, 0, dout.bytes(), ctx->stream));
  // the start vectors, in FP32, in one copy
  int64_t v0_total = 0;
  for (int i = 0; i < ninst; ++i) v0_total += (hams[i]->dim + 31) / 32 * 32;
  std::vector<float> h32((size_t)v0_total, 0.f);
  DBuf<float> v0buf(v0_total);
  std::vector<int64_t> off_h(ninst);
  for (int i = 0; i < ninst; ++i) {
    off_h[i] = (i == 0) ? 0 : off_h[i - 1] + (hams[i - 1]->dim + 31) / 32 * 32;
    for (int64_t q = 0; q < hams[i]->dim; ++q) h32[(size_t)(off_h[i] + q)] = (float)v0s[i][q];
  }
  QD_CUDA(cudaMemcpyAsync(v0buf.p, h32.data(), h32.size() * sizeof(float), cudaMemcpyHostToDevice, ctx->stream));
  // the work list: large instances, then small ones
  std::vector<BatchInst> list(ninst);
  int nlarge = 0;
  for (int q = 0; q < ninst; ++q) nlarge += (hams[order[q]]->dim >= kClusterMinDim) ? 1 : 0;
  // cluster size: the largest whose resident clusters hold every large instance at once, else 2
  int ctas = 2, nclusters = resident_clusters<2>(ctx);
  if (resident_clusters<8>(ctx) >= nlarge) {
    ctas = 8;
    nclusters = resident_clusters<8>(ctx);
  } else if (resident_clusters<4>(ctx) >= nlarge) {
    ctas = 4;
    nclusters = resident_clusters<4>(ctx);
  }
  if (nclusters < 1) nlarge = 0;  // no cluster fits: every instance on one CTA
  for (int q = 0; q < ninst; ++q) {
    const int i = order[q];
    const qd_ham* H = hams[i];
    BatchInst& I = list[q];
    std::memset(&I, 0, sizeof(I));
    I.dim = H->dim;
    I.steps = steps;
    I.ld = (H->dim + 31) / 32 * 32;
    I.rowptr = H->rowptr.p;
    I.colidx = H->colidx.p;
    I.vals_f = H->vals_f.p;
    I.vals_d = H->vals_r.p;
    I.v0 = v0buf.p + off_h[i];
    I.V = arena.p + off_V[i];
    I.w = arena.p + off_w[i];
    I.psi = arena.p + off_psi[i];
    I.out = dout.p + (size_t)i * 8;
  }
  DBuf<BatchInst> dlist(ninst);
  QD_CUDA(cudaMemcpyAsync(dlist.p, list.data(), ninst * sizeof(BatchInst), cudaMemcpyHostToDevice, ctx->stream));
  DBuf<unsigned> counter(2);
  QD_CUDA(cudaMemsetAsync(counter.p, 0, 2 * sizeof(unsigned), ctx->stream));
  const int nsmall = ninst - nlarge;
  const int grid_large = nlarge ? ctas * std::min(nlarge, nclusters) : 0;
  const int grid_small = nsmall ? std::min(nsmall, 2 * ctx->num_sms) : 0;
  // one scratch region per CTA of either launch (they may run at the same time)
  DBuf<double> tri_work((size_t)std::max(grid_large + grid_small, 1) * 8 * (kBatchMaxSteps + 2));
  double* tri_small = tri_work.p + (size_t)grid_large * 8 * (kBatchMaxSteps + 2);
  // With both classes present the cluster launch goes on a high-priority side
  // stream and the single-CTA launch beside it on the context's stream: the
  // clusters are placed first, and single CTAs take the SM slots the clusters
  // leave (and free at the end).  Every instance is computed by its own CTAs
  // in a fixed order, so the results do not depend on the overlap.
  struct Side {
    cudaStream_t s = nullptr;
    cudaEvent_t in = nullptr, done = nullptr;
    ~Side() {
      if (in) cudaEventDestroy(in);
      if (done) cudaEventDestroy(done);
      if (s) cudaStreamDestroy(s);
    }
  } side;
  cudaStream_t large_stream = ctx->stream;
  if (nlarge > 0 && nsmall > 0) {
    int least = 0, greatest = 0;
    QD_CUDA(cudaDeviceGetStreamPriorityRange(&least, &greatest));
    QD_CUDA(cudaStreamCreateWithPriority(&side.s, cudaStreamNonBlocking, greatest));
    QD_CUDA(cudaEventCreateWithFlags(&side.in, cudaEventDisableTiming));
    QD_CUDA(cudaEventCreateWithFlags(&side.done, cudaEventDisableTiming));
    QD_CUDA(cudaEventRecord(side.in, ctx->stream));  // the list, the start vectors and the counters are in place
    QD_CUDA(cudaStreamWaitEvent(side.s, side.in, 0));
    large_stream = side.s;
  }
  const bool timing = std::getenv("QD_TIMING") != nullptr;
  if (timing) QD_CUDA(cudaEventRecord(ctx->events[12], ctx->stream));
  if (ctas == 8) launch_batch<8>(ctx, large_stream, dlist.p, nlarge, counter.p, tri_work.p, grid_large);
  else if (ctas == 4) launch_batch<4>(ctx, large_stream, dlist.p, nlarge, counter.p, tri_work.p, grid_large);
  else launch_batch<2>(ctx, large_stream, dlist.p, nlarge, counter.p, tri_work.p, grid_large);
  launch_batch<1>(ctx, ctx->stream, dlist.p + nlarge, nsmall, counter.p + 1, tri_small, grid_small);
  if (timing) QD_CUDA(cudaEventRecord(ctx->events[14], ctx->stream));
  if (side.s) {
    QD_CUDA(cudaEventRecord(side.done, side.s));
    QD_CUDA(cudaStreamWaitEvent(ctx->stream, side.done, 0));
  }
  if (timing) QD_CUDA(cudaEventRecord(ctx->events[13], ctx->stream));
  QD_CUDA(cudaMemcpyAsync(out, dout.p, (size_t)ninst * 8 * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  QD_CUDA(cudaStreamSynchronize(ctx->stream));
  if (timing) {
    float a = 0.f, b = 0.f;
    QD_CUDA(cudaEventElapsedTime(&a, ctx->events[12], ctx->events[13]));
    QD_CUDA(cudaEventElapsedTime(&b, ctx->events[12], ctx->events[14]));
    std::fprintf(stderr, "[qd timing] batch: %d large on %d clusters, %d small on %d CTAs: all done at %.3f ms, "
                 "small done at %.3f ms (%d-CTA clusters)\n", nlarge, grid_large / ctas, nsmall, grid_small, a, b, ctas);
  }
}

}  // namespace qd
