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
#include <memory>
#include <numeric>
#include <thread>
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
constexpr int64_t kClusterMinDim = 32768;

constexpr int kWTile = 4096;  // elements of w staged in shared memory for the Gram-Schmidt coefficients

struct BlockScratch {
  float wt[kWTile];
  double red[kBatchThreads / 32];
  double red3[kBatchThreads / 32][3];
  double bcast;
  double bcast3[3];
  double xp[2], bc[2];                    // this CTA's partial of a cluster sum, and the sum
  double xp3[2][3], bc3[2][3];
  double hp[2][kBatchMaxSteps + 2];       // this CTA's partials of the Gram-Schmidt coefficients
  double alpha[kBatchMaxSteps + 2];
  double beta[kBatchMaxSteps + 2];
  double y[kBatchMaxSteps + 2];
  double h[kBatchMaxSteps + 2];
  double c[kBatchMaxSteps + 2];           // update coefficients of the stored vectors
  double scl[kBatchMaxSteps + 2];         // basis vector j is scl[j] * V[j] (V stored unnormalised)
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
  v = warp_sum0(v);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) S.red[warp] = v;
  __syncthreads();
  if (warp == 0) {
    double t = (lane < (int)(blockDim.x >> 5)) ? S.red[lane] : 0.0;
    t = warp_sum0(t);
    if (lane == 0) S.bcast = t;
  }
  __syncthreads();
  return S.bcast;
}

// The same for three values at once.
__device__ void block_sum_all3(double (&v)[3], BlockScratch& S) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int q = 0; q < 3; ++q) v[q] = warp_sum0(v[q]);
  __syncthreads();
  if (lane == 0) {
#pragma unroll
    for (int q = 0; q < 3; ++q) S.red3[warp][q] = v[q];
  }
  __syncthreads();
  if (warp == 0) {
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      double t = (lane < (int)(blockDim.x >> 5)) ? S.red3[lane][q] : 0.0;
      t = warp_sum0(t);
      if (lane == 0) S.bcast3[q] = t;
    }
  }
  __syncthreads();
#pragma unroll
  for (int q = 0; q < 3; ++q) v[q] = S.bcast3[q];
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

// y = H x on rows [lo, hi) (FP32 values, FP32 accumulation), one thread per
// row, two rows per thread at a time (r and r + blockDim.x: two independent
// chains of four gathers), each summed in its entry order.  x is a basis
// vector written earlier in the same launch (by this CTA or, for a cluster, by
// all of its CTAs), so it is read with ordinary loads, not the read-only path.
__device__ __forceinline__ float row_f32(const BatchInst& I, const float* x, int64_t b, int64_t e) {
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
  return acc;
}

// The product of the step and, row by row as it is formed, this thread's
// shares of <V2, y>, <V1, y> and <V1, V2> (FP32 over at most kChunk rows, FP64
// beyond; V2 null on the first step).
struct ProdDots {
  float fa = 0.f, fb = 0.f, fc = 0.f;
  double da = 0.0, db = 0.0, dc = 0.0;
  int cnt = 0;
  __device__ __forceinline__ void add(const float* x, const float* v2, int64_t r, float yr) {
    const float x1 = x[r];
    fb = fmaf(x1, yr, fb);
    if (v2) {
      const float x2 = v2[r];
      fa = fmaf(x2, yr, fa);
      fc = fmaf(x1, x2, fc);
    }
    if (++cnt == kChunk) flush();
  }
  __device__ __forceinline__ void flush() {
    da += (double)fa;
    db += (double)fb;
    dc += (double)fc;
    fa = fb = fc = 0.f;
    cnt = 0;
  }
};

// The same product when every off-diagonal value is one c (uniform hopping, any
// diagonal): y_r = c (sum of x over the row's stored columns) + e_r x_r with
// e_r = d_r - c where the row stores its diagonal (else 0), the column indices
// the only per-entry reads (no values).
__device__ void block_spmv_f32_uniform(const BatchInst& I, const float* x, const float* v2, float* __restrict__ y,
                                       int64_t lo, int64_t hi, ProdDots& pd) {
  const float c = __ldg(I.coff);
  const int64_t bs = blockDim.x;
  int64_t r = lo + threadIdx.x;
  auto finish = [&](int64_t row, float sum) {
    const float yr = fmaf(c, sum, __ldg(I.diag_f + row) * x[row]);
    y[row] = yr;
    pd.add(x, v2, row, yr);
  };
  for (; r + bs < hi; r += 2 * bs) {
    const int64_t b0 = I.rowptr[r], e0 = I.rowptr[r + 1], b1 = I.rowptr[r + bs], e1 = I.rowptr[r + bs + 1];
    float a0 = 0.f, a1 = 0.f;
    int64_t k0 = b0, k1 = b1;
    for (; k0 + 4 <= e0 && k1 + 4 <= e1; k0 += 4, k1 += 4) {  // eight gathers in flight
      const int32_t c0 = I.colidx[k0], c1 = I.colidx[k0 + 1], c2 = I.colidx[k0 + 2], c3 = I.colidx[k0 + 3];
      const int32_t d0 = I.colidx[k1], d1 = I.colidx[k1 + 1], d2 = I.colidx[k1 + 2], d3 = I.colidx[k1 + 3];
      a0 += (x[c0] + x[c1]) + (x[c2] + x[c3]);
      a1 += (x[d0] + x[d1]) + (x[d2] + x[d3]);
    }
    for (; k0 < e0; ++k0) a0 += x[I.colidx[k0]];
    for (; k1 < e1; ++k1) a1 += x[I.colidx[k1]];
    finish(r, a0);
    finish(r + bs, a1);
  }
  if (r < hi) {
    float a0 = 0.f;
    for (int64_t k = I.rowptr[r]; k < I.rowptr[r + 1]; ++k) a0 += x[I.colidx[k]];
    finish(r, a0);
  }
  pd.flush();
}

__device__ void block_spmv_f32(const BatchInst& I, const float* x, const float* v2, float* __restrict__ y, int64_t lo,
                               int64_t hi, ProdDots& pd) {
  const int64_t bs = blockDim.x;
  int64_t r = lo + threadIdx.x;
  for (; r + bs < hi; r += 2 * bs) {
    const int64_t b0 = I.rowptr[r], e0 = I.rowptr[r + 1], b1 = I.rowptr[r + bs], e1 = I.rowptr[r + bs + 1];
    // the two rows' groups of four interleaved: eight gathers in flight
    float a0 = 0.f, a1 = 0.f;
    int64_t k0 = b0, k1 = b1;
    for (; k0 + 4 <= e0 && k1 + 4 <= e1; k0 += 4, k1 += 4) {
      const int32_t c0 = I.colidx[k0], c1 = I.colidx[k0 + 1], c2 = I.colidx[k0 + 2], c3 = I.colidx[k0 + 3];
      const int32_t d0 = I.colidx[k1], d1 = I.colidx[k1 + 1], d2 = I.colidx[k1 + 2], d3 = I.colidx[k1 + 3];
      const float v0 = I.vals_f[k0], v1 = I.vals_f[k0 + 1], w2 = I.vals_f[k0 + 2], v3 = I.vals_f[k0 + 3];
      const float u0 = I.vals_f[k1], u1 = I.vals_f[k1 + 1], u2 = I.vals_f[k1 + 2], u3 = I.vals_f[k1 + 3];
      const float x0 = x[c0], x1 = x[c1], x2 = x[c2], x3 = x[c3];
      const float z0 = x[d0], z1 = x[d1], z2 = x[d2], z3 = x[d3];
      a0 = fmaf(v0, x0, a0);
      a0 = fmaf(v1, x1, a0);
      a0 = fmaf(w2, x2, a0);
      a0 = fmaf(v3, x3, a0);
      a1 = fmaf(u0, z0, a1);
      a1 = fmaf(u1, z1, a1);
      a1 = fmaf(u2, z2, a1);
      a1 = fmaf(u3, z3, a1);
    }
    // the rest of each row, continuing its sum in entry order
    for (; k0 < e0; ++k0) a0 = fmaf(I.vals_f[k0], x[I.colidx[k0]], a0);
    for (; k1 < e1; ++k1) a1 = fmaf(I.vals_f[k1], x[I.colidx[k1]], a1);
    y[r] = a0;
    y[r + bs] = a1;
    pd.add(x, v2, r, a0);
    pd.add(x, v2, r + bs, a1);
  }
  if (r < hi) {
    const float a0 = row_f32(I, x, I.rowptr[r], I.rowptr[r + 1]);
    y[r] = a0;
    pd.add(x, v2, r, a0);
  }
  pd.flush();
}

// ---------------------------------------------------------------- uniform check
struct BunJob {
  int64_t n;
  const int64_t* rowptr;
  const int32_t* colidx;
  const float* vals;
  int* flag;
  float* c;
  float* d;
};

// One CTA per Hamiltonian: c = the first off-diagonal value (rows in order), then flag = 1
// if every off-diagonal value equals c and c is not 0 (an explicit zero off the diagonal
// fails: the uniform form would add it as c), and d_r = diagonal - c where the row stores
// its diagonal, else 0.
__global__ void __launch_bounds__(512) bun_check_kernel(const BunJob* jobs) {
  const BunJob J = jobs[blockIdx.x];
  __shared__ float sc;
  __shared__ int found, bad;
  __shared__ unsigned long long first;  // the first row with an off-diagonal entry
  if (threadIdx.x == 0) {
    found = 0;
    bad = 0;
    first = ~0ull;
  }
  __syncthreads();
  for (int64_t r = threadIdx.x; r < J.n; r += blockDim.x) {
    bool off = false;
    for (int64_t k = J.rowptr[r]; k < J.rowptr[r + 1] && !off; ++k) off = J.colidx[k] != (int32_t)r;
    if (off) {
      atomicMin(&first, (unsigned long long)r);
      break;  // this thread's later rows are larger
    }
  }
  __syncthreads();
  if (threadIdx.x == 0 && first != ~0ull) {
    const int64_t r = (int64_t)first;
    for (int64_t k = J.rowptr[r]; k < J.rowptr[r + 1]; ++k)
      if (J.colidx[k] != (int32_t)r) {
        sc = J.vals[k];
        found = 1;
        break;
      }
  }
  __syncthreads();
  const float c = found ? sc : 0.f;
  for (int64_t r = threadIdx.x; r < J.n; r += blockDim.x) {
    float d = 0.f;  // d_r - c where the row stores its diagonal (its x_r is in the column sum), else 0
    for (int64_t k = J.rowptr[r]; k < J.rowptr[r + 1]; ++k) {
      if (J.colidx[k] == (int32_t)r) d = J.vals[k] - c;
      else if (J.vals[k] != c || c == 0.f) bad = 1;
    }
    J.d[r] = d;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    *J.flag = (found && !bad) ? 1 : 0;
    *J.c = c;
  }
}

// The check for the Hamiltonians of a call that have not had it, in one launch.
static void check_uniform(Ctx* ctx, qd_ham* const* hams, int ninst) {
  std::vector<BunJob> jobs;
  std::vector<qd_ham*> done;
  for (int i = 0; i < ninst; ++i) {
    qd_ham* H = hams[i];
    if (H->bun_checked || std::find(done.begin(), done.end(), H) != done.end()) continue;
    H->bun_d.alloc(H->dim + 4);  // e_r, then c at [dim], the flag's bits at [dim + 1]
    float* c = H->bun_d.p + H->dim;
    jobs.push_back(BunJob{H->dim, H->rowptr.p, H->colidx.p, H->vals_f.p, reinterpret_cast<int*>(c + 1), c,
                          H->bun_d.p});
    done.push_back(H);
  }
  if (jobs.empty()) return;
  DBuf<BunJob> dj(jobs.size());
  QD_CUDA(cudaMemcpyAsync(dj.p, jobs.data(), jobs.size() * sizeof(BunJob), cudaMemcpyHostToDevice, ctx->stream));
  for (size_t j0 = 0; j0 < jobs.size(); j0 += 65535) {
    const unsigned cnt = (unsigned)std::min<size_t>(65535, jobs.size() - j0);
    bun_check_kernel<<<cnt, 512, 0, ctx->stream>>>(dj.p + j0);
    QD_CHECK_LAUNCH();
    QD_LAUNCHED(ctx);
  }
  QD_CUDA(cudaStreamSynchronize(ctx->stream));  // dj is freed on return
  for (qd_ham* H : done) H->bun_checked = true;
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

// The instance totals of three block totals (one cluster barrier).
template <int C>
__device__ void inst_sum3(double (&v)[3], BlockScratch& S, int& buf) {
  if constexpr (C > 1) {
    cg::cluster_group cl = cg::this_cluster();
    if (threadIdx.x == 0) {
#pragma unroll
      for (int q = 0; q < 3; ++q) S.xp3[buf][q] = v[q];
    }
    cl.sync();
    if (threadIdx.x < 3) {
      double t = 0.0;
      for (int r = 0; r < C; ++r) t += cl.map_shared_rank(&S.xp3[buf][0], r)[threadIdx.x];
      S.bc3[buf][threadIdx.x] = t;
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < 3; ++q) v[q] = S.bc3[buf][q];
    buf ^= 1;
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
    const bool uni = I.uniform && __ldg(I.uniform) == 1;
    // v_0 = v0 / ||v0||
    const double nrm0 = sqrt(inst_sum<C>(block_dot(I.v0, I.v0, lo, hi, S), S, buf));
    const float inv0 = (float)(1.0 / nrm0);
    for (int64_t i = lo + threadIdx.x; i < hi; i += blockDim.x) V[i] = I.v0[i] * inv0;
    if (threadIdx.x == 0) {
      S.stop = 0;
      S.scl[0] = 1.0;
    }
    inst_sync<C>();
    int act = I.steps;
    // The basis is stored unnormalised: vector j is scl[j] V[j].  A step forms y = H V[k-1]
    // with the three inner products of the reference's local orthogonalisation, folds
    // u = y - c2 V[k-2] - c1 V[k-1] into the first read of the Gram-Schmidt pass, and
    // writes the orthogonalised u, times a power of two near 1 / ||u||, to V[k] itself.
    for (int k = 1; k <= I.steps; ++k) {
      const float* v1 = V + (int64_t)(k - 1) * I.ld;
      const float* v2 = (k >= 2) ? V + (int64_t)(k - 2) * I.ld : nullptr;
      const double s1 = S.scl[k - 1], s2 = (k >= 2) ? S.scl[k - 2] : 0.0;
      ProdDots pd;
      if (uni) block_spmv_f32_uniform(I, v1, v2, w, lo, hi, pd);
      else block_spmv_f32(I, v1, v2, w, lo, hi, pd);
      double d3[3] = {pd.da, pd.db, pd.dc};
      block_sum_all3(d3, S);
      inst_sum3<C>(d3, S, buf);
      // bp = <v2, w>, al = <v1, w - bp v2> in the true (normalised) vectors
      const double bp = v2 ? s2 * s1 * d3[0] : 0.0;
      const double al = s1 * (s1 * d3[1] - bp * s2 * d3[2]);
      const float c2 = v2 ? (float)(bp * s2 / s1) : 0.f, c1 = (float)al;
      // one full Gram-Schmidt pass against v_0 .. v_{k-1}
      double nacc = 0.0;  // this thread's share of the stored V[k]'s squared norm
      float tk = 1.f;     // the power of two V[k] is stored with
      {
        const int64_t q0 = lo >> 2, q1 = hi >> 2;
        double* part = (C > 1) ? S.hp[hbuf] : S.h;
        // g_j = <V_j, u>, j < k, and ||u||^2 in part[k]: u formed tile by tile into shared
        // memory (and written back for the update), a warp per basis vector within a
        // tile, eight float4 of V_j in flight per lane
        {
          const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
          for (int j = threadIdx.x; j <= k; j += blockDim.x) part[j] = 0.0;
          double uacc = 0.0;
          for (int64_t t0 = lo; t0 < hi; t0 += kWTile) {
            const int tn = (int)std::min<int64_t>(hi - t0, kWTile);
            const int nq = tn >> 2;  // t0 is a multiple of 32: float4-aligned
            __syncthreads();  // the previous tile's readers are done (and part is zeroed)
            float uf = 0.f;
            for (int i = threadIdx.x; i < nq; i += blockDim.x) {
              float4 u = reinterpret_cast<const float4*>(w + t0)[i];
              const float4 p1 = reinterpret_cast<const float4*>(v1 + t0)[i];
              if (v2) {
                const float4 p2 = reinterpret_cast<const float4*>(v2 + t0)[i];
                u.x = fmaf(-c2, p2.x, u.x);
                u.y = fmaf(-c2, p2.y, u.y);
                u.z = fmaf(-c2, p2.z, u.z);
                u.w = fmaf(-c2, p2.w, u.w);
              }
              u.x = fmaf(-c1, p1.x, u.x);
              u.y = fmaf(-c1, p1.y, u.y);
              u.z = fmaf(-c1, p1.z, u.z);
              u.w = fmaf(-c1, p1.w, u.w);
              reinterpret_cast<float4*>(S.wt)[i] = u;
              reinterpret_cast<float4*>(w + t0)[i] = u;
              uf = fmaf(u.x, u.x, uf);
              uf = fmaf(u.y, u.y, uf);
              uf = fmaf(u.z, u.z, uf);
              uf = fmaf(u.w, u.w, uf);
            }
            for (int i = (nq << 2) + threadIdx.x; i < tn; i += blockDim.x) {
              float u = w[t0 + i];
              if (v2) u = fmaf(-c2, v2[t0 + i], u);
              u = fmaf(-c1, v1[t0 + i], u);
              S.wt[i] = u;
              w[t0 + i] = u;
              uf = fmaf(u, u, uf);
            }
            uacc += (double)uf;  // at most kWTile / blockDim.x = 8 elements per thread per tile
            __syncthreads();
            const float4* ws4 = reinterpret_cast<const float4*>(S.wt);
            for (int j = warp; j < k; j += nw) {
              const float* vj = V + (int64_t)j * I.ld + t0;
              const float4* vj4 = reinterpret_cast<const float4*>(vj);
              double dacc = 0.0;
              float acc = 0.f;
              int i = lane;
              for (; i + 224 < nq; i += 256) {  // 8 float4 per lane: 128 elements in two FP32 chunks
                float4 x[8];
#pragma unroll
                for (int q = 0; q < 8; ++q) x[q] = vj4[i + 32 * q];
#pragma unroll
                for (int q = 0; q < 8; ++q) {
                  const float4 y = ws4[i + 32 * q];
                  acc = fmaf(x[q].x, y.x, acc);
                  acc = fmaf(x[q].y, y.y, acc);
                  acc = fmaf(x[q].z, y.z, acc);
                  acc = fmaf(x[q].w, y.w, acc);
                  if (q == 3 || q == 7) {
                    dacc += (double)acc;
                    acc = 0.f;
                  }
                }
              }
              int cnt = 0;
              for (; i < nq; i += 32) {
                const float4 x = vj4[i], y = ws4[i];
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
              for (int ii = (nq << 2) + lane; ii < tn; ii += 32) acc = fmaf(vj[ii], S.wt[ii], acc);
              dacc += (double)acc;
              dacc = warp_sum0(dacc);
              if (lane == 0) part[j] += dacc;  // tile by tile, in order: the same bits in every run
            }
          }
          // ||u||^2 of this CTA's rows into part[k]
          uacc = warp_sum0(uacc);
          __syncthreads();
          if (lane == 0) S.red[warp] = uacc;
          __syncthreads();
          if (threadIdx.x == 0) {
            double t = 0.0;
            for (int q = 0; q < nw; ++q) t += S.red[q];
            part[k] = t;
          }
        }
        if constexpr (C > 1) {  // the coefficients of the whole vector, the same bits in every CTA
          cg::cluster_group cl = cg::this_cluster();
          cl.sync();
          for (int j = threadIdx.x; j <= k; j += blockDim.x) {
            double t = 0.0;
            for (int r = 0; r < C; ++r) t += *cl.map_shared_rank(&S.hp[hbuf][j], r);
            S.h[j] = t;
          }
          hbuf ^= 1;
        }
        __syncthreads();
        // update coefficients of the stored vectors: u' = u - sum_j scl[j]^2 g_j V[j]
        for (int j = threadIdx.x; j < k; j += blockDim.x) S.c[j] = S.scl[j] * S.scl[j] * S.h[j];
        {
          int e2 = 0;
          const double un = sqrt(S.h[k]);
          if (un > 0.0 && std::isfinite(un)) {
            frexp(un, &e2);
            tk = ldexpf(1.f, -e2);  // tk ||u|| in [0.5, 1)
          }
        }
        __syncthreads();
        // V[k] = tk (u - sum_j c_j V[j]), and its squared norm (FP32 over at most kChunk elements)
        const float4* wm4 = reinterpret_cast<const float4*>(w);
        float4* vk4 = reinterpret_cast<float4*>(V + (int64_t)k * I.ld);
        const int64_t bs = blockDim.x;
        float nf = 0.f;
        int ncnt = 0;
        int64_t i = q0 + threadIdx.x;
        for (; i + bs < q1; i += 2 * bs) {  // two float4 of u per thread: two independent chains
          float4 x = wm4[i], u = wm4[i + bs];
#pragma unroll 4
          for (int j = 0; j < k; ++j) {
            const float c = -(float)S.c[j];
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
          x = make_float4(x.x * tk, x.y * tk, x.z * tk, x.w * tk);
          u = make_float4(u.x * tk, u.y * tk, u.z * tk, u.w * tk);
          vk4[i] = x;
          vk4[i + bs] = u;
          nf = fmaf(x.x, x.x, nf);
          nf = fmaf(x.y, x.y, nf);
          nf = fmaf(x.z, x.z, nf);
          nf = fmaf(x.w, x.w, nf);
          nf = fmaf(u.x, u.x, nf);
          nf = fmaf(u.y, u.y, nf);
          nf = fmaf(u.z, u.z, nf);
          nf = fmaf(u.w, u.w, nf);
          if (++ncnt == kChunk / 8) {
            nacc += (double)nf;
            nf = 0.f;
            ncnt = 0;
          }
        }
        nacc += (double)nf;
        nf = 0.f;
        ncnt = 0;
        for (; i < q1; i += bs) {
          float4 x = wm4[i];
#pragma unroll 4
          for (int j = 0; j < k; ++j) {
            const float c = -(float)S.c[j];
            const float4 y = reinterpret_cast<const float4*>(V + (int64_t)j * I.ld)[i];
            x.x = fmaf(c, y.x, x.x);
            x.y = fmaf(c, y.y, x.y);
            x.z = fmaf(c, y.z, x.z);
            x.w = fmaf(c, y.w, x.w);
          }
          x = make_float4(x.x * tk, x.y * tk, x.z * tk, x.w * tk);
          vk4[i] = x;
          nf = fmaf(x.x, x.x, nf);
          nf = fmaf(x.y, x.y, nf);
          nf = fmaf(x.z, x.z, nf);
          nf = fmaf(x.w, x.w, nf);
          if (++ncnt == kChunk / 4) {
            nacc += (double)nf;
            nf = 0.f;
            ncnt = 0;
          }
        }
        float* vk = V + (int64_t)k * I.ld;
        for (int64_t i = (q1 << 2) + threadIdx.x; i < hi; i += blockDim.x) {
          float wi = w[i];
          for (int j = 0; j < k; ++j) wi = fmaf(-(float)S.c[j], V[(int64_t)j * I.ld + i], wi);
          wi *= tk;
          vk[i] = wi;
          nf = fmaf(wi, wi, nf);
        }
        nacc += (double)nf;
      }
      const double nst = sqrt(inst_sum<C>(block_sum_all(nacc, S), S, buf));  // ||V[k]|| as stored
      const double nr = s1 * nst / (double)tk;                               // beta_k
      if (threadIdx.x == 0) {
        S.alpha[k] = al + s1 * s1 * S.h[k - 1];  // al + <v_{k-1}, u> in the true vectors
        S.beta[k] = nr;
        S.scl[k] = (nst > 0.0) ? 1.0 / nst : 0.0;
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
      inst_sync<C>();  // the next product reads all of V[k]
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
      for (int k = 0; k < act; ++k) acc = fmaf((float)(S.y[k] * S.scl[k]), V[(int64_t)k * I.ld + i], acc);
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
    QD_REQUIRE(hams[i]->dim >= 1, QD_ERR_INVALID, "instance %d: the sector has no state", i);
  }
  // QD_BATCH_UNIFORM=0 keeps the valued product for every instance
  const char* uenv = std::getenv("QD_BATCH_UNIFORM");
  const bool uniform_ok = !(uenv && std::strcmp(uenv, "0") == 0);
  if (uniform_ok) check_uniform(ctx, hams, ninst);
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
  std::unique_ptr<float[]> h32(new float[(size_t)std::max<int64_t>(v0_total, 1)]);
  DBuf<float> v0buf(v0_total);
  std::vector<int64_t> off_h(ninst);
  for (int i = 0; i < ninst; ++i) off_h[i] = (i == 0) ? 0 : off_h[i - 1] + (hams[i - 1]->dim + 31) / 32 * 32;
  {
    // FP64 -> FP32 on up to eight host threads, instances dealt round-robin (padding zeroed)
    const int nt = (int)std::max<int64_t>(1, std::min<int64_t>(8, v0_total >> 20));
    auto convert = [&](int t) {
      for (int i = t; i < ninst; i += nt) {
        const int64_t d = hams[i]->dim, ld = (d + 31) / 32 * 32;
        float* o = h32.get() + off_h[i];
        const double* v = v0s[i];
        for (int64_t q = 0; q < d; ++q) o[q] = (float)v[q];
        for (int64_t q = d; q < ld; ++q) o[q] = 0.f;
      }
    };
    std::vector<std::thread> pool;
    for (int t = 1; t < nt; ++t) pool.emplace_back(convert, t);
    convert(0);
    for (auto& th : pool) th.join();
  }
  QD_CUDA(cudaMemcpyAsync(v0buf.p, h32.get(), (size_t)v0_total * sizeof(float), cudaMemcpyHostToDevice,
                          ctx->stream));
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
    I.uniform = uniform_ok ? reinterpret_cast<const int*>(H->bun_d.p + H->dim + 1) : nullptr;
    I.coff = H->bun_d.p + H->dim;
    I.diag_f = H->bun_d.p;
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
