// traj.cu -- quantum-jump trajectory ensembles (the jump loop of
// programs/hubbard_diss.cpp:439-482 with lindblad_weight :520-529,
// QJ_operator :514-517 and bsearch :565-577) for diagonal jump operators
// L_j = sqrt(gamma) n_{bit_j}.
//
// Per step and trajectory, as the reference does:
//   weights w_j = <psi| n_j^dagger n_j |psi> / <psi|psi>, wtot = sum_j w_j;
//   if u1 < gamma * wtot * dt: jump into channel bsearch(cumulative w / wtot, u2),
//       psi <- n_j psi / ||n_j psi||;
//   else psi <- exp(-i H_eff dt) psi / ||.||;
//   record the observables <psi| n_a n_b |psi>.
// The reference's per-step shift +(i/2) gamma wtot I of H_eff only rescales
// the state, which is renormalised right after, so it is not applied; the
// random numbers are Philox4x32-10 keyed by (seed, trajectory, step), so the
// oracle replays every decision.
//
// GB300 form (resident kernel): one CTA per trajectory at a time, persistent
// over the ensemble.  H_eff is shared by every trajectory and small (config:
// Hubbard L=8, dim 4,900, 44,100 stored entries), so each CTA stages it in
// shared memory once -- rows in 32-row slices with their columns in gather
// order, each entry a 16-bit column with the sign of the uniform off-diagonal
// value c in its top bit (a lane's entries 2j and 2j+1 in one 32-bit word;
// when no entry carries -c the kernel's sums are plain adds), the diagonal
// (shifted by the centre mu of its range) in registers --
// together with two complex64 copies of the trajectory's vector.  A step is
// then K products H - mu of the shared-memory vector (the gathers never leave
// the SM) summed into the truncated Taylor series of exp(-i tau (H - mu)),
// S sub-steps of tau = dt / S, with (S, K) from the series' remainder bound
// (tau ||H - mu|| <= 1 and ||R_K|| <= theta^(K+1) / (K+1)! e^theta <= 1e-8,
// the scheme of A. H. Al-Mohy and N. J. Higham, SIAM J. Sci. Comput. 33
// (2011) 488-511, with one sub-step size); the factor exp(-i tau mu) is
// dropped with the renormalisation.  Weights, norm and observables come from
// one block reduction of the new vector per step; HBM sees only the observable
// records.  The state's norm is carried, not divided out: the next products
// start from psi / ||psi||.
//
// Operators the resident form does not cover (dim > 5,120, registers of more
// than 32 bits, or off-diagonal values other than +-c) run each step as a
// batched FP64 Arnoldi exponential of every trajectory (kbatch.cu, the
// reference's evolve with m vectors) followed by the decision kernel below on
// complex128 states.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <utility>
#include <vector>

#include "kbatch.cuh"
#include "krylov.cuh"
#include "philox.cuh"
#include "traj.cuh"

namespace qd {

constexpr int kTrajRpt = 8;        // 32-row slices per warp of the resident kernel
constexpr int kTrajMaxWarps = 20;  // 640 threads: up to 102 registers a thread
constexpr int kTrajMaxDimRes = kTrajRpt * kTrajMaxWarps * 32;  // 5,120 rows
constexpr int kTrajRedStride = 34;  // floats per warp row of the reduction scratch
constexpr int kTrajMaxTaylor = 32;

__host__ __device__ inline int traj_bsearch(const double* wt, int nchan, double u) {
  // bsearch of hubbard_diss.cpp:565-577 on wt[0..nchan] (wt[0] = 0, wt[nchan] = 1)
  int is = 0, ie = nchan + 1;
  while (ie - is > 1) {
    const int mid = is + (ie - is) / 2;
    if (u < wt[mid]) ie = mid;
    else is = mid;
  }
  return is < nchan ? is : nchan - 1;
}

// ---------------------------------------------------------------- resident kernel
struct TrajResArgs {
  int n, nsl, nwarps;
  int ntraj, nsteps, nchan, nobs;
  int K, S;
  float tau;          // dt / S
  float2 coff;        // the off-diagonal value c
  double gamma, dt;
  uint64_t seed;
  uint32_t chanmask;  // union of the channel bits
  int chan_bit[kTrajMaxChan];
  uint32_t obs_mask[kTrajMaxObs];
  // smem segment sizes (elements)
  int tb_len;         // per vector buffer: n + 1 rounded up to 2 (slot n is a zero)
  int ent_len;        // entries rounded up to 8
  const uint16_t* ent;   // entry k of slice row l at sdesc.x + 64 (k / 2) + 2 l + k % 2: column | sign << 15
  const uint16_t* rid;   // row of each slot (n: padding)
  const uint32_t* st;    // state bits of each slot
  const int2* sdesc;     // per slice: entry offset, width
  const float2* dg;      // per slot: diagonal - mu
  const float2* psi0;    // normalised start vector
  float* obs;            // (step * nobs + k) * ntraj + b
  unsigned long long* jumps;
};

struct TrajSmem {
  float2* tb[2];
  uint16_t* ent;
  uint16_t* rid;
  uint32_t* st;
  int2* sd;
  float* red;
  const int* chan_bit;      // shared copies of the argument arrays (indexed at run time)
  const uint32_t* obs_mask;
};

__device__ __forceinline__ float traj_warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Block sums of q_j = sum over the block's rows of |acc|^2 f_j(state), j < nq,
// into res[0 .. nq-1]; f_j chosen by `kind`: 0 the step's quantities
// (1, popcount(state & chanmask), observables), 1 the channel weights.
template <int kind>
__device__ __forceinline__ void traj_block_sums(const TrajResArgs& A, const TrajSmem& M, const float2 (&acc)[kTrajRpt],
                                                int nq, float* res) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int q = 0; q < nq; ++q) {
    float v = 0.f;
#pragma unroll
    for (int i = 0; i < kTrajRpt; ++i) {
      const int s = warp + i * A.nwarps;
      if (s < A.nsl) {
        const float p = fmaf(acc[i].x, acc[i].x, acc[i].y * acc[i].y);
        const uint32_t st = M.st[32 * s + lane];
        float f;
        if (kind == 0) {
          f = (q == 0) ? 1.f
                       : (q == 1 ? (float)__popc(st & A.chanmask)
                                 : (((st & M.obs_mask[q - 2]) == M.obs_mask[q - 2]) ? 1.f : 0.f));
        } else {
          f = (float)((st >> M.chan_bit[q]) & 1u);
        }
        v = fmaf(p, f, v);
      }
    }
    v = traj_warp_sum(v);
    if (lane == 0) M.red[warp * kTrajRedStride + q] = v;
  }
  __syncthreads();
  if (threadIdx.x < nq) {
    double t = 0.0;
    for (int w = 0; w < A.nwarps; ++w) t += M.red[w * kTrajRedStride + threadIdx.x];
    res[threadIdx.x] = (float)t;
  }
  __syncthreads();
}

template <bool kSigned>
__global__ void __launch_bounds__(kTrajMaxWarps * 32, 1) traj_resident_kernel(TrajResArgs A) {
  extern __shared__ __align__(16) unsigned char traj_smem[];
  __shared__ float res[2 + kTrajMaxObs];
  __shared__ float resc[kTrajMaxChan];
  __shared__ int s_jump;
  __shared__ double s_u2;
  __shared__ int s_chan_bit[kTrajMaxChan];
  __shared__ uint32_t s_obs_mask[kTrajMaxObs];
  TrajSmem M;
  M.tb[0] = reinterpret_cast<float2*>(traj_smem);
  M.tb[1] = M.tb[0] + A.tb_len;
  M.ent = reinterpret_cast<uint16_t*>(M.tb[1] + A.tb_len);
  M.rid = M.ent + A.ent_len;
  M.st = reinterpret_cast<uint32_t*>(M.rid + 32 * A.nsl);
  M.sd = reinterpret_cast<int2*>(M.st + 32 * A.nsl);
  M.red = reinterpret_cast<float*>(M.sd + A.nsl + (A.nsl & 1));
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  // stage the operator (once per CTA)
  {
    const uint4* src = reinterpret_cast<const uint4*>(A.ent);
    uint4* dst = reinterpret_cast<uint4*>(M.ent);
    for (int i = tid; i < A.ent_len / 8; i += blockDim.x) dst[i] = src[i];
    for (int i = tid; i < 32 * A.nsl; i += blockDim.x) {
      M.rid[i] = A.rid[i];
      M.st[i] = A.st[i];
    }
    for (int i = tid; i < A.nsl; i += blockDim.x) M.sd[i] = A.sdesc[i];
    if (tid == 0) {
      M.tb[0][A.n] = make_float2(0.f, 0.f);
      M.tb[1][A.n] = make_float2(0.f, 0.f);
#pragma unroll
      for (int j = 0; j < kTrajMaxChan; ++j) s_chan_bit[j] = A.chan_bit[j];
#pragma unroll
      for (int k = 0; k < kTrajMaxObs; ++k) s_obs_mask[k] = A.obs_mask[k];
    }
  }
  M.chan_bit = s_chan_bit;
  M.obs_mask = s_obs_mask;
  float2 dg[kTrajRpt];
#pragma unroll
  for (int i = 0; i < kTrajRpt; ++i) {
    const int s = warp + i * A.nwarps;
    dg[i] = (s < A.nsl) ? A.dg[32 * s + lane] : make_float2(0.f, 0.f);
  }
  __syncthreads();
  const int nq = 2 + A.nobs;
  unsigned long long njumps = 0;

  for (int b = blockIdx.x; b < A.ntraj; b += gridDim.x) {
    float2 acc[kTrajRpt];
    int cb = 0;
#pragma unroll
    for (int i = 0; i < kTrajRpt; ++i) {
      const int s = warp + i * A.nwarps;
      acc[i] = make_float2(0.f, 0.f);
      if (s < A.nsl) {
        const int r = M.rid[32 * s + lane];
        if (r < A.n) {
          acc[i] = A.psi0[r];
          M.tb[0][r] = acc[i];
        }
      }
    }
    traj_block_sums<0>(A, M, acc, nq, res);
    if (tid < A.nobs) A.obs[(size_t)tid * A.ntraj + b] = res[2 + tid] / res[0];

    for (int step = 1; step <= A.nsteps; ++step) {
      if (tid == 0) {
        double u1, u2;
        philox_uniform2(A.seed, (uint32_t)b, (uint32_t)step, u1, u2);
        const double wtot = (double)res[1] / (double)res[0];
        s_jump = (wtot > 0.0 && u1 < A.gamma * wtot * A.dt) ? 1 : 0;
        s_u2 = u2;
      }
      __syncthreads();
      if (s_jump) {
        // channel weights of the current state, then psi <- n_j psi (norm carried)
        traj_block_sums<1>(A, M, acc, A.nchan, resc);
        if (tid == 0) {
          // bsearch on the cumulative weights normalised by their total: the channel j
          // with wt[j] <= u2 < wt[j+1] (a scan gives the same index on a monotone table)
          double tot = 0.0;
          for (int j = 0; j < A.nchan; ++j) tot += (double)resc[j];
          double cum = 0.0;
          int ch = 0;
          for (int j = 1; j < A.nchan; ++j) {
            cum += (double)resc[j - 1];
            if (cum / tot <= s_u2) ch = j;
          }
          s_jump = 1 + ch;
          ++njumps;
        }
        __syncthreads();
        const int bit = s_chan_bit[s_jump - 1];
#pragma unroll
        for (int i = 0; i < kTrajRpt; ++i) {
          const int s = warp + i * A.nwarps;
          if (s < A.nsl) {
            const int slot = 32 * s + lane;
            const int r = M.rid[slot];
            if (r < A.n) {
              if (!((M.st[slot] >> bit) & 1u)) acc[i] = make_float2(0.f, 0.f);
              M.tb[cb][r] = acc[i];
            }
          }
        }
      } else {
        // psi <- exp(-i dt (H - mu)) psi / ||psi||: S sub-steps of K Taylor terms
        const float sc = rsqrtf(res[0]);
        for (int sub = 0; sub < A.S; ++sub) {
          if (sub == 0) {
#pragma unroll
            for (int i = 0; i < kTrajRpt; ++i) acc[i] = make_float2(acc[i].x * sc, acc[i].y * sc);
          }
          int rb = cb;
          for (int k = 1; k <= A.K; ++k) {
            // t_k = (-i tau / k) (H - mu) t_{k-1}; t_0 = the vector in tb[cb] (times sc on the first sub-step)
            const float f = A.tau / (float)k * ((sub == 0 && k == 1) ? sc : 1.f);
            const float2* __restrict__ src = M.tb[rb];
            float2* __restrict__ dst = M.tb[rb ^ 1];
            // Two slices at a time (i and i + 1): their entry loads and gathers interleave, so a
            // lane has four independent gathers in flight; each row keeps its own sums in entry
            // order (even entries in s, odd ones in u).
            auto gather = [&](uint32_t pr, float& sx, float& sy, float& ux, float& uy) {
              const uint32_t ev = pr & 0xffffu, fv = pr >> 16;
              if (kSigned) {
                const float2 x = src[ev & 0x7fffu], y = src[fv & 0x7fffu];
                const float sg = __uint_as_float(0x3f800000u | ((ev & 0x8000u) << 16));
                const float tg = __uint_as_float(0x3f800000u | ((fv & 0x8000u) << 16));
                sx = fmaf(sg, x.x, sx);
                sy = fmaf(sg, x.y, sy);
                ux = fmaf(tg, y.x, ux);
                uy = fmaf(tg, y.y, uy);
              } else {  // every entry carries +c: plain sums
                const float2 x = src[ev], y = src[fv];
                sx += x.x;
                sy += x.y;
                ux += y.x;
                uy += y.y;
              }
            };
            auto finish = [&](int i, int r, float sx, float sy) {
              if (r < A.n) {
                const float2 o = src[r];
                // v = c * sum + dg * own
                const float vx = fmaf(A.coff.x, sx, fmaf(-A.coff.y, sy, fmaf(dg[i].x, o.x, -dg[i].y * o.y)));
                const float vy = fmaf(A.coff.x, sy, fmaf(A.coff.y, sx, fmaf(dg[i].x, o.y, dg[i].y * o.x)));
                // t = (-i f) v = (f vy, -f vx)
                const float2 t = make_float2(f * vy, -f * vx);
                dst[r] = t;
                acc[i].x += t.x;
                acc[i].y += t.y;
              }
            };
#pragma unroll
            for (int i = 0; i < kTrajRpt; i += 2) {
              const int s0 = warp + i * A.nwarps, s1 = s0 + A.nwarps;
              if (s0 < A.nsl) {
                const bool has1 = s1 < A.nsl;
                const int2 d0 = M.sd[s0];
                const int2 d1 = has1 ? M.sd[s1] : make_int2(0, 0);
                const int r0 = M.rid[32 * s0 + lane];
                const int r1 = has1 ? (int)M.rid[32 * s1 + lane] : A.n;
                // a lane's entries 2j and 2j+1 share one 32-bit word (widths are even)
                const uint32_t* e0 = reinterpret_cast<const uint32_t*>(M.ent + d0.x) + lane;
                const uint32_t* e1 = reinterpret_cast<const uint32_t*>(M.ent + d1.x) + lane;
                const int w0 = d0.y >> 1, w1 = d1.y >> 1;
                float sx0 = 0.f, sy0 = 0.f, ux0 = 0.f, uy0 = 0.f;
                float sx1 = 0.f, sy1 = 0.f, ux1 = 0.f, uy1 = 0.f;
                const int wm = min(w0, w1);
                int q = 0;
                for (; q < wm; ++q) {
                  const uint32_t p0 = e0[32 * q], p1 = e1[32 * q];
                  gather(p0, sx0, sy0, ux0, uy0);
                  gather(p1, sx1, sy1, ux1, uy1);
                }
                for (int q0 = q; q0 < w0; ++q0) gather(e0[32 * q0], sx0, sy0, ux0, uy0);
                for (int q1 = q; q1 < w1; ++q1) gather(e1[32 * q1], sx1, sy1, ux1, uy1);
                finish(i, r0, sx0 + ux0, sy0 + uy0);
                if (has1) finish(i + 1, r1, sx1 + ux1, sy1 + uy1);
              }
            }
            __syncthreads();
            rb ^= 1;
          }
          // the sub-step's result into the buffer that held t_{K-1} (its readers are done)
          cb = rb ^ 1;
#pragma unroll
          for (int i = 0; i < kTrajRpt; ++i) {
            const int s = warp + i * A.nwarps;
            if (s < A.nsl) {
              const int r = M.rid[32 * s + lane];
              if (r < A.n) M.tb[cb][r] = acc[i];
            }
          }
          __syncthreads();
        }
      }
      traj_block_sums<0>(A, M, acc, nq, res);
      if (tid < A.nobs) A.obs[((size_t)step * A.nobs + tid) * A.ntraj + b] = res[2 + tid] / res[0];
    }
  }
  if (tid == 0 && njumps) atomicAdd(A.jumps, njumps);
}

// The resident form of H_eff built on the host (32-row slices as wide as their
// longest row).  Returns false when the operator is outside the form.
struct TrajHostForm {
  int n = 0, nsl = 0, nwarps = 0, ent_len = 0;
  std::vector<uint16_t> ent, rid;
  std::vector<uint32_t> st;
  std::vector<int2> sdesc;
  std::vector<float2> dg;
  cplx coff{0.0, 0.0};
  double norm = 0.0;  // bound on ||H - mu||_2: max of the 1- and infinity-norms
  bool any_neg = false;  // some entry carries -c
};

// Dynamic shared memory of the resident kernel for dim n, nsl slices and ent_len entries.
static size_t traj_smem_bytes(int n, int nsl, int ent_len) {
  const size_t tb_len = (size_t)(n + 2) / 2 * 2;
  return 2 * tb_len * sizeof(float2) + (size_t)ent_len * 2 + (size_t)32 * nsl * 2 + (size_t)32 * nsl * 4 +
         (size_t)(nsl + (nsl & 1)) * sizeof(int2) + (size_t)kTrajMaxWarps * kTrajRedStride * sizeof(float);
}

static bool traj_build_resident(qd_ham* H, TrajHostForm& F, size_t max_smem) {
  const int64_t n = H->dim;
  if (n < 1 || n > kTrajMaxDimRes || H->sec->nbits > 32) return false;
  std::vector<int64_t> rp(n + 1);
  std::vector<int32_t> ci(H->nnz);
  std::vector<cplx> v(H->nnz);
  std::vector<uint64_t> basis(n);
  Ctx* ctx = H->ctx;
  QD_CUDA(cudaMemcpyAsync(rp.data(), H->rowptr.p, (n + 1) * sizeof(int64_t), cudaMemcpyDeviceToHost, ctx->stream));
  if (H->nnz) {
    QD_CUDA(cudaMemcpyAsync(ci.data(), H->colidx.p, H->nnz * sizeof(int32_t), cudaMemcpyDeviceToHost, ctx->stream));
    QD_CUDA(cudaMemcpyAsync(v.data(), H->vals_c.p, H->nnz * sizeof(cplx), cudaMemcpyDeviceToHost, ctx->stream));
  }
  QD_CUDA(cudaMemcpyAsync(basis.data(), H->sec->basis.p, n * sizeof(uint64_t), cudaMemcpyDeviceToHost, ctx->stream));
  QD_CUDA(cudaStreamSynchronize(ctx->stream));
  // the uniform off-diagonal value c (entries equal to c or -c; explicit zeros skipped)
  bool have_c = false;
  cplx c{0.0, 0.0};
  std::vector<cplx> d(n, cplx{0.0, 0.0});
  std::vector<int> cnt(n, 0);
  for (int64_t r = 0; r < n; ++r) {
    for (int64_t k = rp[r]; k < rp[r + 1]; ++k) {
      const cplx a = v[k];
      if (ci[k] == r) {
        d[r] = a;
        continue;
      }
      if (a.re == 0.0 && a.im == 0.0) continue;
      if (!have_c) {
        c = a;
        have_c = true;
      }
      const bool pos = (a.re == c.re && a.im == c.im), neg = (a.re == -c.re && a.im == -c.im);
      if (!pos && !neg) return false;
      ++cnt[r];
    }
  }
  // 32-row slices of the rows in their own order, each row's columns in gather order (by the
  // highest bit in which the column's state differs from the row's, highest first): rows of one
  // block of the high bits share their high-bit transitions, so lane l's k-th gather and lane
  // l+1's hit neighbouring words (no bank conflict), and a row's own value sits at its lane.
  // Where that layout's padding leaves no room, rows sorted by their entry count instead.
  F.nsl = (int)((n + 31) / 32);
  std::vector<int> order(n);
  for (int64_t r = 0; r < n; ++r) order[r] = (int)r;
  {
    int64_t slots = 0;
    for (int s = 0; s < F.nsl; ++s) {
      int w = 0;
      for (int l = 0; l < 32 && 32 * s + l < n; ++l) w = std::max(w, cnt[32 * s + l]);
      slots += 32 * ((w + 1) & ~1);
    }
    if (traj_smem_bytes((int)n, F.nsl, (int)((slots + 7) / 8 * 8)) > max_smem)
      std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return cnt[a] > cnt[b]; });
  }
  F.n = (int)n;
  F.nwarps = (F.nsl + kTrajRpt - 1) / kTrajRpt;
  F.rid.assign((size_t)32 * F.nsl, (uint16_t)n);
  F.st.assign((size_t)32 * F.nsl, 0u);
  F.dg.assign((size_t)32 * F.nsl, make_float2(0.f, 0.f));
  F.sdesc.resize(F.nsl);
  // centre of the diagonal's range
  double rmin = 1e300, rmax = -1e300, imin = 1e300, imax = -1e300;
  for (int64_t r = 0; r < n; ++r) {
    rmin = std::min(rmin, d[r].re);
    rmax = std::max(rmax, d[r].re);
    imin = std::min(imin, d[r].im);
    imax = std::max(imax, d[r].im);
  }
  const cplx mu{0.5 * (rmin + rmax), 0.5 * (imin + imax)};
  int off = 0;
  for (int s = 0; s < F.nsl; ++s) {
    int w = 0;
    for (int l = 0; l < 32 && 32 * s + l < n; ++l) w = std::max(w, cnt[order[32 * s + l]]);
    w = (w + 1) & ~1;  // entries in pairs per lane
    F.sdesc[s] = make_int2(off, w);
    off += 32 * w;
  }
  F.ent_len = (off + 7) / 8 * 8;
  F.ent.assign((size_t)std::max(F.ent_len, 8), (uint16_t)n);  // padding entries read the zero slot n
  const double cabs = std::hypot(c.re, c.im);
  std::vector<double> colsum(n, 0.0);
  double rowmax = 0.0;
  for (int s = 0; s < F.nsl; ++s) {
    for (int l = 0; l < 32; ++l) {
      const int slot = 32 * s + l;
      if (slot >= n) break;
      const int r = order[slot];
      F.rid[slot] = (uint16_t)r;
      F.st[slot] = (uint32_t)basis[r];
      const double dre = d[r].re - mu.re, dim_ = d[r].im - mu.im;
      F.dg[slot] = make_float2((float)dre, (float)dim_);
      std::vector<std::pair<int, uint16_t>> row;  // (gather key, entry)
      for (int64_t k = rp[r]; k < rp[r + 1]; ++k) {
        const cplx a = v[k];
        if (ci[k] == r || (a.re == 0.0 && a.im == 0.0)) continue;
        const bool neg = !(a.re == c.re && a.im == c.im);
        const uint64_t dif = basis[r] ^ basis[ci[k]];
        const int key = dif ? 63 - __builtin_clzll(dif) : -1;
        row.emplace_back(key, (uint16_t)(ci[k] | (neg ? 0x8000 : 0)));
        colsum[ci[k]] += cabs;
      }
      std::stable_sort(row.begin(), row.end(),
                       [](const std::pair<int, uint16_t>& x, const std::pair<int, uint16_t>& y) {
                         return x.first > y.first;
                       });
      for (size_t q = 0; q < row.size(); ++q)
        F.ent[F.sdesc[s].x + 64 * (q >> 1) + 2 * l + (q & 1)] = row[q].second;
      for (const auto& e : row) F.any_neg |= (e.second & 0x8000) != 0;
      const double dd = std::hypot(dre, dim_);
      rowmax = std::max(rowmax, dd + cnt[r] * cabs);
      colsum[r] += dd;
    }
  }
  double colmax = 0.0;
  for (double x : colsum) colmax = std::max(colmax, x);
  F.coff = c;
  F.norm = std::max(rowmax, colmax);
  return true;
}

// Truncation tolerance of the Taylor series per step: a sixth of the complex64
// state's own rounding per step (about 6e-8 in 2-norm against the exact
// exponential), so the series adds no error the FP32 state would not.
constexpr double kTrajTaylorTol = 1e-8;

// (S, K) for exp(-i dt A) with ||A|| <= norm: S sub-steps of tau = dt / S with
// theta = tau norm <= 1, K the least degree with theta^(K+1)/(K+1)! e^theta <= kTrajTaylorTol.
static void traj_taylor_plan(double dt, double norm, int kmax, int* S, int* K) {
  int s = std::max(1, (int)std::ceil(dt * norm));
  for (;; ++s) {
    const double th = dt * norm / s;
    double term = th;  // th^(k+1)/(k+1)! at k = 0
    int k = 0;
    while (term * std::exp(th) > kTrajTaylorTol && k < kTrajMaxTaylor) {
      ++k;
      term *= th / (k + 1);
    }
    if (k <= kmax) {
      *S = s;
      *K = std::max(k, 1);
      return;
    }
  }
}

// ---------------------------------------------------------------- fallback: FP64 Arnoldi steps
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
  cplx* psi;             // current states (n x ntraj), overwritten with the next ones
  const cplx* psi_new;   // exp(-i H_eff dt) psi / ||psi|| (kbatch)
  double* w;             // per trajectory: nchan weights + norm^2 (stride kTrajMaxChan + 1)
  float* obs;            // (step * nobs + k) * ntraj + b, normalised observables
  int* jumps;            // per trajectory jump count
  const int* chan_bits;
  const uint64_t* obs_mask;  // observable k: state contributes when (s & mask_k) == mask_k
};

constexpr int kTrajThreads = 256;

__global__ void __launch_bounds__(kTrajThreads) traj_step_kernel(TrajArgs A) {
  __shared__ double s_red[kTrajThreads / 32][kTrajMaxChan + 1 + kTrajMaxObs];
  __shared__ int s_jump;  // -2: initial state, -1: evolve, else channel
  const int b = blockIdx.x;
  if (b >= A.ntraj) return;
  double* wb = A.w + (size_t)b * (kTrajMaxChan + 1);
  if (threadIdx.x == 0) {
    int jump = -2;
    if (A.step > 0) {
      // decision from the current state's weights (unnormalised, norm^2 in wb[kTrajMaxChan])
      double wt[kTrajMaxChan + 1];
      wt[0] = 0.0;
      for (int j = 0; j < A.nchan; ++j) wt[j + 1] = wt[j] + wb[j];
      const double wtot = wt[A.nchan] / wb[kTrajMaxChan];
      for (int j = 0; j <= A.nchan; ++j) wt[j] /= wt[A.nchan];
      double u1, u2;
      philox_uniform2(A.seed, (uint32_t)b, (uint32_t)A.step, u1, u2);
      jump = -1;
      if (wtot > 0.0 && u1 < A.gamma * wtot * A.dt) {
        jump = traj_bsearch(wt, A.nchan, u2);
        A.jumps[b] += 1;
      }
    }
    s_jump = jump;
  }
  __syncthreads();
  const int jump = s_jump;
  const uint64_t jmask = (jump >= 0) ? (1ull << A.chan_bits[jump]) : 0ull;
  double acc[kTrajMaxChan + 1 + kTrajMaxObs];
#pragma unroll
  for (int q = 0; q < kTrajMaxChan + 1 + kTrajMaxObs; ++q) acc[q] = 0.0;
  cplx* col = A.psi + (size_t)b * A.ld;
  const cplx* ncol = A.psi_new + (size_t)b * A.ld;
  for (int64_t s = threadIdx.x; s < A.n; s += blockDim.x) {
    const uint64_t st = A.basis[s];
    cplx x;
    if (jump == -2) x = col[s];
    else if (jump >= 0) x = (st & jmask) ? col[s] : mkc(0.0, 0.0);
    else x = ncol[s];
    if (jump != -2) col[s] = x;
    const double p = x.re * x.re + x.im * x.im;
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
    double v = acc[q];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) s_red[warp][q] = v;
  }
  __syncthreads();
  if (threadIdx.x < kTrajMaxChan + 1 + kTrajMaxObs) {
    const int q = threadIdx.x;
    double t = 0.0;
    for (int w = 0; w < kTrajThreads / 32; ++w) t += s_red[w][q];
    s_red[0][q] = t;
  }
  __syncthreads();
  if (threadIdx.x <= kTrajMaxChan) wb[threadIdx.x] = s_red[0][threadIdx.x];
  if (threadIdx.x < A.nobs) {
    const double nrm2 = s_red[0][kTrajMaxChan];
    A.obs[((size_t)A.step * A.nobs + threadIdx.x) * A.ntraj + b] =
        (float)(s_red[0][kTrajMaxChan + 1 + threadIdx.x] / nrm2);
  }
}

__global__ void init_states_kernel(cplx* psi, int64_t n, int64_t ld, int ntraj, const cplx* psi0, double inv) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int b = blockIdx.y;
  if (i >= n || b >= ntraj) return;
  const cplx v = psi0[i];
  psi[(size_t)b * ld + i] = mkc(v.re * inv, v.im * inv);
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

static bool traj_force_fallback() {
  const char* e = std::getenv("QD_TRAJ_ARNOLDI");
  return e && std::strcmp(e, "1") == 0;
}

void traj_run(qd_ham* H, const qd_traj_desc& d, const double* psi0_host, double* obs_mean, double* obs_stderr,
              int64_t* jumps_total, double* timings, int* path) {
  Ctx* ctx = H->ctx;
  const int64_t n = H->dim;
  QD_REQUIRE(d.ntraj >= 1 && d.nsteps >= 0, QD_ERR_INVALID, "ntraj >= 1 and nsteps >= 0 required");
  QD_REQUIRE(d.nchan >= 1 && d.nchan <= kTrajMaxChan, QD_ERR_UNSUPPORTED, "1..%d jump channels", kTrajMaxChan);
  QD_REQUIRE(d.nobs >= 0 && d.nobs <= kTrajMaxObs, QD_ERR_UNSUPPORTED, "at most %d observables", kTrajMaxObs);
  QD_REQUIRE(d.dt > 0.0 && d.gamma >= 0.0, QD_ERR_INVALID, "dt > 0 and gamma >= 0 required");
  QD_REQUIRE(d.m >= 2 && d.m <= 32, QD_ERR_UNSUPPORTED, "Krylov dimension m must be in 2..32");
  QD_REQUIRE(n >= 1 && n <= (int64_t)INT32_MAX, QD_ERR_UNSUPPORTED, "dimension out of range");
  for (int j = 0; j < d.nchan; ++j)
    QD_REQUIRE(d.chan_bits[j] >= 0 && d.chan_bits[j] < H->sec->nbits, QD_ERR_INVALID, "channel %d: bad bit", j);
  std::vector<uint64_t> masks(kTrajMaxObs, 0ull);
  for (int k = 0; k < d.nobs; ++k) {
    QD_REQUIRE(d.obs_a[k] >= 0 && d.obs_a[k] < H->sec->nbits && d.obs_b[k] >= 0 && d.obs_b[k] < H->sec->nbits,
               QD_ERR_INVALID, "observable %d: bad bit", k);
    masks[k] = (1ull << d.obs_a[k]) | (1ull << d.obs_b[k]);
  }
  double n0 = 0.0;
  for (int64_t i = 0; i < n; ++i) n0 += psi0_host[2 * i] * psi0_host[2 * i] + psi0_host[2 * i + 1] * psi0_host[2 * i + 1];
  QD_REQUIRE(n0 > 0.0, QD_ERR_INVALID, "initial state is zero");
  const double inv0 = 1.0 / std::sqrt(n0);

  cudaEvent_t e0, e1, e2;
  QD_CUDA(cudaEventCreate(&e0));
  QD_CUDA(cudaEventCreate(&e1));
  QD_CUDA(cudaEventCreate(&e2));
  struct EvGuard {
    cudaEvent_t a, b, c;
    ~EvGuard() {
      cudaEventDestroy(a);
      cudaEventDestroy(b);
      cudaEventDestroy(c);
    }
  } evg{e0, e1, e2};
  QD_CUDA(cudaEventRecord(e0, ctx->stream));
  const int nrows = (d.nsteps + 1) * d.nobs;
  DBuf<float> obs((size_t)std::max(nrows, 1) * d.ntraj);
  DBuf<unsigned long long> jumps_dev(1);
  QD_CUDA(cudaMemsetAsync(jumps_dev.p, 0, sizeof(unsigned long long), ctx->stream));
  int64_t tot = 0;

  TrajHostForm F;
  int maxsm = 0;
  QD_CUDA(cudaDeviceGetAttribute(&maxsm, cudaDevAttrMaxSharedMemoryPerBlockOptin, ctx->device));
  const size_t smem_cap = (size_t)std::max(maxsm - 1024, 0);
  const bool resident = !traj_force_fallback() && traj_build_resident(H, F, smem_cap);
  if (path) {
    path[0] = resident ? 0 : 1;
    path[1] = d.m - 1;
  }
  if (resident) {
    TrajResArgs A;
    std::memset(&A, 0, sizeof(A));
    A.n = F.n;
    A.nsl = F.nsl;
    A.nwarps = F.nwarps;
    A.ntraj = d.ntraj;
    A.nsteps = d.nsteps;
    A.nchan = d.nchan;
    A.nobs = d.nobs;
    traj_taylor_plan(d.dt, F.norm, d.m - 1, &A.S, &A.K);
    if (path) path[1] = A.K * A.S;
    A.tau = (float)(d.dt / A.S);
    A.coff = make_float2((float)F.coff.re, (float)F.coff.im);
    A.gamma = d.gamma;
    A.dt = d.dt;
    A.seed = d.seed;
    for (int j = 0; j < d.nchan; ++j) {
      A.chan_bit[j] = d.chan_bits[j];
      A.chanmask |= 1u << d.chan_bits[j];
    }
    for (int k = 0; k < d.nobs; ++k) A.obs_mask[k] = (uint32_t)masks[k];
    A.tb_len = (F.n + 2) / 2 * 2;
    A.ent_len = F.ent_len;
    DBuf<uint16_t> ent(F.ent.size()), rid(F.rid.size());
    DBuf<uint32_t> st(F.st.size());
    DBuf<int2> sdesc(F.sdesc.size());
    DBuf<float2> dg(F.dg.size()), p0(F.n);
    std::vector<float2> hp0(F.n);
    for (int64_t i = 0; i < n; ++i)
      hp0[i] = make_float2((float)(psi0_host[2 * i] * inv0), (float)(psi0_host[2 * i + 1] * inv0));
    QD_CUDA(cudaMemcpyAsync(ent.p, F.ent.data(), F.ent.size() * 2, cudaMemcpyHostToDevice, ctx->stream));
    QD_CUDA(cudaMemcpyAsync(rid.p, F.rid.data(), F.rid.size() * 2, cudaMemcpyHostToDevice, ctx->stream));
    QD_CUDA(cudaMemcpyAsync(st.p, F.st.data(), F.st.size() * 4, cudaMemcpyHostToDevice, ctx->stream));
    QD_CUDA(cudaMemcpyAsync(sdesc.p, F.sdesc.data(), F.sdesc.size() * sizeof(int2), cudaMemcpyHostToDevice,
                            ctx->stream));
    QD_CUDA(cudaMemcpyAsync(dg.p, F.dg.data(), F.dg.size() * sizeof(float2), cudaMemcpyHostToDevice, ctx->stream));
    QD_CUDA(cudaMemcpyAsync(p0.p, hp0.data(), F.n * sizeof(float2), cudaMemcpyHostToDevice, ctx->stream));
    A.ent = ent.p;
    A.rid = rid.p;
    A.st = st.p;
    A.sdesc = sdesc.p;
    A.dg = dg.p;
    A.psi0 = p0.p;
    A.obs = obs.p;
    A.jumps = jumps_dev.p;
    const size_t smem = traj_smem_bytes(F.n, F.nsl, A.ent_len);
    if (smem <= smem_cap) {
      auto kern = F.any_neg ? traj_resident_kernel<true> : traj_resident_kernel<false>;
      QD_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
      const int threads = 32 * F.nwarps;
      int occ = 0;
      QD_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, threads, smem));
      QD_REQUIRE(occ >= 1, QD_ERR_UNSUPPORTED, "trajectory kernel does not fit an SM");
      const int grid = (int)std::min<int64_t>(d.ntraj, (int64_t)occ * ctx->num_sms);
      QD_CUDA(cudaEventRecord(e1, ctx->stream));
      kern<<<grid, threads, smem, ctx->stream>>>(A);
      QD_CHECK_LAUNCH();
      QD_LAUNCHED(ctx);
      unsigned long long j = 0;
      QD_CUDA(cudaMemcpyAsync(&j, jumps_dev.p, sizeof(j), cudaMemcpyDeviceToHost, ctx->stream));
      QD_CUDA(cudaStreamSynchronize(ctx->stream));
      tot = (int64_t)j;
    } else {
      F.n = 0;  // too large for one SM's shared memory: the Arnoldi steps below
    }
    if (F.n == 0 && path) {
      path[0] = 1;
      path[1] = d.m - 1;
    }
  }
  if (!resident || F.n == 0) {
    QD_CUDA(cudaEventRecord(e1, ctx->stream));
    const int64_t ld = (n + 31) / 32 * 32;
    DBuf<cplx> psi((size_t)ld * d.ntraj), psi_new((size_t)ld * d.ntraj);
    QD_CUDA(cudaMemsetAsync(psi.p, 0, psi.bytes(), ctx->stream));
    QD_CUDA(cudaMemsetAsync(psi_new.p, 0, psi_new.bytes(), ctx->stream));
    DBuf<cplx> p0(n);
    QD_CUDA(cudaMemcpyAsync(p0.p, psi0_host, n * sizeof(cplx), cudaMemcpyHostToDevice, ctx->stream));
    init_states_kernel<<<dim3((unsigned)ceil_div(n, 256), d.ntraj), 256, 0, ctx->stream>>>(psi.p, n, ld, d.ntraj,
                                                                                       p0.p, inv0);
    QD_CHECK_LAUNCH();
    QD_LAUNCHED(ctx);
    DBuf<double> w((size_t)d.ntraj * (kTrajMaxChan + 1));
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
    A.step = 0;
    traj_step_kernel<<<d.ntraj, kTrajThreads, 0, ctx->stream>>>(A);
    QD_CHECK_LAUNCH();
    QD_LAUNCHED(ctx);
    for (int step = 1; step <= d.nsteps; ++step) {
      krylov_batch(H, psi.p, ld, d.ntraj, d.dt, d.m, psi_new.p, nullptr, ld, nullptr);
      A.step = step;
      traj_step_kernel<<<d.ntraj, kTrajThreads, 0, ctx->stream>>>(A);
      QD_CHECK_LAUNCH();
      QD_LAUNCHED(ctx);
    }
    std::vector<int> hj(d.ntraj);
    QD_CUDA(cudaMemcpyAsync(hj.data(), jumps.p, d.ntraj * sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    QD_CUDA(cudaStreamSynchronize(ctx->stream));
    for (int v : hj) tot += v;
  }
  if (nrows > 0) {
    DBuf<double> dm(nrows), ds(nrows);
    traj_reduce_kernel<<<(unsigned)ceil_div(nrows, 128), 128, 0, ctx->stream>>>(obs.p, d.ntraj, nrows, dm.p, ds.p);
    QD_CHECK_LAUNCH();
    QD_LAUNCHED(ctx);
    QD_CUDA(cudaMemcpyAsync(obs_mean, dm.p, nrows * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    if (obs_stderr)
      QD_CUDA(cudaMemcpyAsync(obs_stderr, ds.p, nrows * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  }
  QD_CUDA(cudaEventRecord(e2, ctx->stream));
  QD_CUDA(cudaStreamSynchronize(ctx->stream));
  if (jumps_total) *jumps_total = tot;
  if (timings) {
    float a = 0.f, b2 = 0.f;
    cudaEventElapsedTime(&a, e0, e1);
    cudaEventElapsedTime(&b2, e1, e2);
    timings[0] = a;
    timings[1] = b2;
  }
}

}  // namespace qd
