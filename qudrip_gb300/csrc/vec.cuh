// vec.cuh -- value-type traits and deterministic grid reductions.
//
// Real Hamiltonians with real vectors run in `double`; everything else in
// `cplx` (complex128).  Reductions are deterministic: every thread sums its
// grid-stride slice in index order, blocks combine by a fixed shuffle tree,
// and the last block to finish adds the block partials in a fixed order.
#pragma once

#include "common.cuh"

namespace qd {

// ---------------------------------------------------------------- scalar traits
__device__ __forceinline__ double vzero(double) { return 0.0; }
__device__ __forceinline__ cplx vzero(cplx) { return mkc(0.0, 0.0); }

// acc + a * x
__device__ __forceinline__ double vfma(double a, double x, double acc) { return fma(a, x, acc); }
__device__ __forceinline__ cplx vfma(double a, cplx x, cplx acc) {
  return mkc(fma(a, x.re, acc.re), fma(a, x.im, acc.im));
}
__device__ __forceinline__ cplx vfma(cplx a, cplx x, cplx acc) {
  return mkc(fma(-a.im, x.im, fma(a.re, x.re, acc.re)), fma(a.im, x.re, fma(a.re, x.im, acc.im)));
}
__device__ __forceinline__ cplx vfma(cplx a, double x, cplx acc) {
  return mkc(fma(a.re, x, acc.re), fma(a.im, x, acc.im));
}

// acc + conj(a) * b
__device__ __forceinline__ double vdotfma(double a, double b, double acc) { return fma(a, b, acc); }
__device__ __forceinline__ cplx vdotfma(cplx a, cplx b, cplx acc) {
  return mkc(fma(a.im, b.im, fma(a.re, b.re, acc.re)), fma(-a.im, b.re, fma(a.re, b.im, acc.im)));
}

__device__ __forceinline__ double vadd(double a, double b) { return a + b; }
__device__ __forceinline__ cplx vadd(cplx a, cplx b) { return mkc(a.re + b.re, a.im + b.im); }
__device__ __forceinline__ double vscale(double s, double x) { return s * x; }
__device__ __forceinline__ cplx vscale(double s, cplx x) { return mkc(s * x.re, s * x.im); }
__device__ __forceinline__ double vnorm2(double x) { return x * x; }
__device__ __forceinline__ double vnorm2(cplx x) { return fma(x.re, x.re, x.im * x.im); }
// x - a * y
__device__ __forceinline__ double vsubmul(double x, double a, double y) { return fma(-a, y, x); }
__device__ __forceinline__ cplx vsubmul(cplx x, cplx a, cplx y) {
  return mkc(fma(a.im, y.im, fma(-a.re, y.re, x.re)), fma(-a.im, y.re, fma(-a.re, y.im, x.im)));
}

__device__ __forceinline__ double shfl_xor(double v, int o) { return __shfl_xor_sync(0xffffffffu, v, o); }
__device__ __forceinline__ double shfl_down(double v, int o) { return __shfl_down_sync(0xffffffffu, v, o); }
__device__ __forceinline__ cplx shfl_down(cplx v, int o) {
  return mkc(__shfl_down_sync(0xffffffffu, v.re, o), __shfl_down_sync(0xffffffffu, v.im, o));
}
__device__ __forceinline__ cplx shfl_xor(cplx v, int o) {
  return mkc(__shfl_xor_sync(0xffffffffu, v.re, o), __shfl_xor_sync(0xffffffffu, v.im, o));
}

__device__ __forceinline__ double ld_cg(const double* p) { return __ldcg(p); }
__device__ __forceinline__ cplx ld_cg(const cplx* p) {
  const double2 d = __ldcg(reinterpret_cast<const double2*>(p));
  return mkc(d.x, d.y);
}

// read-only (non-coherent) loads
__device__ __forceinline__ double ld_ro(const double* p) { return __ldg(p); }
__device__ __forceinline__ float ld_ro(const float* p) { return __ldg(p); }
__device__ __forceinline__ cplx ld_ro(const cplx* p) {
  const double2 d = __ldg(reinterpret_cast<const double2*>(p));
  return mkc(d.x, d.y);
}

// Three sums reduced together in one grid reduction.
template <typename T>
struct Tri {
  T a, b, c;
};
template <typename T>
__device__ __forceinline__ Tri<T> vzero(Tri<T>) {
  return Tri<T>{vzero(T{}), vzero(T{}), vzero(T{})};
}
template <typename T>
__device__ __forceinline__ Tri<T> vadd(Tri<T> x, Tri<T> y) {
  return Tri<T>{vadd(x.a, y.a), vadd(x.b, y.b), vadd(x.c, y.c)};
}
template <typename T>
__device__ __forceinline__ Tri<T> shfl_xor(Tri<T> v, int o) {
  return Tri<T>{shfl_xor(v.a, o), shfl_xor(v.b, o), shfl_xor(v.c, o)};
}
template <typename T>
__device__ __forceinline__ Tri<T> shfl_down(Tri<T> v, int o) {
  return Tri<T>{shfl_down(v.a, o), shfl_down(v.b, o), shfl_down(v.c, o)};
}
template <typename T>
__device__ __forceinline__ Tri<T> ld_cg(const Tri<T>* p) {
  return Tri<T>{ld_cg(&p->a), ld_cg(&p->b), ld_cg(&p->c)};
}

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = vadd(v, shfl_xor(v, o));
  return v;
}

// The warp's sum in lane 0 only (the other lanes hold partial sums): the same
// operand pairs as warp_sum's lane 0, so the same bits, with adds only in the
// lanes still needed at each level (a fifth of warp_sum's FP64 work).
template <typename T>
__device__ __forceinline__ T warp_sum0(T v) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const T t = shfl_down(v, o);
    if (lane < o) v = vadd(v, t);
  }
  return v;
}

// Sum over the block; the result is valid in thread 0.  smem >= 32 entries.
// Each level of the trees adds only in the lanes whose sum is still needed
// (lane < offset) and the warp totals take log2(warps) levels, not five: lane
// 0 pairs its operands exactly as the butterfly of warp_sum does, with less
// work for GB300's narrow FP64 pipe.
template <typename T>
__device__ __forceinline__ T block_sum(T v, T* smem) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nw = (blockDim.x + 31) >> 5;
  v = warp_sum0(v);
  __syncthreads();
  if (lane == 0) smem[warp] = v;
  __syncthreads();
  T r = vzero(v);
  if (warp == 0) {
    r = (lane < nw) ? smem[lane] : vzero(v);
    int top = 1;
    while (top < nw) top <<= 1;
    for (int o = top >> 1; o > 0; o >>= 1) {
      const T t = shfl_down(r, o);
      if (lane < o) r = vadd(r, t);
    }
  }
  return r;
}

// Grid reduction slot: per-block partials and ticket counters (zero at rest).
// With `gpart` set the reduction is two-level: blocks are grouped by
// kRedGroup, the last block of each group sums the group (ticket[1 + group]),
// the last group sums the group totals (ticket[0]).  Without it the last
// block sums every block partial.
constexpr int kRedGroup = 64;
constexpr int kRedMaxGroups = 1024;

template <typename T>
struct GridRed {
  T* partials;
  unsigned int* ticket;
  T* gpart = nullptr;
};

// Ticket of a grid reduction: one atomic increment at device scope with
// acquire-release order.  Its release half publishes the caller's earlier
// writes (the block's partial, and through the preceding block barrier those
// of its other threads); its acquire half, in the thread that draws the last
// ticket, makes every partial released before it visible to that thread and,
// through the block barrier that follows, to the rest of its block.  This
// replaces a full fence before the increment and a fence in every thread of
// the last block after it.
__device__ __forceinline__ unsigned ticket_add(unsigned int* p) {
  unsigned old;
  asm volatile("atom.acq_rel.gpu.global.add.u32 %0, [%1], 1;" : "=r"(old) : "l"(p) : "memory");
  return old;
}

// Thread t's share of a block's sum over p[0, count): p[t] + p[t + blockDim] +
// ... added in that order, with kInFlight loads issued before their additions
// (one round trip to L2 per kInFlight terms instead of one per term).
template <int kInFlight, typename T>
__device__ __forceinline__ T strided_sum(const T* p, int count, T zero) {
  T acc = zero;
  for (int i0 = threadIdx.x; i0 < count; i0 += kInFlight * (int)blockDim.x) {
    T x[kInFlight];
#pragma unroll
    for (int u = 0; u < kInFlight; ++u) {
      const int i = i0 + u * (int)blockDim.x;
      x[u] = i < count ? ld_cg(p + i) : zero;
    }
#pragma unroll
    for (int u = 0; u < kInFlight; ++u)
      if (i0 + u * (int)blockDim.x < count) acc = vadd(acc, x[u]);
  }
  return acc;
}

// Every thread of every block calls this with its value; the last block to
// arrive returns true in all its threads and thread 0 of it writes *total
// (and, with `held` set, keeps the total there: no reload of *total).
template <typename T>
__device__ __forceinline__ bool grid_sum_flat(T v, GridRed<T> R, T* total, T* held = nullptr) {
  __shared__ T smem[32];
  __shared__ bool last;
  const T b = block_sum(v, smem);
  if (threadIdx.x == 0) {
    R.partials[blockIdx.x] = b;
    last = (ticket_add(R.ticket) == gridDim.x - 1);
  }
  __syncthreads();
  if (!last) return false;
  const T acc = strided_sum<4>(R.partials, (int)gridDim.x, vzero(v));
  const T tot = block_sum(acc, smem);
  if (threadIdx.x == 0) {
    *total = tot;
    *R.ticket = 0u;
    if (held) *held = tot;
  }
  return true;
}

// A one-level grid reduction for the Lanczos step's inner products: every block
// posts its block total; the last block to arrive loads all the partials at once
// (thread t takes partials t, t + blockDim, ... in turn) and forms the total with
// one block sum, returning true in all its threads; thread 0 of it writes *total.
// The one-launch step and the two-launch products both reduce their dots this
// way, so both forms of the step carry the same bits.  With `held` set, thread
// 0 of the last block also keeps the total there (no reload of *total).
template <typename T>
__device__ __forceinline__ bool grid_sum_ordered(T v, GridRed<T> R, T* total, T* held = nullptr) {
  __shared__ T smem_o[32];
  __shared__ bool last_o;
  const T b = block_sum(v, smem_o);
  if (threadIdx.x == 0) {
    R.partials[blockIdx.x] = b;
    last_o = (ticket_add(R.ticket) == gridDim.x - 1);
  }
  __syncthreads();
  if (!last_o) return false;
  // two triples in flight keep the one-launch step within its 40 registers
  const T acc = strided_sum<sizeof(T) <= 16 ? 4 : 2>(R.partials, (int)gridDim.x, vzero(v));
  const T tot = block_sum(acc, smem_o);
  if (threadIdx.x == 0) {
    *total = tot;
    *R.ticket = 0u;
    if (held) *held = tot;
  }
  return true;
}

template <typename T>
__device__ __forceinline__ bool grid_sum(T v, GridRed<T> R, T* total, T* held = nullptr) {
  if (!R.gpart) return grid_sum_flat(v, R, total, held);
  __shared__ T smem2[32];
  __shared__ bool last2;
  const T b = block_sum(v, smem2);
  const unsigned group = blockIdx.x / kRedGroup;
  const unsigned gsize = min((unsigned)kRedGroup, gridDim.x - group * kRedGroup);
  const unsigned ngroups = (gridDim.x + kRedGroup - 1) / kRedGroup;
  if (threadIdx.x == 0) {
    R.partials[blockIdx.x] = b;
    last2 = (ticket_add(R.ticket + 1 + group) == gsize - 1);
  }
  __syncthreads();
  if (!last2) return false;
  const T acc = strided_sum<4>(R.partials + group * kRedGroup, (int)gsize, vzero(v));
  const T gs = block_sum(acc, smem2);
  if (threadIdx.x == 0) {
    R.gpart[group] = gs;
    R.ticket[1 + group] = 0u;
    last2 = (ticket_add(R.ticket) == ngroups - 1);
  }
  __syncthreads();
  if (!last2) return false;
  const T acc2 = strided_sum<4>(R.gpart, (int)ngroups, vzero(v));
  const T tot = block_sum(acc2, smem2);
  if (threadIdx.x == 0) {
    *total = tot;
    *R.ticket = 0u;
    if (held) *held = tot;
  }
  return true;
}

}  // namespace qd
