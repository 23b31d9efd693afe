// fxblock.cu -- the uniform-coupling product on the block layout of a sector (kernel code 122).
//
// A sector ranked by the combinatorial number system (one popcount over the
// whole register, or two on a low and a high field) lists its states in
// ascending order, i.e. by their high part h first: every high part owns one
// contiguous block of rows, and inside a block the rows run over the low parts
// l of one popcount in ascending order, so row(h, l) = off[h] + rank_low(l).
// The operator's transitions (the compiled terms, each a support, an input
// pattern on it and a flip) then fall into three kinds:
//   * low  (support in the low part):  the column stays in the row's block,
//     at position rank_low(l ^ flip): a table of the targets of every low
//     part l, shared by all blocks, gives them (ladj, a few KB, cached);
//   * high (support in the high part): the column sits at the same position
//     i of another block off[h ^ flip] + i: a table of the target blocks of
//     every high part h (hadj); the 32 lanes of a warp hold consecutive rows
//     of one block, so these gathers are consecutive 16-byte loads;
//   * crossing (a support over both parts, e.g. the bond between the halves
//     of a chain): the column is ranked from the two parts directly.
// No column index is read and no row is searched: each row reads its 32-bit
// state, its diagonal and x, and gathers its fixed-point X values (mostly from
// its own block, which the CTA's 256 consecutive rows share, or as coalesced
// runs).  The integer sums are exact, so the products carry the bits of the
// stored-column form (code 120); the one-launch Lanczos step runs this form on
// the same grid, row order and reduction tree, so the whole recurrence is
// bit-identical to code 120's.  The form is kept only after a check over
// every row that its columns are exactly the stored ones.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "fxstep.cuh"
#include "fxsum.cuh"
#include "ham.cuh"
#include "krylov.cuh"

namespace qd {

constexpr int kBlkMaxCross = 8;
constexpr int kBlkMaxBits = 16;  // per part: tables of 2^16 entries at most

struct BlockRows {
  const uint32_t* state;     // the basis in 32 bits
  const int32_t* off;        // 2^highbits: first row of block h
  const uint16_t* rank_low;  // 2^lowbits: rank of l among the low parts of its popcount
  const uint8_t* ldeg;       // 2^lowbits: low targets of l
  const uint16_t* ladj;      // 2^lowbits x lstride: their positions in the block
  const uint8_t* hdeg;       // 2^highbits: high targets of h
  const int32_t* hadj;       // 2^highbits x hstride: first row of each target block
  const __int128* X;
  int lowbits, lstride, hstride, ncross;
  uint32_t cross[3 * kBlkMaxCross];  // support, input pattern, flip
  __device__ const BlockRows& bind(unsigned char*) const { return *this; }
  __device__ __forceinline__ __int128 row_sum(int64_t r) const {
    const uint32_t s = __ldcs(state + r);
    const uint32_t lmask = (1u << lowbits) - 1u;
    const uint32_t h = s >> lowbits, l = s & lmask;
    const int base = __ldg(off + h);
    const int i = (int)r - base;
    __int128 sum = 0;
    const int dl = __ldg(ldeg + l);
    const uint16_t* la = ladj + (size_t)l * lstride;
    int j = 0;
#pragma unroll 1
    for (; j + 1 < dl; j += 2) {  // two gathers in flight
      const int p0 = __ldg(la + j), p1 = __ldg(la + j + 1);
      const __int128 x0 = X[base + p0], x1 = X[base + p1];
      sum += x0 + x1;
    }
    if (j < dl) sum += X[base + __ldg(la + j)];
    const int dh = __ldg(hdeg + h);
    const int32_t* ha = hadj + (size_t)h * hstride;
    j = 0;
#pragma unroll 1
    for (; j + 1 < dh; j += 2) {
      const int b0 = __ldg(ha + j), b1 = __ldg(ha + j + 1);
      const __int128 x0 = X[b0 + i], x1 = X[b1 + i];
      sum += x0 + x1;
    }
    if (j < dh) sum += X[__ldg(ha + j) + i];
#pragma unroll 1
    for (int t = 0; t < ncross; ++t) {
      if ((s & cross[3 * t]) != cross[3 * t + 1]) continue;
      const uint32_t c = s ^ cross[3 * t + 2];
      sum += X[__ldg(off + (c >> lowbits)) + __ldg(rank_low + (c & lmask))];
    }
    return sum;
  }
  // The same sum with the row's own block staged in shared memory: xs holds the X values of
  // rows [g0, g0 + len) of the group that contains the row's whole block.
  __device__ __forceinline__ __int128 row_sum_staged(int r, const __int128* xs, int g0) const {
    const uint32_t s = __ldcs(state + r);
    const uint32_t lmask = (1u << lowbits) - 1u;
    const uint32_t h = s >> lowbits, l = s & lmask;
    const int base = __ldg(off + h);
    const int i = r - base;
    const __int128* xb = xs + (base - g0);
    __int128 sum = 0;
    const int dh = __ldg(hdeg + h);
    const int32_t* ha = hadj + (size_t)h * hstride;
    int j = 0;
#pragma unroll 1
    for (; j + 1 < dh; j += 2) {  // the other blocks' values first: their loads are the long ones
      const int b0 = __ldg(ha + j), b1 = __ldg(ha + j + 1);
      const __int128 x0 = X[b0 + i], x1 = X[b1 + i];
      sum += x0 + x1;
    }
    if (j < dh) sum += X[__ldg(ha + j) + i];
#pragma unroll 1
    for (int t = 0; t < ncross; ++t) {
      if ((s & cross[3 * t]) != cross[3 * t + 1]) continue;
      const uint32_t c = s ^ cross[3 * t + 2];
      sum += X[__ldg(off + (c >> lowbits)) + __ldg(rank_low + (c & lmask))];
    }
    const int dl = __ldg(ldeg + l);
    const uint16_t* la = ladj + (size_t)l * lstride;
#pragma unroll 4
    for (j = 0; j < dl; ++j) sum += xb[__ldg(la + j)];
    return sum;
  }
};

// Every row's block-form columns against its stored columns (fxsum.cu): the
// same number, each one present, no repeats.
__global__ void fx_block_check_kernel(int64_t n, BlockRows B, const int32_t* rowptr, const int32_t* colidx,
                                      int* bad) {
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
    const uint32_t s = B.state[r];
    const uint32_t lmask = (1u << B.lowbits) - 1u;
    const uint32_t h = s >> B.lowbits, l = s & lmask;
    const int base = B.off[h];
    const int i = (int)r - base;
    int cols[64];
    int cnt = 0;
    bool ok = base >= 0 && i >= 0;
    for (int j = 0; j < B.ldeg[l] && ok; ++j) {
      if (cnt == 64) ok = false;
      else cols[cnt++] = base + B.ladj[(size_t)l * B.lstride + j];
    }
    for (int j = 0; j < B.hdeg[h] && ok; ++j) {
      if (cnt == 64) ok = false;
      else cols[cnt++] = B.hadj[(size_t)h * B.hstride + j] + i;
    }
    for (int t = 0; t < B.ncross && ok; ++t) {
      if ((s & B.cross[3 * t]) != B.cross[3 * t + 1]) continue;
      const uint32_t c = s ^ B.cross[3 * t + 2];
      const int ob = B.off[c >> B.lowbits];
      if (cnt == 64 || ob < 0) ok = false;
      else cols[cnt++] = ob + B.rank_low[c & lmask];
    }
    const int b = rowptr[r], e = rowptr[r + 1];
    if (ok && cnt != e - b) ok = false;
    for (int a = 0; a < cnt && ok; ++a) {
      if (cols[a] < 0 || cols[a] >= n || cols[a] == (int)r) ok = false;
      for (int q = 0; q < a && ok; ++q)
        if (cols[q] == cols[a]) ok = false;
      bool found = false;
      for (int k = b; k < e && !found; ++k) found = colidx[k] == cols[a];
      if (!found) ok = false;
    }
    if (!ok) atomicOr(bad, 1);
  }
}

// Without stored columns (the matrix-free form): every row's block-form columns hold exactly the
// states the operator's transitions reach from the row's state, each once.
__global__ void fx_block_check_states_kernel(int64_t n, BlockRows B, const uint32_t* trans, int ntrans, int* bad) {
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
    const uint32_t s = B.state[r];
    const uint32_t lmask = (1u << B.lowbits) - 1u;
    const uint32_t h = s >> B.lowbits, l = s & lmask;
    const int base = B.off[h];
    const int i = (int)r - base;
    int cols[64];
    int cnt = 0;
    bool ok = base >= 0 && i >= 0;
    for (int j = 0; j < B.ldeg[l] && ok; ++j) {
      if (cnt == 64) ok = false;
      else cols[cnt++] = base + B.ladj[(size_t)l * B.lstride + j];
    }
    for (int j = 0; j < B.hdeg[h] && ok; ++j) {
      if (cnt == 64) ok = false;
      else cols[cnt++] = B.hadj[(size_t)h * B.hstride + j] + i;
    }
    for (int t = 0; t < B.ncross && ok; ++t) {
      if ((s & B.cross[3 * t]) != B.cross[3 * t + 1]) continue;
      const uint32_t c = s ^ B.cross[3 * t + 2];
      const int ob = B.off[c >> B.lowbits];
      if (cnt == 64 || ob < 0) ok = false;
      else cols[cnt++] = ob + B.rank_low[c & lmask];
    }
    int want = 0;
    for (int t = 0; t < ntrans; ++t) want += ((s & trans[3 * t]) == trans[3 * t + 1]) ? 1 : 0;
    if (ok && cnt != want) ok = false;
    for (int a = 0; a < cnt && ok; ++a) {
      if (cols[a] < 0 || cols[a] >= n || cols[a] == (int)r) {
        ok = false;
        break;
      }
      for (int q = 0; q < a && ok; ++q)
        if (cols[q] == cols[a]) ok = false;
      const uint32_t sc = B.state[cols[a]];
      bool found = false;
      for (int t = 0; t < ntrans && !found; ++t)
        found = (s & trans[3 * t]) == trans[3 * t + 1] && (s ^ trans[3 * t + 2]) == sc;
      if (!found) ok = false;
    }
    if (!ok) atomicOr(bad, 1);
  }
}

__global__ void fx_block_state_kernel(int64_t n, const uint64_t* basis, uint32_t* out) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = (uint32_t)basis[i];
}

// y = s (d x + c 2^-F sum X): the plain product of the block form (timing).
__global__ void __launch_bounds__(256) spmv_fx_block_kernel(int64_t n, BlockRows B, const double* __restrict__ diag,
                                                            const double* __restrict__ x, double* __restrict__ y,
                                                            double cF) {
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
    const __int128 sum = B.row_sum(r);
    y[r] = fma(cF, (double)sum, __ldcs(diag + r) * __ldg(x + r));
  }
}

// The product fused with the Lanczos step's three inner products (the two-launch step), on the grid,
// row order and reduction tree of spmv_fx_dots_kernel: the same bits as code 120's.
template <bool kHas2>
__global__ void __launch_bounds__(256, 6) spmv_fx_block_dots_kernel(
    int64_t n, BlockRows B, const double* __restrict__ diag, const double* __restrict__ x,
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
    const __int128 s = B.row_sum(r);
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

// ---------------------------------------------------------------- staged one-launch step
// The whole Lanczos step on the block layout with each CTA owning a contiguous
// run of rows made of whole blocks, grouped so that a group (one or more
// consecutive blocks, at most kBlkGroupRows rows unless one block is larger)
// is staged in shared memory by one bulk (TMA) copy: the low-part gathers of
// every row then come from shared memory, and only the other blocks' values
// (coalesced, warp-uniform targets) and the crossing transitions go to L2.
// The next group's copy is issued before the current group is summed (two
// buffers, an mbarrier each).  w stays in shared memory for the update half,
// as in lz_fx_step_kernel; the three dots, the bounded grid barrier that
// publishes alpha and beta, and the update follow that kernel.  Each row's w
// carries the bits of code 120's product; the dots add in another order, so
// alpha and beta agree with code 120's to rounding.
constexpr int kBlkGroupRows = 1024;
constexpr unsigned kBlkCopySpinLimit = 1u << 24;  // polls of a group's copy before giving up

struct BlkPart {
  const int2* groups;     // first and end row of each group
  const int32_t* cta_first;  // first group of each CTA (nctas + 1 entries)
  int max_group;          // rows of the largest group (staging buffer length)
  int max_cta;            // rows of the largest CTA run (w length)
};

__device__ __forceinline__ uint32_t blk_smem_addr(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void blk_issue_copy(__int128* dst, const __int128* src, int rows, uint64_t* bar) {
  const uint32_t bytes = (uint32_t)rows * 16u;
  asm volatile("mbarrier.arrive.expect_tx.shared.b64 _, [%0], %1;" ::"r"(blk_smem_addr(bar)), "r"(bytes)
               : "memory");
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          blk_smem_addr(dst)),
      "l"(src), "r"(bytes), "r"(blk_smem_addr(bar))
      : "memory");
}

// Bounded wait for the phase `parity` of an mbarrier; false when it ran out.
__device__ __forceinline__ bool blk_wait(uint64_t* bar, unsigned parity) {
  for (unsigned polls = 0; polls < kBlkCopySpinLimit; ++polls) {
    uint32_t done = 0;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(blk_smem_addr(bar)), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

template <int kThreads, bool kHas2>
__global__ void __launch_bounds__(kThreads, 1024 / kThreads) lz_fx_blkstep_kernel(BlockRows B, BlkPart P,
                                                                                 FxStepArgs a) {
  if (a.stop) {
    const int st = *a.stop;
    if (st != 0 && st < a.step) return;
  }
  extern __shared__ __align__(16) unsigned char blk_smem[];
  __int128* xs0 = reinterpret_cast<__int128*>(blk_smem);
  __int128* xs1 = xs0 + P.max_group;
  double* wst = reinterpret_cast<double*>(xs1 + P.max_group);
  __shared__ __align__(8) uint64_t bar[2];
  __shared__ unsigned e0;
  __shared__ int waited_out, copy_bad;
  __shared__ double ab[2];
  const int g0 = P.cta_first[blockIdx.x], g1 = P.cta_first[blockIdx.x + 1];
  const int crow0 = (g0 < g1) ? P.groups[g0].x : 0;
  const int crow1 = (g0 < g1) ? P.groups[g1 - 1].y : 0;
  if (threadIdx.x == 0) {
    e0 = *reinterpret_cast<volatile unsigned*>(a.epoch);
    waited_out = 0;
    copy_bad = 0;
    asm volatile("mbarrier.init.shared.b64 [%0], 1;" ::"r"(blk_smem_addr(&bar[0])) : "memory");
    asm volatile("mbarrier.init.shared.b64 [%0], 1;" ::"r"(blk_smem_addr(&bar[1])) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  if (threadIdx.x == 0 && g0 < g1) {
    const int2 gr = P.groups[g0];
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    blk_issue_copy(xs0, B.X + gr.x, gr.y - gr.x, &bar[0]);
  }
  // first half: w = s1 (d x + c 2^-F sum X) and the three dots
  const double sc = *a.s1;
  Tri<double> acc = vzero(Tri<double>{});
  // per buffer: the parity of its next phase and whether a copy into it is in flight (the same
  // values in every thread: each wait's outcome is agreed by the whole block)
  unsigned par0 = 0, par1 = 0;
  bool out0 = g0 < g1, out1 = false;
  for (int g = g0; g < g1; ++g) {
    const int buf = (g - g0) & 1;
    __int128* xs = buf ? xs1 : xs0;
    if (g + 1 < g1) {  // the other buffer's readers passed the barrier below
      if (threadIdx.x == 0) {
        const int2 nx = P.groups[g + 1];
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        blk_issue_copy(buf ? xs0 : xs1, B.X + nx.x, nx.y - nx.x, &bar[buf ^ 1]);
      }
      if (buf) out0 = true;
      else out1 = true;
    }
    if (!__syncthreads_and(blk_wait(&bar[buf], buf ? par1 : par0))) {
      // a copy that did not land: flag the solve and stop issuing or reading copies
      if (threadIdx.x == 0) copy_bad = 1;
      break;
    }
    if (buf) {
      par1 ^= 1u;
      out1 = false;
    } else {
      par0 ^= 1u;
      out0 = false;
    }
    const int2 gr = P.groups[g];
    for (int r = gr.x + (int)threadIdx.x; r < gr.y; r += blockDim.x) {
      const __int128 s = B.row_sum_staged(r, xs, gr.x);
      const double xr = __ldcs(a.x + r);
      const double w = sc * fma(a.cF, (double)s, a.diag ? __ldcs(a.diag + r) * xr : 0.0);
      wst[r - crow0] = w;
      acc.b = fma(xr, w, acc.b);
      if (kHas2) {
        const double v2 = __ldcs(a.V2 + r);
        acc.a = fma(v2, w, acc.a);
        acc.c = fma(xr, v2, acc.c);
      }
    }
    __syncthreads();
  }
  // copies still in flight (only after a wait ran out) get one more bounded wait before the
  // block moves on, so none lands after the block has left
  if (out0) blk_wait(&bar[0], par0);
  if (out1) blk_wait(&bar[1], par1);
  __syncthreads();
  if (threadIdx.x == 0 && copy_bad) atomicExch(a.ovf + 1, 1);
  if (grid_sum(acc, a.red, a.dots) && threadIdx.x < 32) {
    double bt = 0.0, al = 0.0;
    if (threadIdx.x == 0) {
      const Tri<double> d = *a.dots;
      bt = kHas2 ? (*a.s2) * d.a : 0.0;
      double t = d.b;
      if (kHas2) t = fma(-(bt * (*a.s2)), d.c, t);
      al = (*a.s1) * t;
      *a.beta = bt;
      *a.alpha = al;
    }
    if (!a.hold_publish) mbox_publish(a.mbox, a.epoch, e0, al, bt);
  }
  if (threadIdx.x == 0) {
    double al, bt;
    if (!mbox_wait(a.mbox, e0, a.spin_limit ? a.spin_limit : kStepSpinLimit, 200, &al, &bt)) {
      waited_out = 1;
      atomicExch(a.ovf + 1, 1);
    }
    ab[0] = al;
    ab[1] = bt;
  }
  __syncthreads();
  // second half: v_k = (w - (beta s2) V2) - (alpha s1) V1 on the CTA's rows
  double acc0 = 0.0;
  int out = 0;
  if (!waited_out) {
    const double al = (*a.s1) * ab[0];
    const double bt = kHas2 ? (*a.s2) * ab[1] : 0.0;
    for (int r = crow0 + (int)threadIdx.x; r < crow1; r += blockDim.x) {
      double o = wst[r - crow0];
      if (kHas2) o = fma(-bt, __ldcs(a.V2 + r), o);
      o = fma(-al, __ldcs(a.x + r), o);
      __stcs(a.Vk + r, o);
      a.Xk[r] = fx_from_double(o, a.F, &out);
      acc0 = fma(o, o, acc0);
    }
  }
  if (out) a.ovf[0] = 1;
  // every block arrives here, waited out or not, so the ticket counts stay whole
  double n2 = 0.0;
  if (grid_sum(acc0, a.rd, a.nrm2, &n2) && threadIdx.x == 0) {
    const double nr = sqrt(n2);
    *a.nrm = nr;
    *a.sk = 1.0 / nr;
    if (nr < 1e-10 && a.stop && *a.stop == 0) *a.stop = a.step;  // sparse_algorithm.hpp:421
  }
}

static BlockRows block_rows(const FxForm& f, const __int128* X) {
  BlockRows B;
  std::memset(&B, 0, sizeof(B));
  B.state = f.blk_state32.p;
  B.off = f.blk_off.p;
  B.rank_low = f.blk_rank.p;
  B.ldeg = f.blk_ldeg.p;
  B.ladj = f.blk_ladj.p;
  B.hdeg = f.blk_hdeg.p;
  B.hadj = f.blk_hadj.p;
  B.X = X;
  B.lowbits = f.blk_lowbits;
  B.lstride = f.blk_lstride;
  B.hstride = f.blk_hstride;
  B.ncross = f.blk_ncross;
  for (int q = 0; q < 3 * kBlkMaxCross; ++q) B.cross[q] = f.blk_cross[q];
  return B;
}

static void drop_block(FxForm& f) {
  f.blk_state32.release();
  f.blk_off.release();
  f.blk_rank.release();
  f.blk_ldeg.release();
  f.blk_ladj.release();
  f.blk_hdeg.release();
  f.blk_hadj.release();
}

// The tables of the block form for the transitions of value c; false when the
// sector or the terms do not give this form.
static bool make_block(qd_ham* H, FxForm& f, std::vector<uint32_t>* trans_out = nullptr) {
  const SectorView& V = H->sec->view;
  if (!H->from_terms || V.rank_kind != 1 || V.nbits > 32 || H->dim >= (1ll << 31)) return false;
  int lowbits = 0;
  uint32_t fmask[2] = {0u, 0u};
  int fk[2] = {0, 0};
  const int nbits = V.nbits;
  if (V.nfields == 1) {
    const Field& F = V.fields[0];
    if (F.is_free || F.lo != 0 || F.width != nbits) return false;
    // a short low half: a block's own values span a few cache lines, so a warp's low-half gathers
    // touch few lines; the long high half's targets are coalesced runs.  QD_FX_BLOCK_LOW overrides.
    lowbits = std::min(nbits / 2, 8);
    const char* el = std::getenv("QD_FX_BLOCK_LOW");
    if (el) lowbits = std::atoi(el);
    lowbits = std::max(lowbits, nbits - kBlkMaxBits);
    fmask[0] = (nbits >= 32) ? 0xffffffffu : ((1u << nbits) - 1u);
    fk[0] = F.k;
  } else if (V.nfields == 2) {
    const Field& A0 = V.fields[0];
    const Field& A1 = V.fields[1];
    const Field& Lo = (A0.lo < A1.lo) ? A0 : A1;
    const Field& Hi = (A0.lo < A1.lo) ? A1 : A0;
    if (Lo.is_free || Hi.is_free || Lo.lo != 0 || Hi.lo != Lo.width || Lo.width + Hi.width != nbits) return false;
    lowbits = Lo.width;
    fmask[0] = (1u << Lo.width) - 1u;
    fmask[1] = (uint32_t)((((uint64_t)1 << Hi.width) - 1) << Hi.lo);
    fk[0] = Lo.k;
    fk[1] = Hi.k;
  } else {
    return false;
  }
  const int highbits = nbits - lowbits;
  if (lowbits < 1 || highbits < 1 || lowbits > kBlkMaxBits || highbits > kBlkMaxBits) return false;
  const uint32_t lmask = (1u << lowbits) - 1u;
  std::vector<MfEntry> off, dia;
  try {
    compile_terms(H, off, dia);
  } catch (const Error&) {  // terms the compiled form does not take
    clear_error();
    return false;
  }
  struct Tr {
    uint32_t sup, outb, flip;
  };
  std::vector<Tr> low, high, cross;
  for (const MfEntry& e : off) {
    if (e.amp.im != 0.0 || e.jw != 0) return false;
    if (e.amp.re == 0.0) continue;  // an explicit zero is no column of the uniform form
    if (e.amp.re != f.c) return false;
    const Tr t{(uint32_t)e.sup, (uint32_t)e.outb, (uint32_t)e.flip};
    bool in = true;
    for (int q = 0; q < V.nfields; ++q)
      in &= __builtin_popcount(t.outb & fmask[q]) == __builtin_popcount((t.outb ^ t.flip) & fmask[q]);
    if (!in) continue;  // the target leaves the sector: the lowering drops it
    for (const std::vector<Tr>* L : {&low, &high, &cross})
      for (const Tr& u : *L)
        if (u.sup == t.sup && u.outb == t.outb && u.flip == t.flip) return false;  // 2c on one column
    if ((t.sup & ~lmask) == 0u) low.push_back(t);
    else if ((t.sup & lmask) == 0u) high.push_back(t);
    else cross.push_back(t);
  }
  if ((int)cross.size() > kBlkMaxCross || (low.empty() && high.empty() && cross.empty())) return false;
  if (trans_out)
    for (const std::vector<Tr>* L : {&low, &high, &cross})
      for (const Tr& t : *L) trans_out->insert(trans_out->end(), {t.sup, t.outb, t.flip});
  // ranks of the low parts, blocks of the high parts
  const uint32_t nl = 1u << lowbits, nh = 1u << highbits;
  std::vector<uint16_t> rank_low(nl);
  {
    std::vector<int> cnt(lowbits + 1, 0);
    for (uint32_t l = 0; l < nl; ++l) {
      const int k = __builtin_popcount(l);
      if (cnt[k] > 0xffff) return false;
      rank_low[l] = (uint16_t)cnt[k]++;
    }
  }
  int64_t C[33][33];
  for (int a = 0; a <= 32; ++a)
    for (int b = 0; b <= 32; ++b) C[a][b] = (b == 0) ? 1 : (a == 0 ? 0 : C[a - 1][b - 1] + C[a - 1][b]);
  std::vector<int32_t> offs(nh, -1);
  int64_t row = 0;
  for (uint32_t h = 0; h < nh; ++h) {
    const int ph = __builtin_popcount(h);
    int kl;
    if (V.nfields == 1) {
      kl = fk[0] - ph;
    } else {
      if (ph != fk[1]) continue;
      kl = fk[0];
    }
    if (kl < 0 || kl > lowbits) continue;
    offs[h] = (int32_t)row;
    row += C[lowbits][kl];
  }
  if (row != H->dim) return false;  // not the sector's layout
  // targets of every low part and every high part
  std::vector<std::vector<uint16_t>> la(nl);
  size_t lstride = 1, hstride = 1;
  for (uint32_t l = 0; l < nl; ++l) {
    for (const Tr& t : low)
      if ((l & t.sup) == t.outb) la[l].push_back(rank_low[l ^ t.flip]);
    lstride = std::max(lstride, la[l].size());
  }
  std::vector<std::vector<int32_t>> ha(nh);
  for (uint32_t h = 0; h < nh; ++h) {
    if (offs[h] < 0) continue;
    for (const Tr& t : high)
      if ((h & (t.sup >> lowbits)) == (t.outb >> lowbits)) {
        const int32_t b = offs[h ^ (t.flip >> lowbits)];
        if (b < 0) return false;
        ha[h].push_back(b);
      }
    hstride = std::max(hstride, ha[h].size());
  }
  if (lstride > 255 || hstride > 255) return false;
  std::vector<uint8_t> ldeg(nl), hdeg(nh);
  std::vector<uint16_t> ladj(nl * lstride, 0);
  std::vector<int32_t> hadj(nh * hstride, 0);
  for (uint32_t l = 0; l < nl; ++l) {
    ldeg[l] = (uint8_t)la[l].size();
    std::copy(la[l].begin(), la[l].end(), ladj.begin() + (size_t)l * lstride);
  }
  for (uint32_t h = 0; h < nh; ++h) {
    hdeg[h] = (uint8_t)ha[h].size();
    std::copy(ha[h].begin(), ha[h].end(), hadj.begin() + (size_t)h * hstride);
  }
  Ctx* ctx = H->ctx;
  const int64_t n = H->dim;
  f.blk_lowbits = lowbits;
  f.blk_lstride = (int)lstride;
  f.blk_hstride = (int)hstride;
  f.blk_ncross = (int)cross.size();
  std::memset(f.blk_cross, 0, sizeof(f.blk_cross));
  for (size_t q = 0; q < cross.size(); ++q) {
    f.blk_cross[3 * q] = cross[q].sup;
    f.blk_cross[3 * q + 1] = cross[q].outb;
    f.blk_cross[3 * q + 2] = cross[q].flip;
  }
  f.blk_off.alloc(nh);
  f.blk_rank.alloc(nl);
  f.blk_ldeg.alloc(nl);
  f.blk_ladj.alloc(ladj.size());
  f.blk_hdeg.alloc(nh);
  f.blk_hadj.alloc(hadj.size());
  f.blk_state32.alloc(n);
  QD_CUDA(cudaMemcpyAsync(f.blk_off.p, offs.data(), nh * 4, cudaMemcpyHostToDevice, ctx->stream));
  QD_CUDA(cudaMemcpyAsync(f.blk_rank.p, rank_low.data(), nl * 2, cudaMemcpyHostToDevice, ctx->stream));
  QD_CUDA(cudaMemcpyAsync(f.blk_ldeg.p, ldeg.data(), nl, cudaMemcpyHostToDevice, ctx->stream));
  QD_CUDA(cudaMemcpyAsync(f.blk_ladj.p, ladj.data(), ladj.size() * 2, cudaMemcpyHostToDevice, ctx->stream));
  QD_CUDA(cudaMemcpyAsync(f.blk_hdeg.p, hdeg.data(), nh, cudaMemcpyHostToDevice, ctx->stream));
  QD_CUDA(cudaMemcpyAsync(f.blk_hadj.p, hadj.data(), hadj.size() * 4, cudaMemcpyHostToDevice, ctx->stream));
  const int g = (int)std::max<int64_t>(1, std::min<int64_t>(ceil_div(n, 256), (int64_t)ctx->num_sms * 8));
  fx_block_state_kernel<<<g, 256, 0, ctx->stream>>>(n, H->sec->basis.p, f.blk_state32.p);
  QD_CHECK_LAUNCH();
  QD_LAUNCHED(ctx);
  QD_CUDA(cudaStreamSynchronize(ctx->stream));  // the host tables are temporaries
  return true;
}

static bool make_block_part(Ctx* ctx, const qd_ham* H, FxForm& f);
static bool block_staged() {
  const char* e = std::getenv("QD_FX_BLOCK_STAGED");
  return e && std::strcmp(e, "1") == 0;
}


bool ham_build_fx_block(qd_ham* H) {
  FxForm& f = *H->fx;
  if (f.blk_state != 0) return f.blk_state > 0;
  f.blk_state = -1;
  if (!make_block(H, f)) {
    drop_block(f);
    return false;
  }
  Ctx* ctx = H->ctx;
  const int64_t n = H->dim;
  DBuf<int> bad(1);
  QD_CUDA(cudaMemsetAsync(bad.p, 0, sizeof(int), ctx->stream));
  const int g = (int)std::max<int64_t>(1, std::min<int64_t>(ceil_div(n, 256), (int64_t)ctx->num_sms * 8));
  fx_block_check_kernel<<<g, 256, 0, ctx->stream>>>(n, block_rows(f, nullptr), f.rowptr.p, f.colidx.p, bad.p);
  QD_CHECK_LAUNCH();
  QD_LAUNCHED(ctx);
  int b = 1;
  QD_CUDA(cudaMemcpyAsync(&b, bad.p, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  QD_CUDA(cudaStreamSynchronize(ctx->stream));
  if (b) {
    drop_block(f);
    return false;
  }
  f.blk_state = 1;
  if (block_staged()) make_block_part(ctx, H, f);  // the staged step's partition, before any stream capture
  return true;
}

// The block layout on the form built from the terms alone (the matrix-free Lanczos path), checked
// against the transitions' target states (there are no stored columns).
bool ham_build_mf_fx_block(qd_ham* H) {
  FxForm& f = *H->mfx;
  if (f.blk_state != 0) return f.blk_state > 0;
  f.blk_state = -1;
  std::vector<uint32_t> trans;
  if (!make_block(H, f, &trans) || trans.empty()) {
    drop_block(f);
    return false;
  }
  Ctx* ctx = H->ctx;
  const int64_t n = H->dim;
  DBuf<uint32_t> dtr(trans.size());
  DBuf<int> bad(1);
  QD_CUDA(cudaMemcpyAsync(dtr.p, trans.data(), trans.size() * 4, cudaMemcpyHostToDevice, ctx->stream));
  QD_CUDA(cudaMemsetAsync(bad.p, 0, sizeof(int), ctx->stream));
  const int g = (int)std::max<int64_t>(1, std::min<int64_t>(ceil_div(n, 256), (int64_t)ctx->num_sms * 8));
  fx_block_check_states_kernel<<<g, 256, 0, ctx->stream>>>(n, block_rows(f, nullptr), dtr.p, (int)(trans.size() / 3),
                                                          bad.p);
  QD_CHECK_LAUNCH();
  QD_LAUNCHED(ctx);
  int b = 1;
  QD_CUDA(cudaMemcpyAsync(&b, bad.p, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  QD_CUDA(cudaStreamSynchronize(ctx->stream));
  if (b) {
    drop_block(f);
    return false;
  }
  f.blk_state = 1;
  return true;
}

void launch_fx_block_dots(Ctx* ctx, const qd_ham* H, const FxForm& f, const double* x, const __int128* X,
                          const double* V2, double* y, const double* s1, const double* s2, const int* stop, int step,
                          double* beta, double* alpha, Tri<double>* dots, GridRed<Tri<double>> red, int grid) {
  const double cF = std::ldexp(f.c, -f.F);
  const BlockRows B = block_rows(f, X);
  if (V2)
    spmv_fx_block_dots_kernel<true><<<grid, 256, 0, ctx->stream>>>(H->dim, B, f.diag.p, x, V2, y, cF, s1, s2, stop,
                                                                    step, beta, alpha, dots, red);
  else
    spmv_fx_block_dots_kernel<false><<<grid, 256, 0, ctx->stream>>>(H->dim, B, f.diag.p, x, x, y, cF, s1, s1, stop,
                                                                     step, beta, alpha, dots, red);
  QD_CHECK_LAUNCH();
  QD_LAUNCHED(ctx);
}

// Groups of whole blocks and their runs per CTA for the staged step; false when the
// step's shared memory leaves no room for the grid on the device at once.
static bool make_block_part(Ctx* ctx, const qd_ham* H, FxForm& f) {
  if (f.blk_part_state != 0) return f.blk_part_state > 0;
  f.blk_part_state = -1;
  const int64_t n = H->dim;
  const int nh = 1 << (H->sec->view.nbits - f.blk_lowbits);
  std::vector<int32_t> offs(nh);
  QD_CUDA(cudaMemcpyAsync(offs.data(), f.blk_off.p, nh * 4, cudaMemcpyDeviceToHost, ctx->stream));
  QD_CUDA(cudaStreamSynchronize(ctx->stream));
  std::vector<int> starts;  // block starts in row order (off is ascending over the valid high parts)
  for (int h = 0; h < nh; ++h)
    if (offs[h] >= 0) starts.push_back(offs[h]);
  starts.push_back((int)n);
  std::vector<int2> groups;
  int gstart = starts[0];
  for (size_t b = 1; b < starts.size(); ++b) {
    // close the group before block b - 1 would push it past the row limit
    const int bstart = starts[b - 1];
    if (bstart > gstart && starts[b] - gstart > kBlkGroupRows) {
      groups.push_back(make_int2(gstart, bstart));
      gstart = bstart;
    }
  }
  groups.push_back(make_int2(gstart, (int)n));
  int maxg = 0;
  for (const int2& g : groups) maxg = std::max(maxg, g.y - g.x);
  int dev_smem = 0;
  QD_CUDA(cudaDeviceGetAttribute(&dev_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, ctx->device));
  int coop = 0;
  QD_CUDA(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, ctx->device));
  if (!coop) return false;
  // 512-thread CTAs two per SM, else 1024-thread CTAs one per SM (w of twice the rows)
  for (int per_sm = 2; per_sm >= 1; --per_sm) {
    const int threads = 1024 / per_sm;
    const int nctas = ctx->num_sms * per_sm;
    // contiguous runs of groups with about n / nctas rows each
    std::vector<int32_t> first(nctas + 1, (int)groups.size());
    int maxc = 0;
    size_t g = 0;
    for (int c = 0; c < nctas; ++c) {
      first[c] = (int)g;
      const int64_t target = (int64_t)(c + 1) * n / nctas;
      const int r0 = (g < groups.size()) ? groups[g].x : (int)n;
      while (g < groups.size() && (groups[g].y <= target || (int)g == first[c])) ++g;
      const int r1 = (g > (size_t)first[c]) ? groups[g - 1].y : r0;
      maxc = std::max(maxc, r1 - r0);
    }
    first[nctas] = (int)groups.size();
    if (g < groups.size()) continue;  // more groups than runs (cannot happen with rows >= CTAs)
    const size_t smem = (size_t)2 * maxg * 16 + (size_t)maxc * 8;
    if (smem + 2048 > (size_t)dev_smem) continue;
    auto k1 = (threads == 512) ? lz_fx_blkstep_kernel<512, true> : lz_fx_blkstep_kernel<1024, true>;
    auto k0 = (threads == 512) ? lz_fx_blkstep_kernel<512, false> : lz_fx_blkstep_kernel<1024, false>;
    QD_CUDA(cudaFuncSetAttribute(k1, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    QD_CUDA(cudaFuncSetAttribute(k0, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int occ = 0, occ0 = 0;
    QD_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k1, threads, smem));
    QD_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ0, k0, threads, smem));
    if (std::min(occ, occ0) < per_sm) continue;
    f.blk_threads = threads;
    f.blk_groups.alloc(groups.size());
    f.blk_cta_first.alloc(first.size());
    QD_CUDA(cudaMemcpyAsync(f.blk_groups.p, groups.data(), groups.size() * sizeof(int2), cudaMemcpyHostToDevice,
                            ctx->stream));
    QD_CUDA(cudaMemcpyAsync(f.blk_cta_first.p, first.data(), first.size() * 4, cudaMemcpyHostToDevice, ctx->stream));
    QD_CUDA(cudaStreamSynchronize(ctx->stream));
    f.blk_nctas = nctas;
    f.blk_max_group = maxg;
    f.blk_max_cta = maxc;
    f.blk_smem = smem;
    f.blk_part_state = 1;
    return true;
  }
  return false;
}

// The one-launch step of the block form: by default the grid, row order and reduction tree of
// code 120's step (lz_fx_step_kernel), bit-identical to it; QD_FX_BLOCK_STAGED=1 runs the staged
// step above instead (groups of whole blocks copied into shared memory).
bool launch_fx_block_step(Ctx* ctx, const qd_ham* H, const FxForm& f, FxStepArgs a, int grid) {
  (void)H;
  if (!block_staged()) return fx_step_launch(ctx, block_rows(f, a.X), a, grid, 0);
  if (f.blk_part_state <= 0) return false;  // no partition fits: the two-launch step
  BlkPart P;
  P.groups = f.blk_groups.p;
  P.cta_first = f.blk_cta_first.p;
  P.max_group = f.blk_max_group;
  P.max_cta = f.blk_max_cta;
  const BlockRows B = block_rows(f, a.X);
  auto kern = (f.blk_threads == 512) ? (a.V2 ? lz_fx_blkstep_kernel<512, true> : lz_fx_blkstep_kernel<512, false>)
                                     : (a.V2 ? lz_fx_blkstep_kernel<1024, true> : lz_fx_blkstep_kernel<1024, false>);
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)f.blk_nctas);
  cfg.blockDim = dim3((unsigned)f.blk_threads);
  cfg.dynamicSmemBytes = f.blk_smem;
  cfg.stream = ctx->stream;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeCooperative;
  at[0].val.cooperative = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  QD_CUDA(cudaLaunchKernelEx(&cfg, kern, B, P, a));
  QD_LAUNCHED(ctx);
  return true;
}

void launch_fx_block(Ctx* ctx, const qd_ham* H, const FxForm& f, const double* x, const __int128* X, double* y) {
  const int64_t n = H->dim;
  spmv_fx_block_kernel<<<(unsigned)std::max<int64_t>(1, ceil_div(n, 256)), 256, 0, ctx->stream>>>(
      n, block_rows(f, X), f.diag.p, x, y, std::ldexp(f.c, -f.F));
  QD_CHECK_LAUNCH();
  QD_LAUNCHED(ctx);
}

}  // namespace qd
