// fxstep.cuh -- one Lanczos step of the uniform-coupling form in one launch.
//
// A step of sparse_algorithm.hpp:395-425 is w = H v1; alpha, beta from
// <v2,w>, <v1,w>, <v1,v2>; v_k = (w - beta v2) - alpha v1; n_k = ||v_k||.
// Split in two launches (the fused product and dots, then the update) the
// step writes w to HBM and reads it back, and pays a launch boundary with its
// ramp and tail.  Here one cooperative launch does both halves: every thread
// keeps the w of its own rows in shared memory (rows r = gtid + i * stride,
// slot i * 256 + tid), the last block to post its partials of the three dots
// forms their total (one level: all its threads load the partials at once),
// publishes alpha and beta in a mailbox, every block waits for them (a bounded
// wait), and then updates the same rows it produced (in
// adjacent pairs, for 16-byte accesses): reads v1, v2, writes v_k, its
// fixed-point copy for the next product, and its share of ||v_k||^2.
//
// Per-element arithmetic is that of spmv_fx_dots_kernel + lz_update_kernel,
// and the dots use the same grid, row order and reduction order
// (grid_sum_ordered), so alpha, beta and v_k carry the same bits as the
// two-launch step; only the norm's reduction tree differs.
#pragma once

#include "fxsum.cuh"
#include "vec.cuh"

namespace qd {

// Polls of the mailbox before a block gives up on the others (with the
// back-off below, about a second; a healthy step waits a few microseconds).
constexpr unsigned kStepSpinLimit = 1u << 22;

// The mailbox through which the block that forms alpha and beta hands them to
// every block: two sets, used by alternate launches (the parity of an epoch
// word that every launch bumps), of 16 copies on separate 128-byte lines; block
// b reads copy b mod 16, so the polls spread over 16 lines.  Every entry is
// written once per launch from kMboxEmpty, a signalling NaN that no arithmetic
// produces: a block that reads two entries other than kMboxEmpty holds the
// final alpha and beta, with no fence and no second read.  The publisher also
// empties the other set for the next launch; the kernel boundary orders that
// before the next launch's reads.  A launch that publishes nothing (a step
// past a breakdown, or the test hold below) leaves both sets and the epoch as
// they were, so every launch starts with the set of its parity empty.
constexpr int kMboxCopies = 16;
constexpr int kMboxStride = 16;  // doubles from one copy to the next (128 bytes)
constexpr int kMboxDoubles = 2 * kMboxCopies * kMboxStride;
constexpr long long kMboxEmpty = 0x7ff0000000000001LL;

__device__ __forceinline__ double ld_relaxed_f64(const double* p) {
  double v;
  asm volatile("ld.relaxed.gpu.global.f64 %0, [%1];" : "=d"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_relaxed_f64(double* p, double v) {
  asm volatile("st.relaxed.gpu.global.f64 [%0], %1;" : : "l"(p), "d"(v) : "memory");
}

// Called by warp 0 of the publishing block (all 32 lanes, al and bt valid in
// lane 0): lanes 0-15 write the copies of this launch's set, lanes 16-31 empty
// the other set, lane 0 bumps the epoch.
__device__ __forceinline__ void mbox_publish(double* mbox, unsigned* epoch, unsigned e0, double al, double bt) {
  const int lane = threadIdx.x & 31;
  al = __shfl_sync(0xffffffffu, al, 0);
  bt = __shfl_sync(0xffffffffu, bt, 0);
  const bool pub = lane < kMboxCopies;
  const int set = (int)((e0 & 1u) ^ (pub ? 0u : 1u));
  double* m = mbox + (set * kMboxCopies + (lane & (kMboxCopies - 1))) * kMboxStride;
  const double empty = __longlong_as_double(kMboxEmpty);
  st_relaxed_f64(m, pub ? al : empty);
  st_relaxed_f64(m + 1, pub ? bt : empty);
  if (lane == 0) atomicAdd(epoch, 1u);
}

// Thread 0 of every block: wait (at most `limit` polls) for this launch's
// alpha and beta.  Returns false when the wait ran out.
__device__ __forceinline__ bool mbox_wait(const double* mbox, unsigned e0, unsigned limit, int backoff_ns,
                                          double* al, double* bt) {
  const double* m = mbox + ((int)(e0 & 1u) * kMboxCopies + (int)(blockIdx.x & (kMboxCopies - 1))) * kMboxStride;
  for (unsigned polls = 0;; ++polls) {
    *al = ld_relaxed_f64(m);
    *bt = ld_relaxed_f64(m + 1);
    if (__double_as_longlong(*al) != kMboxEmpty && __double_as_longlong(*bt) != kMboxEmpty) return true;
    if (polls >= limit) return false;
    __nanosleep(backoff_ns);
  }
}

struct FxStepArgs {
  int64_t n;
  const double* diag;   // null: every diagonal entry is 0
  const double* x;      // V1, unnormalised (s1 = 1 / ||V1||)
  const __int128* X;    // fixed-point copy of V1
  const double* V2;     // V2 (kHas2), unnormalised (s2 = 1 / ||V2||)
  double cF;            // c 2^-F
  const double* s1;
  const double* s2;
  int* stop;
  int step;
  double* beta;
  double* alpha;
  Tri<double>* dots;
  GridRed<Tri<double>> red;
  unsigned* epoch;      // bumped once per launch by the block that publishes alpha and beta
  double* mbox;         // kMboxDoubles entries: alpha and beta for every block
  double* Vk;
  double* nrm2;
  double* nrm;
  double* sk;
  GridRed<double> rd;
  __int128* Xk;
  int F;
  int* ovf;             // ovf[0]: an element left the fixed-point range; ovf[1]: a wait ran out
  int rows;             // rows per thread: the length of each thread's w column in shared memory
  unsigned spin_limit;  // polls before a block gives up (0: kStepSpinLimit)
  int hold_publish;     // test control: the publishing block publishes nothing, so every
                        // block's wait runs out after spin_limit polls
};

// Src supplies a row's fixed-point off-diagonal sum: bind(smem) once per
// block (every thread calls it; it may stage tables in smem and ends with a
// block barrier) returns an object whose row_sum(r) gives the row's sum.
template <class Src, bool kHas2>
__global__ void __launch_bounds__(256, 6) lz_fx_step_kernel(Src src, FxStepArgs a) {
  if (a.stop) {
    const int st = *a.stop;
    if (st != 0 && st < a.step) return;
  }
  extern __shared__ __align__(16) unsigned char fx_step_smem[];
  double* wst = reinterpret_cast<double*>(fx_step_smem);
  __shared__ unsigned e0;
  __shared__ int waited_out;
  __shared__ double ab[2];
  __shared__ double s2s;  // s2, read once (the publishing thread and the update need it)
  if (threadIdx.x == 0) {
    e0 = *reinterpret_cast<volatile unsigned*>(a.epoch);
    waited_out = 0;
    s2s = kHas2 ? *a.s2 : 0.0;
  }
  const auto& rows = src.bind(fx_step_smem + (size_t)a.rows * 256 * sizeof(double));
  __syncthreads();

  // first half: w = s1 (d x + c 2^-F sum X) and the three dots
  const double sc = *a.s1;
  Tri<double> acc = vzero(Tri<double>{});
  // row indices fit in 32 bits (the columns are int32); 32-bit indices keep
  // the loop within the 40 registers of six resident blocks per SM
  const int n = (int)a.n;
  const int stride = (int)(gridDim.x * blockDim.x);
  double* wp = wst + threadIdx.x;
  for (int r = (int)(blockIdx.x * blockDim.x + threadIdx.x); r < n; r += stride, wp += 256) {
    const __int128 s = rows.row_sum(r);
    const double xr = __ldcs(a.x + r);
    const double dx = a.diag ? __ldcs(a.diag + r) * xr : 0.0;
    const double w = sc * fma(a.cF, (double)s, dx);
    *wp = w;
    acc.b = fma(xr, w, acc.b);
    if (kHas2) {
      const double v2 = __ldcs(a.V2 + r);
      acc.a = fma(v2, w, acc.a);
      acc.c = fma(xr, v2, acc.c);
    }
  }
  // The three dots: every block posts its partial; the last to post forms the total (one
  // level, all its threads loading the partials at once), stores alpha and beta and
  // publishes them in the mailbox; every block waits for them (a bounded wait).
  Tri<double> d;
  if (grid_sum_ordered(acc, a.red, a.dots, &d) && threadIdx.x < 32) {
    double bt = 0.0, al = 0.0;
    if (threadIdx.x == 0) {
      bt = kHas2 ? s2s * d.a : 0.0;
      double t = d.b;
      if (kHas2) t = fma(-(bt * s2s), d.c, t);
      al = sc * t;
      *a.beta = bt;
      *a.alpha = al;
    }
    if (!a.hold_publish) mbox_publish(a.mbox, a.epoch, e0, al, bt);
  }
  if (threadIdx.x == 0) {
    double al, bt;
    if (!mbox_wait(a.mbox, e0, a.spin_limit ? a.spin_limit : kStepSpinLimit, 32, &al, &bt)) {
      waited_out = 1;
      atomicExch(a.ovf + 1, 1);
    }
    ab[0] = al;
    ab[1] = bt;
  }
  __syncthreads();

  // second half: v_k = (w - (beta s2) V2) - (alpha s1) V1 on the same rows
  double acc0 = 0.0;
  int out = 0;
  if (!waited_out) {
    const double al = sc * ab[0];
    const double bt = kHas2 ? s2s * ab[1] : 0.0;
    // The block's rows of pass i are 256 consecutive rows; here thread t takes
    // the adjacent pair 2 (t % 128) + {0, 1} of the passes i = t / 128 (mod 2),
    // with 16-byte loads and stores, two passes per iteration.
    const int m2 = (threadIdx.x & 127) * 2;
    const int base = (int)(blockIdx.x * blockDim.x) + m2;
    int i = threadIdx.x >> 7;
    for (; i + 2 < a.rows; i += 4) {
      const int ra = base + i * stride, rb = ra + 2 * stride;
      if (rb + 1 >= n) break;
      double2 oa = *reinterpret_cast<const double2*>(wst + i * 256 + m2);
      double2 ob = *reinterpret_cast<const double2*>(wst + (i + 2) * 256 + m2);
      const double2 qa = __ldcs(reinterpret_cast<const double2*>(a.x + ra));
      const double2 qb = __ldcs(reinterpret_cast<const double2*>(a.x + rb));
      if (kHas2) {
        const double2 pa = __ldcs(reinterpret_cast<const double2*>(a.V2 + ra));
        const double2 pb = __ldcs(reinterpret_cast<const double2*>(a.V2 + rb));
        oa = make_double2(fma(-bt, pa.x, oa.x), fma(-bt, pa.y, oa.y));
        ob = make_double2(fma(-bt, pb.x, ob.x), fma(-bt, pb.y, ob.y));
      }
      oa = make_double2(fma(-al, qa.x, oa.x), fma(-al, qa.y, oa.y));
      ob = make_double2(fma(-al, qb.x, ob.x), fma(-al, qb.y, ob.y));
      __stcs(reinterpret_cast<double2*>(a.Vk + ra), oa);
      __stcs(reinterpret_cast<double2*>(a.Vk + rb), ob);
      a.Xk[ra] = fx_from_double(oa.x, a.F, &out);
      a.Xk[ra + 1] = fx_from_double(oa.y, a.F, &out);
      a.Xk[rb] = fx_from_double(ob.x, a.F, &out);
      a.Xk[rb + 1] = fx_from_double(ob.y, a.F, &out);
      acc0 = fma(oa.x, oa.x, acc0);
      acc0 = fma(oa.y, oa.y, acc0);
      acc0 = fma(ob.x, ob.x, acc0);
      acc0 = fma(ob.y, ob.y, acc0);
    }
    for (; i < a.rows; i += 2) {
      const int r = base + i * stride;
      for (int u = 0; u < 2 && r + u < n; ++u) {
        double o = wst[i * 256 + m2 + u];
        if (kHas2) o = fma(-bt, a.V2[r + u], o);
        o = fma(-al, a.x[r + u], o);
        a.Vk[r + u] = o;
        a.Xk[r + u] = fx_from_double(o, a.F, &out);
        acc0 = fma(o, o, acc0);
      }
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

// Launch one step on `grid` blocks (the grid of the two-launch product, so
// that the dots keep their reduction tree) as a cooperative launch, which
// makes every block resident at once.  Returns false, launching nothing, when
// the w columns and the source's tables do not leave room for the whole grid
// on the device at once; the caller then runs the two-launch step.
template <class Src>
bool fx_step_launch(Ctx* ctx, const Src& src, FxStepArgs a, int grid, size_t table_smem) {
  static const int coop = [&] {  // once per process (thread-safe initialisation)
    int v = 0;
    if (cudaDeviceGetAttribute(&v, cudaDevAttrCooperativeLaunch, ctx->device) != cudaSuccess) v = 0;
    return v;
  }();
  const int64_t per = (int64_t)grid * 256;
  if (!coop || a.n <= 0 || a.n > INT32_MAX - per) return false;
  a.rows = (int)((a.n + per - 1) / per);
  const size_t smem = (size_t)a.rows * 256 * sizeof(double) + table_smem;
  if (smem > 200 * 1024) return false;
  auto kern = a.V2 ? lz_fx_step_kernel<Src, true> : lz_fx_step_kernel<Src, false>;
  if (smem > 48 * 1024) QD_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int occ = 0;
  QD_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, 256, smem));
  if ((int64_t)occ * ctx->num_sms < grid) return false;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)grid);
  cfg.blockDim = dim3(256);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = ctx->stream;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeCooperative;
  at[0].val.cooperative = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  QD_CUDA(cudaLaunchKernelEx(&cfg, kern, src, a));
  QD_LAUNCHED(ctx);
  return true;
}

}  // namespace qd
