// fxslots.cu -- the uniform-coupling product with columns computed on the fly
// (kernel code 121; the slot form is described in fxsum.cuh).
//
// Row r of the uniform-coupling form needs sum_k X[col_k] over its
// off-diagonal columns.  Code 120 reads the columns (4 bytes each, 135 MB at
// L = 24).  Here the columns come from the compiled transitions of the
// operator's terms: a row state s takes the transition of a slot whose input
// pattern it carries, and the target's rank is r plus a table value indexed
// by that pattern and the number of set bits below the support.  Nothing of
// size nnz is read; per row the kernel reads the state (4 B), the diagonal
// and x, and gathers X from L2, lane-adjacent for every slot on bits above
// the warp's low bits.  The price is integer work for every slot of every row
// (24 slots per row at L = 24 against 12.5 stored columns), so the kernel is
// bound by integer issue where code 120 is bound by gather latency.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <vector>

#include "fxstep.cuh"
#include "ham.cuh"
#include "krylov.cuh"

namespace qd {

struct FxSlotArgs {
  int64_t n;
  int nrun;
  int nslot;
  int kk;
  int ndtab;
  const uint4* runs;
  const FxSlot* slots;
  const int2* dtab;
  const uint32_t* basis;
  const double* diag;
  Rank32 R;
};

// ---------------------------------------------------------------- device
__device__ __forceinline__ uint32_t rank32(const Rank32& R, uint32_t c) {
  uint32_t col = 0;
#pragma unroll
  for (int f = 0; f < 2; ++f) {
    if (f >= R.nf) break;
    const uint32_t v = (c >> R.lo[f]) & R.wmask[f];
    const uint32_t* T = R.tab + R.off[f];
    const uint32_t kk = (uint32_t)R.k[f] + 1u;
    uint32_t a = __ldg(T + (v & 255u) * kk);
    uint32_t cb = __popc(v & 255u);
    if (R.nb[f] > 1) {
      a += __ldg(T + (256u + ((v >> 8) & 255u)) * kk + cb);
      cb += __popc((v >> 8) & 255u);
    }
    if (R.nb[f] > 2) {
      a += __ldg(T + (512u + ((v >> 16) & 255u)) * kk + cb);
      cb += __popc((v >> 16) & 255u);
    }
    if (R.nb[f] > 3) a += __ldg(T + (768u + (v >> 24)) * kk + cb);
    col += a * R.stride[f];
  }
  return col;
}

// Run slot Q on row state s: the offset of the target from the row and a 0/1
// weight (0: no transition of the slot applies; the offset is then 0).
__device__ __forceinline__ int2 run_hit(const uint4 Q, const int2* dt, int kk, uint32_t s) {
  const uint32_t pat = (s >> Q.x) & Q.y;
  return dt[(int)Q.w + (int)pat * kk + __popc(s & Q.z)];
}

// Rank slot Q on row state s: whether one of its transitions applies.
__device__ __forceinline__ bool slot_hit(const FxSlot& Q, uint32_t s) {
  const uint32_t v = s & Q.sup;
  bool hit = false;
#pragma unroll
  for (int i = 0; i < kFxSlotWidth; ++i) hit |= (v == Q.outb[i]);
  return hit;
}

// Slots and run tables into shared memory (block-wide; every thread calls).
struct SlotSmem {
  const uint4* runs;
  const FxSlot* slots;
  const int2* dt;
};
__device__ __forceinline__ SlotSmem stage_slots(const FxSlotArgs& A, unsigned char* fxs_smem) {
  uint4* runs = reinterpret_cast<uint4*>(fxs_smem);
  FxSlot* slots = reinterpret_cast<FxSlot*>(fxs_smem + (size_t)A.nrun * sizeof(uint4));
  int2* dt = reinterpret_cast<int2*>(fxs_smem + (size_t)A.nrun * sizeof(uint4) + (size_t)A.nslot * sizeof(FxSlot));
  for (int i = threadIdx.x; i < A.nrun; i += blockDim.x) runs[i] = A.runs[i];
  const int nw = A.nslot * (int)(sizeof(FxSlot) / sizeof(uint32_t));
  for (int i = threadIdx.x; i < nw; i += blockDim.x)
    reinterpret_cast<uint32_t*>(slots)[i] = reinterpret_cast<const uint32_t*>(A.slots)[i];
  for (int i = threadIdx.x; i < A.ndtab; i += blockDim.x) dt[i] = A.dtab[i];
  __syncthreads();
  return SlotSmem{runs, slots, dt};
}

__device__ __forceinline__ SlotSmem stage_slots(const FxSlotArgs& A) {
  extern __shared__ __align__(16) unsigned char fxs_dyn_smem[];
  return stage_slots(A, fxs_dyn_smem);
}

// Off-diagonal fixed-point sum of row r: the slots four at a time, four
// predicated gathers in flight before their adds.
__device__ __forceinline__ __int128 slot_sum(const FxSlotArgs& A, const SlotSmem& S, const __int128* __restrict__ X,
                                             uint32_t s, int r) {
  __int128 sum = 0;
  const __int128* Xr = X + r;
  for (int g = 0; g < A.nrun; g += 4) {
    const int2 h0 = run_hit(S.runs[g], S.dt, A.kk, s), h1 = run_hit(S.runs[g + 1], S.dt, A.kk, s),
               h2 = run_hit(S.runs[g + 2], S.dt, A.kk, s), h3 = run_hit(S.runs[g + 3], S.dt, A.kk, s);
    __int128 t0 = 0, t1 = 0, t2 = 0, t3 = 0;
    if (h0.y) t0 = Xr[h0.x];
    if (h1.y) t1 = Xr[h1.x];
    if (h2.y) t2 = Xr[h2.x];
    if (h3.y) t3 = Xr[h3.x];
    sum += (t0 + t1) + (t2 + t3);
  }
  for (int g = 0; g < A.nslot; ++g) {
    const FxSlot& Q = S.slots[g];
    if (slot_hit(Q, s)) sum += X[rank32(A.R, s ^ Q.flip)];
  }
  return sum;
}

__device__ __forceinline__ bool check_col(int c, int b, int e, const int32_t* colidx, uint32_t* seen) {
  int pos = -1;
  for (int k = b; k < e; ++k)
    if (colidx[k] == c) {
      pos = k - b;
      break;
    }
  if (pos < 0 || ((seen[pos >> 5] >> (pos & 31)) & 1u)) return false;
  seen[pos >> 5] |= 1u << (pos & 31);
  return true;
}

__global__ void __launch_bounds__(256) fx_slots_check_kernel(FxSlotArgs A, const int32_t* rowptr,
                                                             const int32_t* colidx, int* bad) {
  const SlotSmem S = stage_slots(A);
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < A.n; r += (int64_t)gridDim.x * blockDim.x) {
    const uint32_t s = A.basis[r];
    const int b = rowptr[r], e = rowptr[r + 1];
    uint32_t seen[4] = {0u, 0u, 0u, 0u};
    int cnt = 0;
    bool ok = (e - b) <= 128;
    for (int g = 0; g < A.nrun && ok; ++g) {
      const int2 h = run_hit(S.runs[g], S.dt, A.kk, s);
      if (!h.y) continue;
      ++cnt;
      ok = check_col((int)r + h.x, b, e, colidx, seen);
    }
    for (int g = 0; g < A.nslot && ok; ++g) {
      if (!slot_hit(S.slots[g], s)) continue;
      ++cnt;
      ok = check_col((int)rank32(A.R, s ^ S.slots[g].flip), b, e, colidx, seen);
    }
    if (!ok || cnt != e - b) atomicOr(bad, 1);
  }
}

__global__ void basis32_kernel(int64_t n, const uint64_t* basis, uint32_t* out) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = (uint32_t)basis[i];
}

// y = s (d x + c 2^-F sum X): the plain product (scale from the device, or 1).
__global__ void __launch_bounds__(256) spmv_fx_slots_kernel(FxSlotArgs A, const double* __restrict__ x,
                                                            const __int128* __restrict__ X, double* __restrict__ y,
                                                            double cF, const double* scale_dev, const int* stop,
                                                            int step) {
  if (stop) {
    const int st = *stop;
    if (st != 0 && st < step) return;
  }
  const SlotSmem S = stage_slots(A);
  const double sc = scale_dev ? *scale_dev : 1.0;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < A.n; r += stride) {
    const __int128 sum = slot_sum(A, S, X, __ldcs(A.basis + r), (int)r);
    y[r] = sc * fma(cF, (double)sum, __ldcs(A.diag + r) * __ldg(x + r));
  }
}

// The product fused with the Lanczos step's three inner products, exactly as
// spmv_fx_dots_kernel forms them (same grid, same per-thread row order, same
// reduction tree), so code 121 and code 120 give bit-identical recurrences.
template <bool kHas2>
__global__ void __launch_bounds__(256, 6) spmv_fx_slots_dots_kernel(
    FxSlotArgs A, const double* __restrict__ x, const __int128* __restrict__ X, const double* __restrict__ V2,
    double* __restrict__ y, double cF, const double* s1, const double* s2, const int* stop, int step, double* beta,
    double* alpha, Tri<double>* dots, GridRed<Tri<double>> red) {
  if (stop) {
    const int st = *stop;
    if (st != 0 && st < step) return;
  }
  const SlotSmem S = stage_slots(A);
  const double sc = *s1;
  Tri<double> acc = vzero(Tri<double>{});
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < A.n; r += stride) {
    const __int128 sum = slot_sum(A, S, X, __ldcs(A.basis + r), (int)r);
    const double xr = __ldcs(x + r);
    const double w = sc * fma(cF, (double)sum, __ldcs(A.diag + r) * xr);
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

// ---------------------------------------------------------------- host
static FxSlotArgs slot_args(const qd_ham* H, const FxForm& f) {
  FxSlotArgs A;
  std::memset(&A, 0, sizeof(A));
  A.n = H->dim;
  A.nrun = f.nrun;
  A.nslot = f.nslot;
  A.kk = f.kk;
  A.ndtab = f.ndtab;
  A.runs = f.runs.p;
  A.slots = f.slots.p;
  A.dtab = f.dtab.p;
  A.basis = f.basis32.p;
  A.diag = f.diag.p;
  A.R = f.rank;
  return A;
}

static size_t slot_smem(const FxForm& f) {
  return (size_t)f.nrun * sizeof(uint4) + (size_t)f.nslot * sizeof(FxSlot) + (size_t)f.ndtab * sizeof(int2);
}
constexpr size_t kSlotSmemMax = 40 * 1024;

static int slot_grid(Ctx* ctx, int64_t n) {
  return (int)std::max<int64_t>(1, std::min<int64_t>(ceil_div(n, 256), (int64_t)ctx->num_sms * 8));
}

// Colex share of the set bits of a window pattern w whose lowest bit sits at
// field position a, with m set bits of the field below it.
static int64_t window_rank(uint32_t w, int a, int m, const int64_t (*C)[65]) {
  int64_t r = 0;
  int t = 0;
  for (int p = 0; p < 32; ++p)
    if ((w >> p) & 1u) {
      ++t;
      const int n = a + p, k = m + t;
      if (k <= n) r += C[n][k];
    }
  return r;
}

// Slots, tables, the 32-bit basis and (when rank slots exist, or `tables`)
// the byte tables of the form f for the transitions of value c; false when
// the operator's terms do not give this form.
static bool make_slots(qd_ham* H, FxForm& f, double c, bool tables) {
  const SectorView& V = H->sec->view;
  if (!H->from_terms || V.rank_kind != 1 || V.nbits > 32 || H->dim >= (1ll << 31)) return false;
  if (V.nfields < 1 || V.nfields > 2) return false;
  uint32_t fmask[2] = {0u, 0u};
  int kk = 1;
  for (int i = 0; i < V.nfields; ++i) {
    const Field& F = V.fields[i];
    if (F.is_free || F.width < 1 || F.lo + F.width > 32) return false;
    fmask[i] = (uint32_t)((((uint64_t)1 << F.width) - 1) << F.lo);
    kk = std::max(kk, F.k + 1);
  }
  std::vector<MfEntry> off, dia;
  try {
    compile_terms(H, off, dia);
  } catch (const Error&) {  // terms the compiled form does not take: keep the stored columns
    clear_error();
    return false;
  }
  // Transitions of value c with no sign string whose target stays in the
  // sector, into run slots (contiguous support inside one field) and rank
  // slots (everything else).
  struct Run {
    uint32_t sup;
    int field, lo, w;
    std::vector<int64_t> flip;  // per input pattern: flip on the run, or -1
  };
  struct Grp {
    uint32_t sup, flip;
    std::vector<uint32_t> outb;
  };
  std::vector<Run> runs;
  std::vector<Grp> groups;
  for (const MfEntry& e : off) {
    if (e.amp.im != 0.0 || e.jw != 0) return false;
    if (e.amp.re == 0.0) continue;  // an explicit zero is no column of the uniform form
    if (e.amp.re != c) return false;
    const uint32_t sup = (uint32_t)e.sup, outb = (uint32_t)e.outb, flip = (uint32_t)e.flip;
    bool in = true;
    for (int i = 0; i < V.nfields; ++i)
      in &= __builtin_popcount(outb & fmask[i]) == __builtin_popcount((outb ^ flip) & fmask[i]);
    if (!in) continue;  // the target leaves the sector: the lowering drops it
    int fi = -1;
    for (int i = 0; i < V.nfields; ++i)
      if ((sup & ~fmask[i]) == 0u) fi = i;
    const int lo = __builtin_ctz(sup), hi = 31 - __builtin_clz(sup);
    if (fi >= 0 && __builtin_popcount(sup) == hi - lo + 1) {
      const int w = hi - lo + 1;
      const uint32_t pat = (outb >> lo) & ((1u << w) - 1u), fl = (flip >> lo) & ((1u << w) - 1u);
      Run* slot = nullptr;
      for (Run& q : runs) {
        if (q.sup != sup) continue;
        if (q.flip[pat] == (int64_t)fl) return false;  // the same transition twice: the column would take 2c
        if (q.flip[pat] < 0 && !slot) slot = &q;
      }
      if (!slot) {
        runs.push_back(Run{sup, fi, lo, w, std::vector<int64_t>((size_t)1 << w, -1)});
        slot = &runs.back();
      }
      slot->flip[pat] = fl;
      continue;
    }
    Grp* g = nullptr;
    for (Grp& q : groups)
      if (q.sup == sup && q.flip == flip && q.outb.size() < (size_t)kFxSlotWidth) g = &q;
    for (const Grp& q : groups)
      if (q.sup == sup && q.flip == flip)
        for (uint32_t o : q.outb)
          if (o == outb) return false;
    if (!g) {
      groups.push_back(Grp{sup, flip, {}});
      g = &groups.back();
    }
    g->outb.push_back(outb);
  }
  if (runs.empty() && groups.empty()) return false;  // a diagonal operator: nothing to gather
  int64_t C[65][65];
  for (int n = 0; n < 65; ++n)
    for (int k = 0; k < 65; ++k) C[n][k] = (k == 0) ? 1 : (n == 0 ? 0 : C[n - 1][k - 1] + C[n - 1][k]);
  std::vector<uint4> hruns;
  std::vector<int2> dtab;
  for (const Run& q : runs) {
    const Field& F = V.fields[q.field];
    const int a = q.lo - F.lo;
    uint4 d;
    d.x = (uint32_t)q.lo;
    d.y = (1u << q.w) - 1u;
    d.z = fmask[q.field] & (uint32_t)(((uint64_t)1 << q.lo) - 1);
    d.w = (uint32_t)dtab.size();
    for (uint32_t p = 0; p < (1u << q.w); ++p)
      for (int m = 0; m < kk; ++m) {
        int2 v = make_int2(0, 0);  // no transition: weight 0
        if (q.flip[p] >= 0 && m + __builtin_popcount(p) <= F.k) {
          const uint32_t wc = p ^ (uint32_t)q.flip[p];
          const int64_t dl = (window_rank(wc, a, m, C) - window_rank(p, a, m, C)) * F.stride;
          if (dl <= -(1ll << 31) || dl >= (1ll << 31)) return false;
          v = make_int2((int32_t)dl, 1);
        }
        dtab.push_back(v);
      }
    hruns.push_back(d);
  }
  if (hruns.size() % 4) {  // padding run slots: mask 0, so pattern 0, whose table row has weight 0
    uint4 d;
    d.x = 0u;
    d.y = 0u;
    d.z = 0u;
    d.w = (uint32_t)dtab.size();
    dtab.insert(dtab.end(), (size_t)kk, make_int2(0, 0));
    while (hruns.size() % 4) hruns.push_back(d);
  }
  std::vector<FxSlot> slots;
  for (const Grp& g : groups) {
    FxSlot Q;
    std::memset(&Q, 0, sizeof(Q));
    Q.sup = g.sup;
    Q.flip = g.flip;
    for (int j = 0; j < kFxSlotWidth; ++j) Q.outb[j] = (j < (int)g.outb.size()) ? g.outb[j] : ~g.sup;
    slots.push_back(Q);
  }
  while (slots.size() % 4) {  // padding rank slots: sup 0 never matches outb ~0
    FxSlot Q;
    std::memset(&Q, 0, sizeof(Q));
    for (int j = 0; j < kFxSlotWidth; ++j) Q.outb[j] = ~0u;
    slots.push_back(Q);
  }
  f.nrun = (int)hruns.size();
  f.nslot = (int)slots.size();
  f.kk = kk;
  f.ndtab = (int)dtab.size();
  if (slot_smem(f) > kSlotSmemMax) return false;
  Ctx* ctx = H->ctx;
  const int64_t n = H->dim;
  f.runs.alloc(std::max<size_t>(hruns.size(), 1));
  f.slots.alloc(std::max<size_t>(slots.size(), 1));
  f.dtab.alloc(std::max<size_t>(dtab.size(), 1));
  if (!hruns.empty())
    QD_CUDA(cudaMemcpyAsync(f.runs.p, hruns.data(), hruns.size() * sizeof(uint4), cudaMemcpyHostToDevice,
                            ctx->stream));
  if (!slots.empty())
    QD_CUDA(cudaMemcpyAsync(f.slots.p, slots.data(), slots.size() * sizeof(FxSlot), cudaMemcpyHostToDevice,
                            ctx->stream));
  if (!dtab.empty())
    QD_CUDA(cudaMemcpyAsync(f.dtab.p, dtab.data(), dtab.size() * sizeof(int2), cudaMemcpyHostToDevice,
                            ctx->stream));
  std::memset(&f.rank, 0, sizeof(f.rank));
  if (!groups.empty() || tables) {
    MfRank rk;
    std::memset(&rk, 0, sizeof(rk));
    std::vector<int64_t> tab;
    build_tables(H->sec, rk, tab);
    std::vector<uint32_t> t32(std::max<size_t>(tab.size(), 1), 0u);
    for (size_t i = 0; i < tab.size(); ++i) t32[i] = (uint32_t)tab[i];
    f.rtab.alloc(t32.size());
    QD_CUDA(cudaMemcpyAsync(f.rtab.p, t32.data(), t32.size() * 4, cudaMemcpyHostToDevice, ctx->stream));
    QD_CUDA(cudaStreamSynchronize(ctx->stream));  // t32 is a host temporary
    f.rank.nf = V.nfields;
    for (int i = 0; i < V.nfields; ++i) {
      const Field& F = V.fields[i];
      f.rank.lo[i] = F.lo;
      f.rank.k[i] = F.k;
      f.rank.nb[i] = rk.nb[i];
      f.rank.wmask[i] = (F.width >= 32) ? 0xffffffffu : ((1u << F.width) - 1u);
      f.rank.stride[i] = (uint32_t)F.stride;
      f.rank.off[i] = (int)rk.off[i];
    }
    f.rank.tab = f.rtab.p;
  }
  f.basis32.alloc(n);
  basis32_kernel<<<slot_grid(ctx, n), 256, 0, ctx->stream>>>(n, H->sec->basis.p, f.basis32.p);
  QD_CHECK_LAUNCH();
  QD_LAUNCHED(ctx);
  QD_CUDA(cudaStreamSynchronize(ctx->stream));
  return true;
}

static void drop_slots(FxForm& f) {
  f.runs.release();
  f.slots.release();
  f.dtab.release();
  f.basis32.release();
  f.rtab.release();
  f.nrun = f.nslot = f.ndtab = 0;
}

bool ham_build_fx_slots(qd_ham* H) {
  FxForm& f = *H->fx;
  if (f.slots_state != 0) return f.slots_state > 0;
  f.slots_state = -1;
  if (!make_slots(H, f, f.c, false)) {
    drop_slots(f);
    return false;
  }
  Ctx* ctx = H->ctx;
  const int64_t n = H->dim;
  DBuf<int> bad(1);
  QD_CUDA(cudaMemsetAsync(bad.p, 0, sizeof(int), ctx->stream));
  const FxSlotArgs A = slot_args(H, f);
  fx_slots_check_kernel<<<slot_grid(ctx, n), 256, slot_smem(f), ctx->stream>>>(A, f.rowptr.p, f.colidx.p, bad.p);
  QD_CHECK_LAUNCH();
  QD_LAUNCHED(ctx);
  int hb = 1;
  QD_CUDA(cudaMemcpyAsync(&hb, bad.p, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  QD_CUDA(cudaStreamSynchronize(ctx->stream));
  if (hb) {
    drop_slots(f);
    return false;
  }
  f.slots_state = 1;
  return true;
}

// ---------------------------------------------------------------- the form without a stored matrix
// Per row: every column in range, none twice, at most 128; the row bound
// |c| + ... + |c| (one per column, added in turn) + |d_r|, as the stored-matrix
// form sums its values, so both give the same scale F.
__global__ void __launch_bounds__(256) fx_slots_rows_kernel(FxSlotArgs A, double absc, int* bad,
                                                            unsigned long long* rowmax) {
  const SlotSmem S = stage_slots(A);
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < A.n; r += (int64_t)gridDim.x * blockDim.x) {
    const uint32_t s = A.basis[r];
    int cols[128];
    int cnt = 0;
    bool ok = true;
    auto take = [&](int c) {
      if (c < 0 || (int64_t)c >= A.n || cnt >= 128) {
        ok = false;
        return;
      }
      for (int i = 0; i < cnt; ++i) ok &= (cols[i] != c);
      cols[cnt++] = c;
    };
    for (int g = 0; g < A.nrun && ok; ++g) {
      const int2 h = run_hit(S.runs[g], S.dt, A.kk, s);
      if (h.y) take((int)r + h.x);
    }
    for (int g = 0; g < A.nslot && ok; ++g)
      if (slot_hit(S.slots[g], s)) take((int)rank32(A.R, s ^ S.slots[g].flip));
    if (!ok) atomicOr(bad, 1);
    double sum = 0.0;
    for (int i = 0; i < cnt; ++i) sum += absc;
    sum += fabs(A.diag[r]);
    atomicMax(rowmax, (unsigned long long)__double_as_longlong(sum));
  }
}

// Colex rank of a field value (the sector's rank of one field), for the host check.
static int64_t host_colex(uint32_t v, const int64_t (*C)[65]) {
  int64_t r = 0;
  int j = 0;
  for (int p = 0; p < 32; ++p)
    if ((v >> p) & 1u) {
      ++j;
      if (j <= p) r += C[p][j];
    }
  return r;
}

// The run tables against whole-field ranks: for every pattern with a
// transition and every count m of set bits below the run that a state of the
// field can have, two states (the remaining set bits just above the run, or
// at the top of the field) must both move by the tabulated offset.
static bool check_run_tables(const qd_ham* H, const FxForm& f, const std::vector<uint4>& runs,
                             const std::vector<int2>& dtab, const std::vector<std::vector<int64_t>>& flips) {
  const SectorView& V = H->sec->view;
  int64_t C[65][65];
  for (int n = 0; n < 65; ++n)
    for (int k = 0; k < 65; ++k) C[n][k] = (k == 0) ? 1 : (n == 0 ? 0 : C[n - 1][k - 1] + C[n - 1][k]);
  for (size_t q = 0; q < runs.size() && q < flips.size(); ++q) {
    const uint4 R = runs[q];
    int fi = -1;
    for (int i = 0; i < V.nfields; ++i)
      if ((int)R.x >= V.fields[i].lo && (int)R.x < V.fields[i].lo + V.fields[i].width) fi = i;
    if (fi < 0) return false;
    const Field& F = V.fields[fi];
    const int a = (int)R.x - F.lo, w = __builtin_popcount(R.y), above = F.width - a - w;
    for (uint32_t p = 0; p <= R.y; ++p) {
      if (flips[q][p] < 0) continue;
      for (int m = 0; m <= a; ++m) {
        const int rest = F.k - m - __builtin_popcount(p);
        if (rest < 0 || rest > above) continue;
        const int2 d = dtab[R.w + p * f.kk + m];
        if (!d.y) return false;
        for (int place = 0; place < 2; ++place) {
          uint32_t v = (m ? ((1u << m) - 1u) : 0u) | (p << a);
          for (int i = 0; i < rest; ++i) v |= 1u << (place ? (F.width - 1 - i) : (a + w + i));
          const uint32_t vc = v ^ ((uint32_t)flips[q][p] << a);
          const int64_t dl = (host_colex(vc, C) - host_colex(v, C)) * F.stride;
          if (dl != (int64_t)d.x) return false;
        }
      }
    }
  }
  return true;
}

bool ham_build_mf_fx(qd_ham* H) {
  if (H->mfx_state != 0) return H->mfx_state > 0;
  H->mfx_state = -1;
  if (!H->from_terms || !(H->flags & QD_HAM_REAL) || H->dim < 1) return false;
  ham_build_matrix_free(H);
  if (!H->mf_real) return false;
  std::vector<MfEntry> off, dia;
  compile_terms(H, off, dia);
  double c = 0.0;
  for (const MfEntry& e : off)
    if (e.amp.re != 0.0 || e.amp.im != 0.0) {
      c = e.amp.re;
      break;
    }
  if (c == 0.0) return false;
  std::unique_ptr<FxForm> f(new FxForm());
  f->c = c;
  if (!make_slots(H, *f, c, true)) return false;
  // the run tables, checked on the host against whole-field ranks
  {
    std::vector<uint4> runs((size_t)f->nrun);
    std::vector<int2> dtab((size_t)f->ndtab);
    QD_CUDA(cudaMemcpyAsync(runs.data(), f->runs.p, runs.size() * sizeof(uint4), cudaMemcpyDeviceToHost,
                            H->ctx->stream));
    QD_CUDA(cudaMemcpyAsync(dtab.data(), f->dtab.p, dtab.size() * sizeof(int2), cudaMemcpyDeviceToHost,
                            H->ctx->stream));
    QD_CUDA(cudaStreamSynchronize(H->ctx->stream));
    std::vector<std::vector<int64_t>> flips(runs.size());
    for (size_t q = 0; q < runs.size(); ++q) flips[q].assign((size_t)runs[q].y + 1, -1);
    // recover each run slot's flips from its entries: a pattern with weight 1 took one transition
    std::vector<int> seen(runs.size(), 0);
    const SectorView& V = H->sec->view;
    for (const MfEntry& e : off) {
      if (e.amp.re != c || e.amp.im != 0.0) continue;
      bool in = true;  // make_slots keeps only transitions that stay in the sector
      for (int i = 0; i < V.nfields; ++i) {
        const uint32_t fm = (uint32_t)((((uint64_t)1 << V.fields[i].width) - 1) << V.fields[i].lo);
        in &= __builtin_popcount((uint32_t)e.outb & fm) == __builtin_popcount((uint32_t)(e.outb ^ e.flip) & fm);
      }
      if (!in) continue;
      const uint32_t sup = (uint32_t)e.sup;
      const int lo = __builtin_ctz(sup);
      for (size_t q = 0; q < runs.size(); ++q) {
        if ((int)runs[q].x != lo || (runs[q].y << lo) != sup) continue;
        const uint32_t pat = ((uint32_t)e.outb >> lo) & runs[q].y;
        if (flips[q][pat] >= 0) continue;  // a later slot of the same support holds it
        flips[q][pat] = ((uint32_t)e.flip >> lo) & runs[q].y;
        break;
      }
    }
    if (!check_run_tables(H, *f, runs, dtab, flips)) return false;
  }
  Ctx* ctx = H->ctx;
  const int64_t n = H->dim;
  f->diag.alloc(n);
  QD_CUDA(cudaMemcpyAsync(f->diag.p, H->diag_r.p, n * sizeof(double), cudaMemcpyDeviceToDevice, ctx->stream));
  DBuf<int> bad(1);
  DBuf<unsigned long long> rowmax(1);
  QD_CUDA(cudaMemsetAsync(bad.p, 0, sizeof(int), ctx->stream));
  QD_CUDA(cudaMemsetAsync(rowmax.p, 0, sizeof(unsigned long long), ctx->stream));
  fx_slots_rows_kernel<<<slot_grid(ctx, n), 256, slot_smem(*f), ctx->stream>>>(slot_args(H, *f), std::fabs(c),
                                                                              bad.p, rowmax.p);
  QD_CHECK_LAUNCH();
  QD_LAUNCHED(ctx);
  int hb = 1;
  unsigned long long rb = 0;
  QD_CUDA(cudaMemcpyAsync(&hb, bad.p, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  QD_CUDA(cudaMemcpyAsync(&rb, rowmax.p, sizeof(rb), cudaMemcpyDeviceToHost, ctx->stream));
  QD_CUDA(cudaStreamSynchronize(ctx->stream));
  double rm = 0.0;
  std::memcpy(&rm, &rb, 8);
  if (hb || !std::isfinite(rm)) return false;
  const int eb = (int)std::ceil(std::log2(std::max(1.0, rm))) + 1;  // as ham_build_fx
  f->F = 119 - eb;
  f->nnz = 0;
  f->use_slots = true;
  f->slots_state = 1;
  H->mfx = std::move(f);
  H->mfx_state = 1;
  // the block layout, where the sector gives it, replaces the slots (faster one-launch step, the
  // same bits); QD_MF_BLOCK=0 keeps the slots
  const char* e = std::getenv("QD_MF_BLOCK");
  if (!(e && std::strcmp(e, "0") == 0) && ham_build_mf_fx_block(H)) H->mfx->use_blk = true;
  return true;
}

void launch_fx_slots(Ctx* ctx, const qd_ham* H, const FxForm& f, const double* x, const __int128* X, double* y,
                     const double* scale_dev, const int* stop, int step) {
  const double cF = std::ldexp(f.c, -f.F);
  spmv_fx_slots_kernel<<<slot_grid(ctx, H->dim), 256, slot_smem(f), ctx->stream>>>(slot_args(H, f), x, X, y, cF,
                                                                                    scale_dev, stop, step);
  QD_CHECK_LAUNCH();
  QD_LAUNCHED(ctx);
}

// Rows of the slot form for the one-launch step (fxstep.cuh): the tables go
// into shared memory after the w columns.
struct SlotRowsBound {
  FxSlotArgs A;
  SlotSmem S;
  const __int128* X;
  __device__ __int128 row_sum(int64_t r) const { return slot_sum(A, S, X, __ldcs(A.basis + r), (int)r); }
};
struct SlotRows {
  FxSlotArgs A;
  const __int128* X;
  __device__ SlotRowsBound bind(unsigned char* smem) const { return SlotRowsBound{A, stage_slots(A, smem), X}; }
};

bool launch_fx_slots_step(Ctx* ctx, const qd_ham* H, const FxForm& f, const FxStepArgs& a, int grid) {
  return fx_step_launch(ctx, SlotRows{slot_args(H, f), a.X}, a, grid, slot_smem(f));
}

void launch_fx_slots_dots(Ctx* ctx, const qd_ham* H, const FxForm& f, const double* x, const __int128* X,
                          const double* V2, double* y, const double* s1, const double* s2, const int* stop, int step,
                          double* beta, double* alpha, Tri<double>* dots, GridRed<Tri<double>> red, int grid) {
  const double cF = std::ldexp(f.c, -f.F);
  const size_t sm = slot_smem(f);
  if (V2)
    spmv_fx_slots_dots_kernel<true><<<grid, 256, sm, ctx->stream>>>(slot_args(H, f), x, X, V2, y, cF, s1, s2, stop,
                                                                    step, beta, alpha, dots, red);
  else
    spmv_fx_slots_dots_kernel<false><<<grid, 256, sm, ctx->stream>>>(slot_args(H, f), x, X, x, y, cF, s1, s1, stop,
                                                                     step, beta, alpha, dots, red);
  QD_CHECK_LAUNCH();
  QD_LAUNCHED(ctx);
}

}  // namespace qd
