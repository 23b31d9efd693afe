// lower.cu -- `OperatorSum >> index` on the device.
//
// Restates Operator::full_branch / operator>> (operator.hpp:135-267),
// bitOp::branch (operators/bit.hpp:49-85), hopBitOp::branch
// (operators/hopbit.hpp:43-84) and OperatorSum::operator>>
// (operator_abel.hpp:25-34).  One thread per sector column (input state):
//   for each term t, in order:
//     walk every leaf of the gate tree (gates applied last to first; leaf
//     order is lexicographic with the first-applied bit gate most
//     significant, the breadth-first order of full_branch);
//     drop null leaves, leaves with |value| <= 1e-10 and leaves outside
//     the sector; sum leaves that land on the same row in leaf order
//     (setFromTriplets);
//     add coeff_t * M_t into the column's union pattern (Eigen's sparse sum:
//     an entry first seen is 0 + p, a cancellation leaves an explicit zero).
// Every product and sum is one IEEE rounding (no FMA), as in the reference.
// Pass 0 counts entries per column, an exclusive scan gives the CSC column
// pointers, pass 1 writes rows (sorted) and values.  The CSC result is then
// transposed into the CSR compute layout.
#include <algorithm>
#include <cstdlib>
#include <cstring>

#include "ham.cuh"
#include "scan.cuh"

namespace qd {

struct LowerParams {
  SectorView S;
  const TermDev* terms;
  const GateDev* gates;
  int nterms;
  int pad;
};

__device__ __forceinline__ bool leaf_path(const LowerParams& P, const TermDev& T, uint64_t s, int j,
                                          uint64_t& st_out, cplx& v_out) {
  uint64_t st = s;
  cplx v = mkc(1.0, 0.0);
  int bp = T.nbit - 1;
  bool valid = true;
  for (int ig = T.ngates - 1; ig >= 0; --ig) {
    const GateDev& G = P.gates[T.gate_offset + ig];
    if (G.kind == QD_GATE_BIT) {
      const int o = (j >> bp) & 1;
      --bp;
      if (!valid) continue;
      const int b = (int)((st >> G.site) & 1ull);
      const uint64_t above = (G.site + 1 >= 64) ? 0ull : (st >> (G.site + 1));
      const cplx jw = (__popcll(above) & 1) ? mkc((double)G.string, 0.0) : mkc(1.0, 0.0);
      v = cmul_rn(cmul_rn(jw, G.u[b * 2 + o]), v);
      const uint64_t bit = 1ull << G.site;
      st = o ? (st | bit) : (st & ~bit);
    } else {
      if (!valid) continue;
      const int sa = G.site, sb = G.site_b;
      if (sa == sb) {
        const double occ = (double)((st >> sb) & 1ull);
        v = rmul_rn(occ, v);
      } else if (((st >> sb) & 1ull) && !((st >> sa) & 1ull)) {
        const int jw1 = __popcll((sb + 1 >= 64) ? 0ull : (st >> (sb + 1)));
        st &= ~(1ull << sb);
        const int jw2 = __popcll((sa + 1 >= 64) ? 0ull : (st >> (sa + 1)));
        st |= (1ull << sa);
        const int jw = ((jw1 & 1) ? G.string : 1) * ((jw2 & 1) ? G.string : 1);
        v = cmul_rn(mkc((double)jw, 0.0), v);
      } else {
        valid = false;
      }
    }
  }
  st_out = st;
  v_out = v;
  return valid;
}

template <int CAP, int TCAP>
__global__ void __launch_bounds__(128) lower_kernel(LowerParams P, int pass, int64_t* counts,
                                                    const int64_t* colptr, int32_t* rowidx, cplx* vals,
                                                    int* overflow) {
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= P.S.dim) return;
  const uint64_t s = P.S.basis[c];
  int n = 0;
  int rows[CAP];
  cplx acc[CAP];
  int trow[TCAP];
  cplx tval[TCAP];
  for (int t = 0; t < P.nterms; ++t) {
    const TermDev T = P.terms[t];
    const int nleaves = 1 << T.nbit;
    int tn = 0;
    for (int j = 0; j < nleaves; ++j) {
      uint64_t st;
      cplx v;
      if (!leaf_path(P, T, s, j, st, v)) continue;
      if (!(hypot(v.re, v.im) > 1e-10)) continue;  // operator.hpp:255
      const int64_t r = sector_rank(P.S, st);
      if (r >= P.S.dim) continue;  // outside the sector (operator.hpp:196-199)
      int k = 0;
      while (k < tn && trow[k] != (int)r) ++k;
      if (k < tn) {
        tval[k] = cadd_rn(tval[k], v);
      } else {
        if (tn >= TCAP) {
          atomicExch(overflow, 1);
          return;
        }
        trow[tn] = (int)r;
        tval[tn] = v;
        ++tn;
      }
    }
    for (int k = 0; k < tn; ++k) {
      const cplx p = cmul_rn(T.coeff, tval[k]);
      const int r = trow[k];
      int lo = 0, hi = n;
      while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (rows[mid] < r) lo = mid + 1;
        else hi = mid;
      }
      if (lo < n && rows[lo] == r) {
        acc[lo] = cadd_rn(acc[lo], p);
      } else {
        if (n >= CAP) {
          atomicExch(overflow, 1);
          return;
        }
        for (int q = n; q > lo; --q) {
          rows[q] = rows[q - 1];
          acc[q] = acc[q - 1];
        }
        rows[lo] = r;
        acc[lo] = cadd_rn(mkc(0.0, 0.0), p);
        ++n;
      }
    }
  }
  if (pass == 0) {
    counts[c] = n;
  } else {
    const int64_t base = colptr[c];
    for (int k = 0; k < n; ++k) {
      rowidx[base + k] = rows[k];
      vals[base + k] = acc[k];
    }
  }
}

// ---------------------------------------------------------------- transpose
__global__ void histogram_kernel(const int32_t* idx, int64_t nnz, unsigned long long* counts) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k < nnz) atomicAdd(counts + idx[k], 1ull);
}

__global__ void scatter_kernel(int64_t n, const int64_t* ptr, const int32_t* idx, const cplx* vals,
                               const int64_t* out_ptr, unsigned long long* cursor, int32_t* out_idx,
                               cplx* out_vals) {
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n) return;
  for (int64_t k = ptr[c]; k < ptr[c + 1]; ++k) {
    const int32_t r = idx[k];
    const int64_t pos = out_ptr[r] + (int64_t)atomicAdd(cursor + r, 1ull);
    out_idx[pos] = (int32_t)c;
    out_vals[pos] = vals[k];
  }
}

__global__ void sort_segments_kernel(int64_t n, const int64_t* ptr, int32_t* idx, cplx* vals) {
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  const int64_t b = ptr[r], e = ptr[r + 1];
  for (int64_t i = b + 1; i < e; ++i) {
    const int32_t key = idx[i];
    const cplx v = vals[i];
    int64_t j = i - 1;
    while (j >= b && idx[j] > key) {
      idx[j + 1] = idx[j];
      vals[j + 1] = vals[j];
      --j;
    }
    idx[j + 1] = key;
    vals[j + 1] = v;
  }
}

void ham_transpose(Ctx* ctx, int64_t n, const int64_t* ptr, const int32_t* idx, const cplx* vals, int64_t nnz,
                   int64_t* out_ptr, int32_t* out_idx, cplx* out_vals) {
  DBuf<unsigned long long> counts(n + 1);
  QD_CUDA(cudaMemsetAsync(counts.p, 0, (n + 1) * 8, ctx->stream));
  if (nnz > 0) {
    histogram_kernel<<<(unsigned)ceil_div(nnz, 256), 256, 0, ctx->stream>>>(idx, nnz, counts.p);
    QD_CHECK_LAUNCH();
    QD_LAUNCHED(ctx);
  }
  exclusive_scan_i64(ctx, (const int64_t*)counts.p, out_ptr, n + 1);
  QD_CUDA(cudaMemsetAsync(counts.p, 0, (n + 1) * 8, ctx->stream));
  if (n > 0) {
    scatter_kernel<<<(unsigned)ceil_div(n, 256), 256, 0, ctx->stream>>>(n, ptr, idx, vals, out_ptr, counts.p,
                                                                         out_idx, out_vals);
    QD_CHECK_LAUNCH();
    QD_LAUNCHED(ctx);
    sort_segments_kernel<<<(unsigned)ceil_div(n, 256), 256, 0, ctx->stream>>>(n, out_ptr, out_idx, out_vals);
    QD_CHECK_LAUNCH();
    QD_LAUNCHED(ctx);
  }
  QD_CUDA(cudaStreamSynchronize(ctx->stream));
}

// ---------------------------------------------------------------- analysis
// flags[0]: some imaginary part != 0; flags[1]: H != H^dagger; flags[2]: max row nnz
__global__ void analyze_kernel(int64_t n, const int64_t* rowptr, const int32_t* colidx, const cplx* vals,
                               int* flags) {
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  const int64_t b = rowptr[r], e = rowptr[r + 1];
  atomicMax(flags + 2, (int)(e - b));
  for (int64_t k = b; k < e; ++k) {
    const cplx v = vals[k];
    if (v.im != 0.0) atomicOr(flags + 0, 1);
    const int32_t c = colidx[k];
    int64_t lo = rowptr[c], hi = rowptr[c + 1];
    while (lo < hi) {
      const int64_t mid = (lo + hi) >> 1;
      if (colidx[mid] < (int32_t)r) lo = mid + 1;
      else hi = mid;
    }
    cplx w = mkc(0.0, 0.0);
    if (lo < rowptr[c + 1] && colidx[lo] == (int32_t)r) w = vals[lo];
    const double dr = v.re - w.re, di = v.im + w.im;
    const double scale = fabs(v.re) + fabs(v.im) + fabs(w.re) + fabs(w.im);
    if (fabs(dr) + fabs(di) > 1e-13 * scale) atomicOr(flags + 1, 1);
  }
}

__global__ void real_part_kernel(int64_t nnz, const cplx* vals, double* out_d, float* out_f) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nnz) return;
  const double v = vals[k].re;
  out_d[k] = v;
  out_f[k] = (float)v;
}

// ---------------------------------------------------------------- driver
template <int CAP, int TCAP>
static void run_lower(Ctx* ctx, const LowerParams& P, int pass, int64_t* counts, const int64_t* colptr,
                      int32_t* rowidx, cplx* vals, int* overflow) {
  const int64_t dim = P.S.dim;
  lower_kernel<CAP, TCAP><<<(unsigned)ceil_div(dim, 128), 128, 0, ctx->stream>>>(P, pass, counts, colptr,
                                                                                 rowidx, vals, overflow);
  QD_CHECK_LAUNCH();
  QD_LAUNCHED(ctx);
}

typedef void (*LowerFn)(Ctx*, const LowerParams&, int, int64_t*, const int64_t*, int32_t*, cplx*, int*);

static LowerFn pick_lower(int64_t cap_needed, int tcap_needed, int& cap_out) {
  // tcap: leaves of the widest product; cap: bound on distinct rows per column
#define QD_PICK(C, T)                              \
  if (cap_needed <= C && tcap_needed <= T) {       \
    cap_out = C;                                   \
    return &run_lower<C, T>;                       \
  }
  QD_PICK(32, 4)
  QD_PICK(32, 16)
  QD_PICK(128, 16)
  QD_PICK(128, 64)
  QD_PICK(512, 64)
  QD_PICK(512, 256)
#undef QD_PICK
  cap_out = 0;
  return nullptr;
}

void ham_lower(qd_ham* H, const qd_term* terms, int nterms, const qd_gate* gates, int ngates) {
  Ctx* ctx = H->ctx;
  qd_sector* S = H->sec;
  const int nbits = S->nbits;
  QD_REQUIRE(nterms >= 0 && ngates >= 0, QD_ERR_INVALID, "negative term or gate count");
  std::vector<TermDev> ht(std::max(nterms, 1));
  std::vector<GateDev> hg(std::max(ngates, 1));
  int64_t leaf_total = 0;
  int max_leaves = 1;
  for (int g = 0; g < ngates; ++g) {
    const qd_gate& G = gates[g];
    QD_REQUIRE(G.kind == QD_GATE_BIT || G.kind == QD_GATE_HOP, QD_ERR_INVALID, "gate %d: bad kind", g);
    QD_REQUIRE(G.site >= 0 && G.site < nbits, QD_ERR_INVALID, "gate %d: site %d outside %d bits", g, G.site,
               nbits);
    QD_REQUIRE(G.kind != QD_GATE_HOP || (G.site_b >= 0 && G.site_b < nbits), QD_ERR_INVALID,
               "gate %d: site %d outside %d bits", g, G.site_b, nbits);
    GateDev d{};
    d.kind = G.kind;
    d.site = G.site;
    d.site_b = G.site_b;
    d.string = G.string;
    for (int q = 0; q < 4; ++q) d.u[q] = mkc(G.u[2 * q], G.u[2 * q + 1]);
    hg[g] = d;
  }
  for (int t = 0; t < nterms; ++t) {
    const qd_term& T = terms[t];
    QD_REQUIRE(T.ngates >= 0 && T.gate_offset >= 0 && (int64_t)T.gate_offset + T.ngates <= ngates,
               QD_ERR_INVALID, "term %d: gate range outside the gate array", t);
    int nbit = 0;
    for (int g = 0; g < T.ngates; ++g) nbit += (gates[T.gate_offset + g].kind == QD_GATE_BIT);
    QD_REQUIRE(nbit <= 8, QD_ERR_UNSUPPORTED, "term %d: more than 8 bit gates in one product", t);
    TermDev d{};
    d.coeff = mkc(T.coeff_re, T.coeff_im);
    d.gate_offset = T.gate_offset;
    d.ngates = T.ngates;
    d.nbit = nbit;
    ht[t] = d;
    leaf_total += 1ll << nbit;
    max_leaves = std::max(max_leaves, 1 << nbit);
  }
  H->host_terms.assign(terms, terms + nterms);
  H->host_gates.assign(gates, gates + ngates);
  H->from_terms = true;
  const int64_t dim = S->view.dim;
  H->dim = dim;
  DBuf<TermDev> dterms(ht.size());
  DBuf<GateDev> dgates(hg.size());
  QD_CUDA(cudaMemcpyAsync(dterms.p, ht.data(), ht.size() * sizeof(TermDev), cudaMemcpyHostToDevice, ctx->stream));
  QD_CUDA(cudaMemcpyAsync(dgates.p, hg.data(), hg.size() * sizeof(GateDev), cudaMemcpyHostToDevice, ctx->stream));

  // Row-wise lowering from compiled transitions when every term is a
  // product on at most 6 sites (mfree.cu); the tree walk per column otherwise.
  const bool tree_only = std::getenv("QD_LOWER_TREE") != nullptr;
  if (tree_only || !ham_lower_pull(H)) {
    LowerParams P;
    std::memset(&P, 0, sizeof(P));
    P.S = S->view;
    P.terms = dterms.p;
    P.gates = dgates.p;
    P.nterms = nterms;

    // Start with the smallest column capacity that the leaf count allows and
    // grow it only if a column overflows (most operators have short columns).
    int cap = 0;
    const int64_t cap_bound = std::min<int64_t>(leaf_total, std::max<int64_t>(dim, 1));
    DBuf<int> overflow(1);
    DBuf<int64_t> colptr(dim + 1);
    LowerFn fn = nullptr;
    for (int64_t try_cap = 32;; try_cap *= 4) {
      fn = pick_lower(std::min<int64_t>(std::min<int64_t>(try_cap, cap_bound), 512), max_leaves, cap);
      QD_REQUIRE(fn != nullptr, QD_ERR_UNSUPPORTED, "lowering: products with %d leaves are not supported",
                 max_leaves);
      QD_CUDA(cudaMemsetAsync(overflow.p, 0, sizeof(int), ctx->stream));
      QD_CUDA(cudaMemsetAsync(colptr.p, 0, (dim + 1) * 8, ctx->stream));
      if (dim > 0) fn(ctx, P, 0, colptr.p, nullptr, nullptr, nullptr, overflow.p);
      int ovf = 0;
      QD_CUDA(cudaMemcpyAsync(&ovf, overflow.p, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
      QD_CUDA(cudaStreamSynchronize(ctx->stream));
      if (!ovf) break;
      QD_REQUIRE(cap < 512 && cap < cap_bound, QD_ERR_OVERFLOW, "lowering: a column has more than %d entries", cap);
    }
    exclusive_scan_i64(ctx, colptr.p, colptr.p, dim + 1);
    int64_t nnz = 0;
    QD_CUDA(cudaMemcpyAsync(&nnz, colptr.p + dim, 8, cudaMemcpyDeviceToHost, ctx->stream));
    QD_CUDA(cudaStreamSynchronize(ctx->stream));
    QD_REQUIRE(nnz < (int64_t)INT32_MAX * 8, QD_ERR_UNSUPPORTED, "nnz too large");
    H->nnz = nnz;
    DBuf<int32_t> rowidx(nnz + 1);
    DBuf<cplx> cvals(nnz + 1);
    if (dim > 0 && nnz > 0) fn(ctx, P, 1, nullptr, colptr.p, rowidx.p, cvals.p, overflow.p);

    // CSC -> CSR (rows of H); pad the arrays so vector loads past the end stay inside
    H->rowptr.alloc(dim + 2);
    H->colidx.alloc(nnz + 16);
    H->vals_c.alloc(nnz + 16);
    QD_CUDA(cudaMemsetAsync(H->colidx.p, 0, (nnz + 16) * sizeof(int32_t), ctx->stream));
    QD_CUDA(cudaMemsetAsync(H->vals_c.p, 0, (nnz + 16) * sizeof(cplx), ctx->stream));
    ham_transpose(ctx, dim, colptr.p, rowidx.p, cvals.p, nnz, H->rowptr.p, H->colidx.p, H->vals_c.p);
  }

  ham_finish(H);
}

// Flags (real, Hermitian), the longest row and the real copies of the values
// of a CSR matrix held by H.
void ham_finish(qd_ham* H) {
  Ctx* ctx = H->ctx;
  const int64_t dim = H->dim;
  DBuf<int> flags(3);
  QD_CUDA(cudaMemsetAsync(flags.p, 0, 3 * sizeof(int), ctx->stream));
  if (dim > 0) {
    analyze_kernel<<<(unsigned)ceil_div(dim, 256), 256, 0, ctx->stream>>>(dim, H->rowptr.p, H->colidx.p,
                                                                          H->vals_c.p, flags.p);
    QD_CHECK_LAUNCH();
    QD_LAUNCHED(ctx);
  }
  int hf[3];
  QD_CUDA(cudaMemcpyAsync(hf, flags.p, sizeof(hf), cudaMemcpyDeviceToHost, ctx->stream));
  QD_CUDA(cudaStreamSynchronize(ctx->stream));
  H->flags = (hf[0] ? 0 : QD_HAM_REAL) | (hf[1] ? 0 : QD_HAM_HERMITIAN);
  H->max_row_nnz = hf[2];
  const int64_t nnz = H->nnz;
  H->vals_r = DBuf<double>();
  H->vals_f = DBuf<float>();
  H->bun_checked = false;  // the batched solver's uniform-value check follows the values
  H->bun_d = DBuf<float>();
  if (H->flags & QD_HAM_REAL) {
    H->vals_r.alloc(nnz + 16);
    H->vals_f.alloc(nnz + 16);
    QD_CUDA(cudaMemsetAsync(H->vals_r.p, 0, (nnz + 16) * sizeof(double), ctx->stream));
    QD_CUDA(cudaMemsetAsync(H->vals_f.p, 0, (nnz + 16) * sizeof(float), ctx->stream));
    if (nnz > 0) {
      real_part_kernel<<<(unsigned)ceil_div(nnz, 256), 256, 0, ctx->stream>>>(nnz, H->vals_c.p, H->vals_r.p,
                                                                             H->vals_f.p);
      QD_CHECK_LAUNCH();
      QD_LAUNCHED(ctx);
    }
  }
  QD_CUDA(cudaStreamSynchronize(ctx->stream));
}

__global__ void row_abs_max_kernel(int64_t n, const int64_t* rowptr, const cplx* vals, unsigned long long* out) {
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int64_t k = rowptr[r]; k < rowptr[r + 1]; ++k) s += hypot(vals[k].re, vals[k].im);
    atomicMax(out, (unsigned long long)__double_as_longlong(s));
  }
}

// max_r sum_c |H(r, c)| (cached): bounds the spectral radius.
double ham_norm_inf(qd_ham* H) {
  if (H->norm_inf >= 0.0) return H->norm_inf;
  Ctx* ctx = H->ctx;
  DBuf<unsigned long long> m(1);
  QD_CUDA(cudaMemsetAsync(m.p, 0, sizeof(unsigned long long), ctx->stream));
  if (H->dim > 0) {
    const int g = (int)std::max<int64_t>(1, std::min<int64_t>(ceil_div(H->dim, 256), (int64_t)ctx->num_sms * 8));
    row_abs_max_kernel<<<g, 256, 0, ctx->stream>>>(H->dim, H->rowptr.p, H->vals_c.p, m.p);
    QD_CHECK_LAUNCH();
    QD_LAUNCHED(ctx);
  }
  unsigned long long bits = 0;
  QD_CUDA(cudaMemcpyAsync(&bits, m.p, 8, cudaMemcpyDeviceToHost, ctx->stream));
  QD_CUDA(cudaStreamSynchronize(ctx->stream));
  double v = 0.0;
  std::memcpy(&v, &bits, 8);
  H->norm_inf = v;
  return v;
}

// Gershgorin interval of the real parts: per row [Re d - R, Re d + R] with R
// the sum of |off-diagonal| values; keys order doubles as unsigned integers.
__device__ __forceinline__ unsigned long long ordered_key(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}
__host__ __device__ inline double from_ordered_key(unsigned long long k) {
  const unsigned long long b = (k >> 63) ? (k & 0x7fffffffffffffffull) : ~k;
  double x;
  memcpy(&x, &b, 8);
  return x;
}
__global__ void gershgorin_kernel(int64_t n, const int64_t* rowptr, const int32_t* colidx, const cplx* vals,
                                  unsigned long long* lo_neg, unsigned long long* hi) {
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
    double d = 0.0, R = 0.0;
    for (int64_t k = rowptr[r]; k < rowptr[r + 1]; ++k) {
      if (colidx[k] == (int32_t)r) d = vals[k].re;
      else R += hypot(vals[k].re, vals[k].im);
    }
    atomicMax(hi, ordered_key(d + R));
    atomicMax(lo_neg, ordered_key(-(d - R)));
  }
}

// Half the width of the Gershgorin interval: for Hermitian H,
// ||H - c I||_2 <= this, c the interval's centre.
double ham_gershgorin_halfwidth(qd_ham* H) {
  Ctx* ctx = H->ctx;
  if (H->dim <= 0) return 0.0;
  DBuf<unsigned long long> m(2);
  QD_CUDA(cudaMemsetAsync(m.p, 0, 2 * sizeof(unsigned long long), ctx->stream));
  const int g = (int)std::max<int64_t>(1, std::min<int64_t>(ceil_div(H->dim, 256), (int64_t)ctx->num_sms * 8));
  gershgorin_kernel<<<g, 256, 0, ctx->stream>>>(H->dim, H->rowptr.p, H->colidx.p, H->vals_c.p, m.p, m.p + 1);
  QD_CHECK_LAUNCH();
  QD_LAUNCHED(ctx);
  unsigned long long k[2] = {0, 0};
  QD_CUDA(cudaMemcpyAsync(k, m.p, sizeof(k), cudaMemcpyDeviceToHost, ctx->stream));
  QD_CUDA(cudaStreamSynchronize(ctx->stream));
  const double lo = -from_ordered_key(k[0]), hi = from_ordered_key(k[1]);
  return 0.5 * (hi - lo);
}

void ham_ensure_row_order(qd_ham* H) {
  if (H->row_order.p) return;
  const int64_t n = H->dim;
  std::vector<int64_t> rp(n + 1);
  QD_CUDA(cudaMemcpyAsync(rp.data(), H->rowptr.p, (n + 1) * 8, cudaMemcpyDeviceToHost, H->ctx->stream));
  QD_CUDA(cudaStreamSynchronize(H->ctx->stream));
  std::vector<int32_t> order(n > 0 ? n : 1);
  constexpr int64_t kWindow = 256;
  for (int64_t w0 = 0; w0 < n; w0 += kWindow) {
    const int64_t w1 = std::min(n, w0 + kWindow);
    for (int64_t r = w0; r < w1; ++r) order[r] = (int32_t)r;
    std::stable_sort(order.begin() + w0, order.begin() + w1,
                     [&](int32_t a, int32_t b) { return rp[a + 1] - rp[a] > rp[b + 1] - rp[b]; });
  }
  H->row_order.alloc(order.size());
  QD_CUDA(cudaMemcpyAsync(H->row_order.p, order.data(), order.size() * 4, cudaMemcpyHostToDevice, H->ctx->stream));
  QD_CUDA(cudaStreamSynchronize(H->ctx->stream));
}

}  // namespace qd
