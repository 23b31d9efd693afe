// mfree.cu -- matrix-free products y = H x.
//
// The reference's on-the-fly product is Operator::map_acc /
// OperatorSum::map_acc (operator.hpp:215-232, operator_abel.hpp:36-49): it
// expands the operator tree per input state and pushes every leaf into y.
// Here the tree is compiled once on the host into entries (ham.cuh, MfEntry):
// for each term and each input pattern p on the term's support, the leaves
// of the tree are walked exactly as the lowering walks them (same gate order,
// same drop rule |v| <= 1e-10, same leaf-order sums, same rounding), giving
// output patterns q with amplitude coeff * sum.  Entries with q == p build
// the stored diagonal (summed in term order, as the CSR lowering sums them);
// the others are applied on the fly, pulled by output row: the row state s
// takes amp * sign * x[rank(s ^ flip)] from every entry whose output pattern
// it carries.  Nothing of size nnz is stored: the basis (8 B/row), the
// diagonal (8 or 16 B/row) and the vectors are all the product reads from
// HBM, at the price of ranking every target state on the fly.
//
// Ranking: product sectors (combinatorial number system per field) use byte
// tables -- for each field, byte b of its value and the number of set bits
// below that byte give the byte's share of the colex rank, so a rank is one
// table load per byte; other sectors use sector_rank (directory + binary
// search).  The amplitudes keep the JW sign of the bits outside the support
// apart (the parity of c & jw), which multiplies exactly.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "ham.cuh"
#include "krylov.cuh"
#include "scan.cuh"
#include "spmv.cuh"

namespace qd {

// ---------------------------------------------------------------- host compile
static inline cplx h_mul(cplx a, cplx b) {  // one rounding per product and per sum (-ffp-contract=off)
  const double rr = a.re * b.re, ii = a.im * b.im, ri = a.re * b.im, ir = a.im * b.re;
  return mkc(rr - ii, ri + ir);
}
static inline cplx h_add(cplx a, cplx b) { return mkc(a.re + b.re, a.im + b.im); }
static inline uint64_t above_mask(int p) { return (p + 1 >= 64) ? 0ull : (~0ull << (p + 1)); }

static uint64_t deposit(uint64_t v, uint64_t mask) {
  uint64_t out = 0;
  for (int i = 0; mask; ++i) {
    const uint64_t low = mask & (~mask + 1);
    if ((v >> i) & 1ull) out |= low;
    mask &= mask - 1;
  }
  return out;
}

static uint64_t extract(uint64_t s, uint64_t mask) {
  uint64_t out = 0;
  for (int i = 0; mask; ++i) {
    const uint64_t low = mask & (~mask + 1);
    if (s & low) out |= 1ull << i;
    mask &= mask - 1;
  }
  return out;
}

// One leaf of a term's tree on state s (the lowering's leaf_path, host side).
static bool host_leaf(const std::vector<qd_gate>& G, const qd_term& T, int nbit, uint64_t s, int j, uint64_t& st_out,
                      cplx& v_out) {
  uint64_t st = s;
  cplx v = mkc(1.0, 0.0);
  int bp = nbit - 1;
  for (int ig = T.ngates - 1; ig >= 0; --ig) {
    const qd_gate& g = G[T.gate_offset + ig];
    if (g.kind == QD_GATE_BIT) {
      const int o = (j >> bp) & 1;
      --bp;
      const int b = (int)((st >> g.site) & 1ull);
      const uint64_t above = (g.site + 1 >= 64) ? 0ull : (st >> (g.site + 1));
      const cplx jw = (__builtin_popcountll(above) & 1) ? mkc((double)g.string, 0.0) : mkc(1.0, 0.0);
      const cplx u = mkc(g.u[2 * (b * 2 + o)], g.u[2 * (b * 2 + o) + 1]);
      v = h_mul(h_mul(jw, u), v);
      const uint64_t bit = 1ull << g.site;
      st = o ? (st | bit) : (st & ~bit);
    } else {
      const int sa = g.site, sb = g.site_b;
      if (sa == sb) {
        const double occ = (double)((st >> sb) & 1ull);
        v = mkc(occ * v.re, occ * v.im);
      } else if (((st >> sb) & 1ull) && !((st >> sa) & 1ull)) {
        const int jw1 = __builtin_popcountll((sb + 1 >= 64) ? 0ull : (st >> (sb + 1)));
        st &= ~(1ull << sb);
        const int jw2 = __builtin_popcountll((sa + 1 >= 64) ? 0ull : (st >> (sa + 1)));
        st |= (1ull << sa);
        const int jw = ((jw1 & 1) ? g.string : 1) * ((jw2 & 1) ? g.string : 1);
        v = h_mul(mkc((double)jw, 0.0), v);
      } else {
        return false;
      }
    }
  }
  st_out = st;
  v_out = v;
  return true;
}

void compile_terms(const qd_ham* H, std::vector<MfEntry>& off, std::vector<MfEntry>& dia) {
  const std::vector<qd_term>& terms = H->host_terms;
  const std::vector<qd_gate>& gates = H->host_gates;
  for (size_t t = 0; t < terms.size(); ++t) {
    const qd_term& T = terms[t];
    uint64_t sup = 0;
    int nbit = 0;
    for (int g = 0; g < T.ngates; ++g) {
      const qd_gate& G = gates[T.gate_offset + g];
      QD_REQUIRE(G.string == 1 || G.string == -1, QD_ERR_UNSUPPORTED,
                 "term %zu: matrix-free form needs Jordan-Wigner strings of +1 or -1", t);
      sup |= 1ull << G.site;
      if (G.kind == QD_GATE_HOP) sup |= 1ull << G.site_b;
      nbit += (G.kind == QD_GATE_BIT);
    }
    const int nsup = __builtin_popcountll(sup);
    QD_REQUIRE(nsup <= kMfMaxSupport, QD_ERR_UNSUPPORTED, "term %zu: support of %d bits (matrix-free form: <= %d)", t,
               nsup, kMfMaxSupport);
    uint64_t X = 0;  // outside-support parity mask of the whole product
    for (int g = 0; g < T.ngates; ++g) {
      const qd_gate& G = gates[T.gate_offset + g];
      if (G.string != -1) continue;
      if (G.kind == QD_GATE_BIT) X ^= above_mask(G.site) & ~sup;
      else if (G.site != G.site_b) X ^= (above_mask(G.site_b) ^ above_mask(G.site)) & ~sup;
    }
    const cplx coeff = mkc(T.coeff_re, T.coeff_im);
    for (uint64_t p = 0; p < (1ull << nsup); ++p) {
      const uint64_t sp = deposit(p, sup);
      std::vector<uint64_t> tq;
      std::vector<cplx> tv;
      for (int j = 0; j < (1 << nbit); ++j) {
        uint64_t st;
        cplx v;
        if (!host_leaf(gates, T, nbit, sp, j, st, v)) continue;
        if (!(std::hypot(v.re, v.im) > 1e-10)) continue;  // operator.hpp:255
        const uint64_t q = extract(st, sup);
        size_t k = 0;
        while (k < tq.size() && tq[k] != q) ++k;
        if (k < tq.size()) {
          tv[k] = h_add(tv[k], v);
        } else {
          tq.push_back(q);
          tv.push_back(v);
        }
      }
      for (size_t k = 0; k < tq.size(); ++k) {
        MfEntry e;
        e.sup = sup;
        e.outb = deposit(tq[k], sup);
        e.flip = sp ^ e.outb;
        e.jw = X;
        e.amp = h_mul(coeff, tv[k]);
        (e.flip ? off : dia).push_back(e);
      }
    }
  }
}

void build_tables(const qd_sector* S, MfRank& rk, std::vector<int64_t>& tab) {
  int64_t C[64][64];
  for (int n = 0; n < 64; ++n)
    for (int k = 0; k < 64; ++k) C[n][k] = (k == 0) ? 1 : (n == 0 ? 0 : C[n - 1][k - 1] + C[n - 1][k]);
  const SectorView& V = S->view;
  rk.nf = V.nfields;
  for (int f = 0; f < V.nfields; ++f) {
    const Field& F = V.fields[f];
    rk.lo[f] = F.lo;
    rk.width[f] = F.width;
    rk.k[f] = F.k;
    rk.is_free[f] = F.is_free;
    rk.stride[f] = F.stride;
    rk.nb[f] = (F.width + 7) / 8;
    rk.off[f] = (int64_t)tab.size();
    if (F.is_free) continue;
    const int K = F.k;
    for (int b = 0; b < rk.nb[f]; ++b)
      for (int byte = 0; byte < 256; ++byte)
        for (int cb = 0; cb <= K; ++cb) {
          int64_t acc = 0;
          int idx = 0;
          for (int q = 0; q < 8; ++q)
            if ((byte >> q) & 1) {
              const int p = 8 * b + q, j = cb + idx + 1;
              if (p < 64 && j < 64 && j <= p) acc += C[p][j];
              ++idx;
            }
          tab.push_back(acc);
        }
  }
}

// ---------------------------------------------------------------- device
template <typename AV, typename VV>
struct MfArgs {
  int64_t dim;
  const uint64_t* basis;
  const AV* diag;
  const MfEntry* ent;
  int nent;
  int use_tables;
  MfRank rk;
  SectorView S;
  const VV* x;
  VV* y;
  double scale;
  const double* scale_dev;
  const int* stop;
  int step;
};

template <typename AV, typename VV>
__device__ __forceinline__ int64_t mf_rank(const MfArgs<AV, VV>& A, uint64_t c) {
  if (!A.use_tables) return sector_rank(A.S, c);
  int64_t r = 0;
  for (int f = 0; f < A.rk.nf; ++f) {
    const int w = A.rk.width[f];
    const uint64_t v = (c >> A.rk.lo[f]) & ((w >= 64) ? ~0ull : ((1ull << w) - 1));
    if (A.rk.is_free[f]) {
      r += (int64_t)v * A.rk.stride[f];
      continue;
    }
    const int k = A.rk.k[f];
    if (__popcll(v) != k) return A.dim;
    const int64_t* T = A.rk.tab + A.rk.off[f];
    int64_t acc = 0;
    int cb = 0;
    for (int b = 0; b < A.rk.nb[f]; ++b) {
      const unsigned byte = (unsigned)(v >> (8 * b)) & 255u;
      acc += __ldg(T + ((int64_t)b * 256 + byte) * (k + 1) + cb);
      cb += __popc(byte);
    }
    r += acc * A.rk.stride[f];
  }
  return r;
}

__device__ __forceinline__ double amp_of(double*, cplx a) { return a.re; }
__device__ __forceinline__ cplx amp_of(cplx*, cplx a) { return a; }
__device__ __forceinline__ double vneg(double a) { return -a; }
__device__ __forceinline__ cplx vneg(cplx a) { return mkc(-a.re, -a.im); }

template <typename AV, typename VV>
__global__ void __launch_bounds__(256) mf_spmv_kernel(MfArgs<AV, VV> A) {
  extern __shared__ __align__(16) unsigned char mf_smem[];
  uint64_t* s_sup = reinterpret_cast<uint64_t*>(mf_smem);
  uint64_t* s_out = s_sup + A.nent;
  uint64_t* s_flip = s_out + A.nent;
  uint64_t* s_jw = s_flip + A.nent;
  AV* s_amp = reinterpret_cast<AV*>(s_jw + A.nent);
  if (A.stop) {
    const int st = *A.stop;
    if (st != 0 && st < A.step) return;
  }
  for (int e = threadIdx.x; e < A.nent; e += blockDim.x) {
    const MfEntry E = A.ent[e];
    s_sup[e] = E.sup;
    s_out[e] = E.outb;
    s_flip[e] = E.flip;
    s_jw[e] = E.jw;
    s_amp[e] = amp_of((AV*)nullptr, E.amp);
  }
  __syncthreads();
  const double sc = A.scale_dev ? *A.scale_dev : A.scale;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < A.dim; r += stride) {
    const uint64_t s = __ldg(A.basis + r);
    VV acc = vfma(A.diag[r], A.x[r], vzero(VV{}));
    for (int e0 = 0; e0 < A.nent; e0 += 32) {
      const int ne = min(32, A.nent - e0);
      unsigned mask = 0;
      for (int q = 0; q < ne; ++q) mask |= (unsigned)((s & s_sup[e0 + q]) == s_out[e0 + q]) << q;
      while (mask) {
        const int e = e0 + __ffs(mask) - 1;
        mask &= mask - 1;
        const uint64_t c = s ^ s_flip[e];
        const int64_t col = mf_rank(A, c);
        if (col >= A.dim) continue;
        AV a = s_amp[e];
        if (__popcll(c & s_jw[e]) & 1) a = vneg(a);
        acc = vfma(a, ld_ro(A.x + col), acc);
      }
    }
    A.y[r] = vscale(sc, acc);
  }
}

// diagonal: sum of the state-keeping entries in term order, 0 + p first
__global__ void mf_diag_kernel(int64_t dim, const uint64_t* basis, const MfEntry* dia, int nd, cplx* diag) {
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < dim; r += (int64_t)gridDim.x * blockDim.x) {
    const uint64_t s = basis[r];
    cplx acc = mkc(0.0, 0.0);
    for (int e = 0; e < nd; ++e) {
      const MfEntry E = dia[e];
      if ((s & E.sup) != E.outb) continue;
      cplx a = E.amp;
      if (__popcll(s & E.jw) & 1) a = mkc(-a.re, -a.im);
      acc = cadd_rn(acc, a);
    }
    diag[r] = acc;
  }
}

__global__ void mf_diag_real_kernel(int64_t dim, const cplx* dc, double* dr, int* has_imag) {
  bool im = false;
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < dim; r += (int64_t)gridDim.x * blockDim.x) {
    const cplx d = dc[r];
    dr[r] = d.re;
    im |= (d.im != 0.0);
  }
  if (im) atomicOr(has_imag, 1);
}

static int mf_grid(Ctx* ctx, int64_t n) {
  return (int)std::max<int64_t>(1, std::min<int64_t>(ceil_div(n, 256), (int64_t)ctx->num_sms * 8));
}

void ham_build_matrix_free(qd_ham* H) {
  if (H->has_mf) return;
  QD_REQUIRE(H->from_terms, QD_ERR_UNSUPPORTED,
             "the matrix-free form compiles operator terms; this matrix is a sum or a multiple of lowered ones");
  Ctx* ctx = H->ctx;
  const qd_sector* S = H->sec;
  std::vector<MfEntry> off, dia;
  compile_terms(H, off, dia);
  QD_REQUIRE((int)off.size() <= kMfMaxEntries, QD_ERR_UNSUPPORTED,
             "%zu state-changing entries (matrix-free form: <= %d)", off.size(), kMfMaxEntries);
  const int64_t n = H->dim;
  bool real = true;
  for (const MfEntry& e : off) real &= (e.amp.im == 0.0);
  // diagonal
  DBuf<MfEntry> ddia(std::max<size_t>(dia.size(), 1));
  if (!dia.empty())
    QD_CUDA(cudaMemcpyAsync(ddia.p, dia.data(), dia.size() * sizeof(MfEntry), cudaMemcpyHostToDevice, ctx->stream));
  H->diag_c.alloc(n);
  mf_diag_kernel<<<mf_grid(ctx, n), 256, 0, ctx->stream>>>(n, S->basis.p, ddia.p, (int)dia.size(), H->diag_c.p);
  QD_CHECK_LAUNCH();
  QD_LAUNCHED(ctx);
  H->diag_r.alloc(n);
  DBuf<int> him(1);
  QD_CUDA(cudaMemsetAsync(him.p, 0, sizeof(int), ctx->stream));
  mf_diag_real_kernel<<<mf_grid(ctx, n), 256, 0, ctx->stream>>>(n, H->diag_c.p, H->diag_r.p, him.p);
  QD_CHECK_LAUNCH();
  QD_LAUNCHED(ctx);
  int has_im = 0;
  QD_CUDA(cudaMemcpyAsync(&has_im, him.p, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  // entries and rank tables
  H->mf_ent.alloc(std::max<size_t>(off.size(), 1));
  if (!off.empty())
    QD_CUDA(cudaMemcpyAsync(H->mf_ent.p, off.data(), off.size() * sizeof(MfEntry), cudaMemcpyHostToDevice,
                            ctx->stream));
  H->mf_nent = (int)off.size();
  H->mf_tables = (S->view.rank_kind == 1 && S->view.nfields <= 4);
  std::memset(&H->mf_rank, 0, sizeof(H->mf_rank));
  if (H->mf_tables) {
    std::vector<int64_t> tab;
    build_tables(S, H->mf_rank, tab);
    H->mf_tab.alloc(std::max<size_t>(tab.size(), 1));
    if (!tab.empty())
      QD_CUDA(cudaMemcpyAsync(H->mf_tab.p, tab.data(), tab.size() * 8, cudaMemcpyHostToDevice, ctx->stream));
    H->mf_rank.tab = H->mf_tab.p;
    if (S->view.nbits <= 32 && n < (1ll << 31)) {  // 32-bit copy for the 32-bit product
      std::vector<uint32_t> t32(std::max<size_t>(tab.size(), 1), 0u);
      for (size_t i = 0; i < tab.size(); ++i) t32[i] = (uint32_t)tab[i];
      H->mf_tab32.alloc(t32.size());
      QD_CUDA(cudaMemcpyAsync(H->mf_tab32.p, t32.data(), t32.size() * 4, cudaMemcpyHostToDevice, ctx->stream));
    }
  }
  QD_CUDA(cudaStreamSynchronize(ctx->stream));
  H->mf_real = real && !has_im;
  if (H->mf_real) H->diag_c = DBuf<cplx>();
  else H->diag_r = DBuf<double>();
  H->has_mf = true;
}

// 32-bit form of the product for registers of at most 32 bits ranked by
// tables (every model of the configurations): states, masks and table entries
// in 32-bit integers, the fields unrolled, so a row costs about half the
// integer instructions of the 64-bit form.
struct Mf32 {
  int nf;
  int lo[2], k[2], nb[2];
  uint32_t wmask[2];
  uint32_t stride[2];
  int off[2];
  const uint32_t* tab;
};

template <typename AV, typename VV, int NF>
__global__ void __launch_bounds__(256) mf_spmv32_kernel(int64_t dim, const uint64_t* __restrict__ basis,
                                                        const AV* __restrict__ diag, const MfEntry* __restrict__ ent,
                                                        int nent, Mf32 R, const VV* __restrict__ x, VV* __restrict__ y,
                                                        double scale, const double* scale_dev, const int* stop,
                                                        int step) {
  extern __shared__ __align__(16) unsigned char mf_smem32[];
  uint32_t* s_sup = reinterpret_cast<uint32_t*>(mf_smem32);
  uint32_t* s_out = s_sup + nent;
  uint32_t* s_flip = s_out + nent;
  uint32_t* s_jw = s_flip + nent;
  AV* s_amp = reinterpret_cast<AV*>(mf_smem32 + (((size_t)4 * nent * sizeof(uint32_t) + 15) & ~(size_t)15));
  if (stop) {
    const int st = *stop;
    if (st != 0 && st < step) return;
  }
  for (int e = threadIdx.x; e < nent; e += blockDim.x) {
    const MfEntry E = ent[e];
    s_sup[e] = (uint32_t)E.sup;
    s_out[e] = (uint32_t)E.outb;
    s_flip[e] = (uint32_t)E.flip;
    s_jw[e] = (uint32_t)E.jw;
    s_amp[e] = amp_of((AV*)nullptr, E.amp);
  }
  __syncthreads();
  const double sc = scale_dev ? *scale_dev : scale;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < dim; r += stride) {
    const uint32_t s = (uint32_t)__ldg(basis + r);
    VV acc = vfma(diag[r], x[r], vzero(VV{}));
    for (int e0 = 0; e0 < nent; e0 += 32) {
      const int ne = min(32, nent - e0);
      unsigned mask = 0;
      for (int q = 0; q < ne; ++q) mask |= (unsigned)((s & s_sup[e0 + q]) == s_out[e0 + q]) << q;
      while (mask) {
        const int e = e0 + __ffs(mask) - 1;
        mask &= mask - 1;
        const uint32_t c = s ^ s_flip[e];
        uint32_t col = 0;
        bool in = true;
#pragma unroll
        for (int f = 0; f < NF; ++f) {
          const uint32_t v = (c >> R.lo[f]) & R.wmask[f];
          in &= (__popc(v) == R.k[f]);
          const uint32_t* T = R.tab + R.off[f];
          const int kk = R.k[f] + 1;
          uint32_t a = __ldg(T + (v & 255u) * kk);
          int cb = __popc(v & 255u);
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
        if (!in) continue;
        AV a = s_amp[e];
        if (__popc(c & s_jw[e]) & 1) a = vneg(a);
        acc = vfma(a, ld_ro(x + col), acc);
      }
    }
    y[r] = vscale(sc, acc);
  }
}

// Builds the 32-bit form when the register has at most 32 bits, the sector is
// a product of at most two fields and the dimension fits in 32 bits.
static bool mf32_prepare(qd_ham* H, Mf32& R) {
  const SectorView& V = H->sec->view;
  if (!H->mf_tables || V.nbits > 32 || H->dim >= (1ll << 31)) return false;
  int nf = 0;
  for (int f = 0; f < V.nfields; ++f)
    if (!V.fields[f].is_free) ++nf;
  if (nf != V.nfields || nf < 1 || nf > 2) return false;
  if (!H->mf_tab32.p) return false;  // built with the tables (ham_build_matrix_free)
  std::memset(&R, 0, sizeof(R));
  R.nf = nf;
  for (int f = 0; f < nf; ++f) {
    const Field& F = V.fields[f];
    R.lo[f] = F.lo;
    R.k[f] = F.k;
    R.nb[f] = H->mf_rank.nb[f];
    R.wmask[f] = (F.width >= 32) ? 0xffffffffu : ((1u << F.width) - 1u);
    R.stride[f] = (uint32_t)F.stride;
    R.off[f] = (int)H->mf_rank.off[f];
  }
  R.tab = H->mf_tab32.p;
  return true;
}

template <typename AV, typename VV>
static void launch_mf_typed(Ctx* ctx, qd_ham* H, const AV* diag, const VV* x, VV* y, double scale,
                            const double* scale_dev, const int* stop, int step) {
  MfArgs<AV, VV> A;
  std::memset(&A, 0, sizeof(A));
  A.dim = H->dim;
  A.basis = H->sec->basis.p;
  A.diag = diag;
  A.ent = H->mf_ent.p;
  A.nent = H->mf_nent;
  A.use_tables = H->mf_tables ? 1 : 0;
  A.rk = H->mf_rank;
  A.S = H->sec->view;
  A.x = x;
  A.y = y;
  A.scale = scale;
  A.scale_dev = scale_dev;
  A.stop = stop;
  A.step = step;
  Mf32 R;
  if (mf32_prepare(H, R)) {
    const int ne = std::max(H->mf_nent, 1);
    const size_t smem32 = (((size_t)4 * ne * sizeof(uint32_t) + 15) & ~(size_t)15) + (size_t)ne * sizeof(AV);
    if (R.nf == 1)
      mf_spmv32_kernel<AV, VV, 1><<<mf_grid(ctx, H->dim), 256, smem32, ctx->stream>>>(
          H->dim, H->sec->basis.p, diag, H->mf_ent.p, H->mf_nent, R, x, y, scale, scale_dev, stop, step);
    else
      mf_spmv32_kernel<AV, VV, 2><<<mf_grid(ctx, H->dim), 256, smem32, ctx->stream>>>(
          H->dim, H->sec->basis.p, diag, H->mf_ent.p, H->mf_nent, R, x, y, scale, scale_dev, stop, step);
    QD_CHECK_LAUNCH();
    QD_LAUNCHED(ctx);
    return;
  }
  const size_t smem = (size_t)std::max(H->mf_nent, 1) * (4 * sizeof(uint64_t) + sizeof(AV));
  mf_spmv_kernel<AV, VV><<<mf_grid(ctx, H->dim), 256, smem, ctx->stream>>>(A);
  QD_CHECK_LAUNCH();
  QD_LAUNCHED(ctx);
}

template <typename VV>
void launch_mf(Ctx* ctx, qd_ham* H, const VV* x, VV* y, double scale, const double* scale_dev, const int* stop,
               int step) {
  QD_REQUIRE(H->has_mf, QD_ERR_INVALID, "the matrix-free form has not been built");
  if (H->mf_real) {
    launch_mf_typed<double, VV>(ctx, H, H->diag_r.p, x, y, scale, scale_dev, stop, step);
  } else {
    if constexpr (std::is_same<VV, cplx>::value)
      launch_mf_typed<cplx, cplx>(ctx, H, H->diag_c.p, x, y, scale, scale_dev, stop, step);
    else
      QD_REQUIRE(false, QD_ERR_INVALID, "complex matrix-free operator on real vectors");
  }
}

template void launch_mf<double>(Ctx*, qd_ham*, const double*, double*, double, const double*, const int*, int);
template void launch_mf<cplx>(Ctx*, qd_ham*, const cplx*, cplx*, double, const double*, const int*, int);

// ---------------------------------------------------------------- row-wise lowering
// The CSR matrix built from the compiled entries, one thread per row: the
// row state s takes every entry whose output pattern it carries; entries that
// land on the same column add in entry order, which is term order, starting
// from 0 + p -- the union sum of OperatorSum::operator>> (operator_abel.hpp:
// 25-34) with explicit zeros kept.  Leaf sums inside a term, the 1e-10 leaf
// filter and every rounding are those of the tree lowering (compile_terms
// walks the same leaves), so the values equal the tree lowering's; a row
// pulls ~50 pattern tests instead of a column walking every term's tree.
struct PullArgs {
  int64_t dim;
  const uint64_t* basis;
  const MfEntry* ent;
  int nent;
  int use_tables;
  MfRank rk;
  SectorView S;
};

__device__ __forceinline__ int64_t pull_rank(const PullArgs& A, uint64_t c) {
  if (!A.use_tables) return sector_rank(A.S, c);
  int64_t r = 0;
  for (int f = 0; f < A.rk.nf; ++f) {
    const int w = A.rk.width[f];
    const uint64_t v = (c >> A.rk.lo[f]) & ((w >= 64) ? ~0ull : ((1ull << w) - 1));
    if (A.rk.is_free[f]) {
      r += (int64_t)v * A.rk.stride[f];
      continue;
    }
    const int k = A.rk.k[f];
    if (__popcll(v) != k) return A.dim;
    const int64_t* T = A.rk.tab + A.rk.off[f];
    int64_t acc = 0;
    int cb = 0;
    for (int b = 0; b < A.rk.nb[f]; ++b) {
      const unsigned byte = (unsigned)(v >> (8 * b)) & 255u;
      acc += __ldg(T + ((int64_t)b * 256 + byte) * (k + 1) + cb);
      cb += __popc(byte);
    }
    r += acc * A.rk.stride[f];
  }
  return r;
}

constexpr int kPullCap = 64;

__global__ void __launch_bounds__(128) pull_lower_kernel(PullArgs A, int pass, int64_t* counts,
                                                         const int64_t* rowptr, int32_t* colidx, cplx* vals,
                                                         int* overflow) {
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= A.dim) return;
  const uint64_t s = A.basis[r];
  int n = 0;
  int cols[kPullCap];
  cplx acc[kPullCap];
  for (int e = 0; e < A.nent; ++e) {
    const MfEntry E = A.ent[e];
    if ((s & E.sup) != E.outb) continue;
    const uint64_t c = s ^ E.flip;
    const int64_t col = pull_rank(A, c);
    if (col >= A.dim) continue;  // outside the sector (operator.hpp:196-199)
    cplx v = E.amp;
    if (__popcll(c & E.jw) & 1) v = mkc(-v.re, -v.im);
    int lo = 0, hi = n;
    while (lo < hi) {
      const int mid = (lo + hi) >> 1;
      if (cols[mid] < (int)col) lo = mid + 1;
      else hi = mid;
    }
    if (lo < n && cols[lo] == (int)col) {
      acc[lo] = cadd_rn(acc[lo], v);
    } else {
      if (n >= kPullCap) {
        atomicExch(overflow, 1);
        return;
      }
      for (int q = n; q > lo; --q) {
        cols[q] = cols[q - 1];
        acc[q] = acc[q - 1];
      }
      cols[lo] = (int)col;
      acc[lo] = cadd_rn(mkc(0.0, 0.0), v);
      ++n;
    }
  }
  if (pass == 0) {
    counts[r] = n;
  } else {
    const int64_t o = rowptr[r];
    for (int q = 0; q < n; ++q) {
      colidx[o + q] = cols[q];
      vals[o + q] = acc[q];
    }
  }
}

bool ham_lower_pull(qd_ham* H) {
  std::vector<MfEntry> off, dia;
  try {
    compile_terms(H, off, dia);
  } catch (const Error&) {
    clear_error();
    return false;
  }
  off.insert(off.end(), dia.begin(), dia.end());
  if (off.size() > 4096) return false;
  Ctx* ctx = H->ctx;
  const qd_sector* S = H->sec;
  const int64_t dim = S->view.dim;
  DBuf<MfEntry> dent(std::max<size_t>(off.size(), 1));
  if (!off.empty())
    QD_CUDA(cudaMemcpyAsync(dent.p, off.data(), off.size() * sizeof(MfEntry), cudaMemcpyHostToDevice, ctx->stream));
  PullArgs A;
  std::memset(&A, 0, sizeof(A));
  A.dim = dim;
  A.basis = S->basis.p;
  A.ent = dent.p;
  A.nent = (int)off.size();
  A.S = S->view;
  A.use_tables = (S->view.rank_kind == 1 && S->view.nfields <= 4) ? 1 : 0;
  DBuf<int64_t> tab;
  if (A.use_tables) {
    std::vector<int64_t> ht;
    build_tables(S, A.rk, ht);
    tab.alloc(std::max<size_t>(ht.size(), 1));
    if (!ht.empty())
      QD_CUDA(cudaMemcpyAsync(tab.p, ht.data(), ht.size() * 8, cudaMemcpyHostToDevice, ctx->stream));
    A.rk.tab = tab.p;
  }
  DBuf<int> overflow(1);
  QD_CUDA(cudaMemsetAsync(overflow.p, 0, sizeof(int), ctx->stream));
  DBuf<int64_t> rowptr(dim + 2);
  QD_CUDA(cudaMemsetAsync(rowptr.p, 0, (dim + 2) * 8, ctx->stream));
  const unsigned g = (unsigned)std::max<int64_t>(1, ceil_div(dim, 128));
  if (dim > 0) {
    pull_lower_kernel<<<g, 128, 0, ctx->stream>>>(A, 0, rowptr.p, nullptr, nullptr, nullptr, overflow.p);
    QD_CHECK_LAUNCH();
    QD_LAUNCHED(ctx);
  }
  int ovf = 0;
  QD_CUDA(cudaMemcpyAsync(&ovf, overflow.p, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  QD_CUDA(cudaStreamSynchronize(ctx->stream));
  if (ovf) return false;
  exclusive_scan_i64(ctx, rowptr.p, rowptr.p, dim + 1);
  int64_t nnz = 0;
  QD_CUDA(cudaMemcpyAsync(&nnz, rowptr.p + dim, 8, cudaMemcpyDeviceToHost, ctx->stream));
  QD_CUDA(cudaStreamSynchronize(ctx->stream));
  QD_REQUIRE(nnz < (int64_t)INT32_MAX * 8, QD_ERR_UNSUPPORTED, "nnz too large");
  H->nnz = nnz;
  H->rowptr = std::move(rowptr);
  H->colidx.alloc(nnz + 16);
  H->vals_c.alloc(nnz + 16);
  QD_CUDA(cudaMemsetAsync(H->colidx.p, 0, (nnz + 16) * sizeof(int32_t), ctx->stream));
  QD_CUDA(cudaMemsetAsync(H->vals_c.p, 0, (nnz + 16) * sizeof(cplx), ctx->stream));
  if (dim > 0 && nnz > 0) {
    pull_lower_kernel<<<g, 128, 0, ctx->stream>>>(A, 1, nullptr, H->rowptr.p, H->colidx.p, H->vals_c.p, overflow.p);
    QD_CHECK_LAUNCH();
    QD_LAUNCHED(ctx);
  }
  QD_CUDA(cudaStreamSynchronize(ctx->stream));
  return true;
}

void mf_apply_c(qd_ham* H, const cplx* x, cplx* y) {
  ham_build_matrix_free(H);
  launch_mf<cplx>(H->ctx, H, x, y, 1.0, nullptr, nullptr, 0);
}

}  // namespace qd
