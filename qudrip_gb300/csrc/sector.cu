// sector.cu -- sector construction, basis enumeration and ranking kernels.
#include <algorithm>
#include <cstring>

#include "scan.cuh"
#include "sector.cuh"

namespace qd {

constexpr int kMaxCons = 8;

struct ConsPack {
  int ncons;
  int tight;
  int nbits;
  int pad;
  qd_constraint c[kMaxCons];
};

// Evaluate<tight> over all constraints (conservation.hpp:201-218); quantities
// as Nset::eval (:110-112) and Nd::eval (:141-144).
__device__ __forceinline__ bool accept(const ConsPack& P, uint64_t s) {
  for (int i = 0; i < P.ncons; ++i) {
    const qd_constraint& c = P.c[i];
    int64_t q = 0;
    for (int k = 0; k < c.nterms; ++k) {
      const qd_cq_term& t = c.term[k];
      int64_t v;
      if (t.kind == QD_CQ_NSET) {
        v = __popcll(s & t.mask);
      } else {
        const uint64_t m = t.hole ? ((t.nsite >= 64) ? ~0ull : ((1ull << t.nsite) - 1)) : 0ull;
        const uint64_t sh = (t.nsite >= 64) ? 0ull : (s >> t.nsite);
        v = __popcll((sh ^ m) & (s ^ m));
      }
      q += (int64_t)t.coef * v;
    }
    const int d = (int)(q - c.target);
    if (abs(d) > P.tight) return false;
  }
  return true;
}

constexpr int kScanThreads = 256;
constexpr int kScanRun = 64;  // consecutive states per thread
constexpr int64_t kScanBlockStates = (int64_t)kScanThreads * kScanRun;

__global__ void scan_count_kernel(ConsPack P, uint64_t range, int64_t* block_counts) {
  __shared__ int64_t red[kScanThreads / 32];
  const uint64_t base = (uint64_t)blockIdx.x * kScanBlockStates + (uint64_t)threadIdx.x * kScanRun;
  int cnt = 0;
  for (int i = 0; i < kScanRun; ++i) {
    const uint64_t s = base + i;
    if (s < range && accept(P, s)) ++cnt;
  }
  int64_t v = cnt;
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    int64_t t = 0;
    for (int w = 0; w < kScanThreads / 32; ++w) t += red[w];
    block_counts[blockIdx.x] = t;
  }
}

__global__ void scan_fill_kernel(ConsPack P, uint64_t range, const int64_t* block_offsets,
                                 uint64_t* basis) {
  __shared__ int counts[kScanThreads];
  const uint64_t base = (uint64_t)blockIdx.x * kScanBlockStates + (uint64_t)threadIdx.x * kScanRun;
  int cnt = 0;
  for (int i = 0; i < kScanRun; ++i) {
    const uint64_t s = base + i;
    if (s < range && accept(P, s)) ++cnt;
  }
  counts[threadIdx.x] = cnt;
  __syncthreads();
  // exclusive prefix of the block's thread counts (ascending thread order)
  if (threadIdx.x == 0) {
    int run = 0;
    for (int t = 0; t < kScanThreads; ++t) {
      const int c = counts[t];
      counts[t] = run;
      run += c;
    }
  }
  __syncthreads();
  int64_t pos = block_offsets[blockIdx.x] + counts[threadIdx.x];
  for (int i = 0; i < kScanRun; ++i) {
    const uint64_t s = base + i;
    if (s < range && accept(P, s)) basis[pos++] = s;
  }
}

__global__ void unrank_product_kernel(SectorView S, uint64_t* basis) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= S.dim) return;
  uint64_t s = 0;
  for (int f = 0; f < S.nfields; ++f) {
    const Field& F = S.fields[f];
    const int64_t digit = (i / F.stride) % F.count;
    const uint64_t v = F.is_free ? (uint64_t)digit : cns_unrank(S.binom, F.width, F.k, digit);
    s |= v << F.lo;
  }
  basis[i] = s;
}

// dir[t] = first basis index whose state is >= t << shift.
__global__ void directory_kernel(const uint64_t* basis, int64_t dim, int shift, int64_t ndir,
                                 int64_t* dir) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t > ndir) return;
  const uint64_t key = (uint64_t)t << shift;
  int64_t lo = 0, hi = dim;
  while (lo < hi) {
    const int64_t mid = (lo + hi) >> 1;
    if (basis[mid] < key) lo = mid + 1;
    else hi = mid;
  }
  dir[t] = lo;
}

__global__ void rank_kernel(SectorView S, const uint64_t* states, int64_t n, int64_t* ranks) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) ranks[i] = sector_rank(S, states[i]);
}

// --------------------------------------------------------------- host side
static void fill_binom(std::vector<int64_t>& B) {
  B.assign(kBinomN * kBinomN, 0);
  for (int n = 0; n < kBinomN; ++n) {
    B[n * kBinomN + 0] = 1;
    for (int k = 1; k <= n; ++k) {
      const int64_t a = B[(n - 1) * kBinomN + k - 1];
      const int64_t b = (k <= n - 1) ? B[(n - 1) * kBinomN + k] : 0;
      // saturate instead of overflowing (only n >= 63 could overflow)
      B[n * kBinomN + k] = (a > INT64_MAX - b) ? INT64_MAX : a + b;
    }
  }
}

// Product structure: every constraint a single Nset term, coef 1, tight 0,
// clipped masks contiguous and pairwise disjoint.
static bool detect_product(int nbits, const std::vector<qd_constraint>& cons, int tight,
                           std::vector<Field>& fields) {
  if (tight != 0) return false;
  const uint64_t full = (nbits >= 64) ? ~0ull : ((1ull << nbits) - 1);
  uint64_t covered = 0;
  std::vector<Field> fs;
  for (const auto& c : cons) {
    if (c.nterms != 1 || c.term[0].kind != QD_CQ_NSET || c.term[0].coef != 1) return false;
    const uint64_t m = c.term[0].mask & full;
    if (m == 0) return false;
    if (m & covered) return false;
    const int lo = __builtin_ctzll(m);
    const uint64_t run = m >> lo;
    if ((run & (run + 1)) != 0) return false;  // not contiguous
    const int width = 64 - __builtin_clzll(run);
    Field F{};
    F.lo = lo;
    F.width = width;
    F.k = (int)c.target;
    fs.push_back(F);
    covered |= m;
  }
  // free fields for the uncovered bits
  int b = 0;
  while (b < nbits) {
    if (covered & (1ull << b)) {
      ++b;
      continue;
    }
    int e = b;
    while (e < nbits && !(covered & (1ull << e))) ++e;
    Field F{};
    F.lo = b;
    F.width = e - b;
    F.k = 0;
    F.is_free = 1;
    fs.push_back(F);
    b = e;
  }
  std::sort(fs.begin(), fs.end(), [](const Field& a, const Field& c) { return a.lo < c.lo; });
  if ((int)fs.size() > kMaxFields) return false;
  fields = fs;
  return true;
}

void sector_build(qd_sector* S) {
  Ctx* ctx = S->ctx;
  const int nbits = S->nbits;
  std::vector<int64_t> hb;
  fill_binom(hb);
  S->binom.alloc(hb.size());
  QD_CUDA(cudaMemcpyAsync(S->binom.p, hb.data(), hb.size() * 8, cudaMemcpyHostToDevice, ctx->stream));

  SectorView& V = S->view;
  std::memset(&V, 0, sizeof(V));
  V.nbits = nbits;
  V.binom = S->binom.p;

  std::vector<Field> fields;
  if (detect_product(nbits, S->cons, S->tight, fields)) {
    // dim = prod count; strides from the lowest field up
    int64_t stride = 1;
    bool empty = false;
    for (auto& F : fields) {
      if (F.is_free) {
        QD_REQUIRE(F.width < 40, QD_ERR_UNSUPPORTED, "sector: free field of %d bits too large", F.width);
        F.count = 1ll << F.width;
      } else if (F.k > F.width || F.k < 0) {
        F.count = 0;
        empty = true;
      } else {
        F.count = hb[F.width * kBinomN + F.k];
      }
      F.stride = stride;
      if (F.count > 0) {
        QD_REQUIRE(stride <= (int64_t)INT32_MAX / F.count, QD_ERR_UNSUPPORTED,
                   "sector dimension exceeds 2^31-1");
        stride *= F.count;
      }
    }
    const int64_t dim = empty ? 0 : stride;
    QD_REQUIRE(dim < (int64_t)INT32_MAX, QD_ERR_UNSUPPORTED, "sector dimension %lld exceeds 2^31-1",
               (long long)dim);
    V.rank_kind = 1;
    V.nfields = (int)fields.size();
    for (int f = 0; f < V.nfields; ++f) V.fields[f] = fields[f];
    V.dim = dim;
    S->basis.alloc(dim + 1);
    V.basis = S->basis.p;
    if (dim > 0) {
      unrank_product_kernel<<<(unsigned)ceil_div(dim, 256), 256, 0, ctx->stream>>>(V, S->basis.p);
      QD_CHECK_LAUNCH();
      QD_LAUNCHED(ctx);
    }
    return;
  }

  // generic: ordered scan of the full register
  QD_REQUIRE(nbits <= 40, QD_ERR_UNSUPPORTED,
             "sector: constraints without product structure need nbits <= 40 (got %d)", nbits);
  QD_REQUIRE((int)S->cons.size() <= kMaxCons, QD_ERR_UNSUPPORTED, "at most %d constraints", kMaxCons);
  ConsPack P;
  std::memset(&P, 0, sizeof(P));
  P.ncons = (int)S->cons.size();
  P.tight = S->tight;
  P.nbits = nbits;
  for (int i = 0; i < P.ncons; ++i) P.c[i] = S->cons[i];
  const uint64_t range = 1ull << nbits;
  const int64_t nblocks = ceil_div((int64_t)range, kScanBlockStates);
  DBuf<int64_t> counts(nblocks + 1), offsets(nblocks + 1);
  scan_count_kernel<<<(unsigned)nblocks, kScanThreads, 0, ctx->stream>>>(P, range, counts.p);
  QD_CHECK_LAUNCH();
  QD_LAUNCHED(ctx);
  QD_CUDA(cudaMemsetAsync(counts.p + nblocks, 0, 8, ctx->stream));
  exclusive_scan_i64(ctx, counts.p, offsets.p, nblocks + 1);
  int64_t dim = 0;
  QD_CUDA(cudaMemcpyAsync(&dim, offsets.p + nblocks, 8, cudaMemcpyDeviceToHost, ctx->stream));
  QD_CUDA(cudaStreamSynchronize(ctx->stream));
  QD_REQUIRE(dim < (int64_t)INT32_MAX, QD_ERR_UNSUPPORTED, "sector dimension exceeds 2^31-1");
  S->basis.alloc(dim + 1);
  if (dim > 0) {
    scan_fill_kernel<<<(unsigned)nblocks, kScanThreads, 0, ctx->stream>>>(P, range, offsets.p, S->basis.p);
    QD_CHECK_LAUNCH();
    QD_LAUNCHED(ctx);
  }
  V.rank_kind = 0;
  V.dim = dim;
  V.basis = S->basis.p;
  const int dir_bits = std::min(nbits, 20);
  V.dir_shift = nbits - dir_bits;
  const int64_t ndir = 1ll << dir_bits;
  S->dir.alloc(ndir + 1);
  V.dir = S->dir.p;
  directory_kernel<<<(unsigned)ceil_div(ndir + 1, 256), 256, 0, ctx->stream>>>(S->basis.p, dim, V.dir_shift,
                                                                               ndir, S->dir.p);
  QD_CHECK_LAUNCH();
  QD_LAUNCHED(ctx);
  QD_CUDA(cudaStreamSynchronize(ctx->stream));
}

void sector_rank_device(qd_sector* S, const uint64_t* d_states, int64_t n, int64_t* d_ranks) {
  if (n <= 0) return;
  rank_kernel<<<(unsigned)ceil_div(n, 256), 256, 0, S->ctx->stream>>>(S->view, d_states, n, d_ranks);
  QD_CHECK_LAUNCH();
  QD_LAUNCHED(S->ctx);
}

}  // namespace qd
