// sector.cuh -- conserved-quantity sectors on the device.
//
// Restates Constrain / LooseConstrain (conservation.hpp:200-231) and SubIndex
// (index.hpp:187-261): the basis is every accepted state in ascending integer
// order; rank(state) is its position, or dim when the state is outside.
//
// Two ranking schemes:
//  * product sectors (every constraint is a single popcount on a contiguous
//    bit field, fields disjoint, tight == 0) use the combinatorial number
//    system: rank = sum over fields of (colex rank of the field) * stride.
//    Ascending integer order is lexicographic from the highest field down,
//    and within a field colex rank order equals ascending field value, so
//    this is exactly the reference's order.  Basis generation is an unrank
//    per index, no scan.
//  * every other sector (Nd constraints, combinations, overlapping masks,
//    LooseConstrain) is enumerated by an ordered scan of all 2^nbits states
//    and ranked by a directory on the top bits plus a binary search.
#pragma once

#include "common.cuh"

namespace qd {

constexpr int kMaxFields = 16;
constexpr int kMaxBits = 62;
constexpr int kBinomN = 64;  // binom[n][k] for n, k < 64

struct Field {
  int lo;          // lowest bit
  int width;       // number of bits
  int k;           // popcount target (constrained fields)
  int is_free;     // 1: no constraint on these bits
  int64_t count;   // states of this field
  int64_t stride;  // mixed-radix weight in the rank
};

// Device view of a sector, passed by value to kernels.
struct SectorView {
  int nbits;
  int rank_kind;  // 1 = product (CNS), 0 = directory search
  int nfields;
  int dir_shift;  // search: dir index = state >> dir_shift
  int64_t dim;
  const uint64_t* basis;   // dim states, ascending
  const int64_t* binom;    // kBinomN * kBinomN
  const int64_t* dir;      // (1 << (nbits - dir_shift)) + 1 entries (search only)
  Field fields[kMaxFields];
};

#ifdef __CUDACC__
__device__ __forceinline__ int64_t binom_at(const int64_t* binom, int n, int k) {
  return (k < 0 || k > n) ? 0 : __ldg(binom + n * kBinomN + k);
}

// Colex rank of the set bits of v (j-th set bit at position p adds C(p, j)).
__device__ __forceinline__ int64_t cns_rank(const int64_t* binom, uint64_t v) {
  int64_t r = 0;
  int j = 1;
  while (v) {
    const int p = __ffsll((long long)v) - 1;
    r += binom_at(binom, p, j);
    ++j;
    v &= v - 1;
  }
  return r;
}

// Inverse of cns_rank for a field of `width` bits with `k` set.
__device__ __forceinline__ uint64_t cns_unrank(const int64_t* binom, int width, int k, int64_t r) {
  uint64_t v = 0;
  for (int p = width - 1; p >= 0 && k > 0; --p) {
    const int64_t c = binom_at(binom, p, k);
    if (r >= c) {
      v |= 1ull << p;
      r -= c;
      --k;
    }
  }
  return v;
}

__device__ __forceinline__ int64_t sector_rank(const SectorView& S, uint64_t s) {
  if (S.nbits < 64 && (s >> S.nbits) != 0ull) return S.dim;
  if (S.rank_kind == 1) {
    int64_t r = 0;
    for (int f = 0; f < S.nfields; ++f) {
      const Field& F = S.fields[f];
      const uint64_t v = (s >> F.lo) & ((F.width >= 64) ? ~0ull : ((1ull << F.width) - 1));
      if (F.is_free) {
        r += (int64_t)v * F.stride;
      } else {
        if (__popcll(v) != F.k) return S.dim;
        r += cns_rank(S.binom, v) * F.stride;
      }
    }
    return r;
  }
  const uint64_t t = s >> S.dir_shift;
  int64_t lo = __ldg(S.dir + t), hi = __ldg(S.dir + t + 1);
  while (lo < hi) {
    const int64_t mid = (lo + hi) >> 1;
    const uint64_t b = __ldg(S.basis + mid);
    if (b < s) lo = mid + 1;
    else hi = mid;
  }
  if (lo < S.dim && __ldg(S.basis + lo) == s) return lo;
  return S.dim;
}
#endif

}  // namespace qd

struct qd_sector {
  qd::Ctx* ctx = nullptr;
  int nbits = 0;
  int tight = 0;
  std::vector<qd_constraint> cons;
  qd::SectorView view{};
  qd::DBuf<uint64_t> basis;
  qd::DBuf<int64_t> binom;
  qd::DBuf<int64_t> dir;
};
