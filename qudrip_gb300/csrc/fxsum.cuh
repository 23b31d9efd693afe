// fxsum.cuh -- the product with exact fixed-point sums (uniform couplings).
//
// GB300 issues FP64 FMAs at about 1.9 per clock per SM (1.2 TFLOP/s), so a
// FP64 CSR product at L = 24 spends as long in the FP64 pipe (36.6 M FMAs)
// as in HBM, while the integer pipes idle.  Many of the reference's models
// (XY, XXZ/Heisenberg with fields, any uniform hopping) have one value c on
// every off-diagonal entry; then
//     (H x)_r = d_r x_r + c * sum_{k in row r, k != r} x_k,
// and the sum needs no multiplication.  This form stores the diagonal d and
// the off-diagonal columns (int32, no values), keeps beside every Lanczos
// vector a 128-bit fixed-point copy X = round_toward_zero(x * 2^F), and sums
// X over the row with integer adds: the sum is exact, rounded once to FP64.
// F is fixed per Hamiltonian from the bound |x_i| <= max(1, ||H||_inf) that
// every Lanczos vector obeys (unit start vector; n_k <= ||H||), leaving 7
// bits of headroom for up to 128 summands: F = 119 - ceil(log2(bound)), so
// elements down to 2^-66 of the bound convert exactly and the result is at
// least as accurate as a sequential FP64 sum.  A value above the bound sets
// an overflow flag and the solver reruns on the FP64 CSR product.  (Turning
// each gathered FP64 value into fixed point inside the product instead costs
// about 20 integer instructions per gather, more than the copy saves.)
#pragma once

#include <cstdint>

#include "common.cuh"

namespace qd {

// Columns on the fly (kernel code 121).  When the operator came from terms on
// a product sector of at most 32 bits, the off-diagonal columns of row r
// (state s) are not read from memory but computed from the compiled
// transitions (ham.cuh, MfEntry).  A transition whose support is a contiguous
// run of bits of one field changes the colex rank only inside the run, by an
// amount fixed by the run's input pattern p and the number m of set bits of
// the field below the run: its column is r + delta[p][m].  Such transitions
// are grouped into run slots (one support, at most one transition per input
// pattern), each a shift, a mask, a popcount and one table load per row; the
// table holds the offset and a 0/1 weight, so a slot with no transition for
// the row adds X[r] * 0.
// Other transitions go into rank slots (one support and flip, up to four
// input patterns) and rank s ^ flip by byte tables.  All lanes of a warp take
// the same slot at the same time, so for slots on high bits 32 consecutive
// rows gather 32 consecutive X values.  The slot form is kept only after a
// check over every row that its columns are exactly the stored columns of the
// row, so its integer sums, and its products, are bit-identical to code 120's.
constexpr int kFxSlotWidth = 4;
struct FxSlot {    // rank slot
  uint32_t sup;    // support bits
  uint32_t flip;   // input ^ output on the support
  uint32_t pad[2];
  uint32_t outb[kFxSlotWidth];  // input patterns on the support; unused ones hold ~sup (never match)
};
// run slot (uint4): x = lowest bit of the run, y = run mask (after the shift),
// z = bits of the run's field below the run, w = offset of delta[0][0]; the
// table row of pattern p starts at w + p * kk; entries are {offset, weight}.

// Ranking of a product sector of at most two constrained fields in 32 bits by
// byte tables (mfree.cu builds the same tables for its 32-bit product).
struct Rank32 {
  int nf;
  int lo[2], k[2], nb[2];
  uint32_t wmask[2];
  uint32_t stride[2];
  int off[2];
  const uint32_t* tab;
};

struct FxForm {
  DBuf<int32_t> rowptr;  // dim + 1 (off-diagonal entries only), row by row: the source of the
  DBuf<int32_t> colidx;  // slice layout and of the slot check; columns in gather order (fx_fill_kernel)
  DBuf<double> diag;     // d_r (0 where the CSR has no diagonal entry)
  double c = 0.0;        // the common off-diagonal value
  bool diag_zero = false;  // every diagonal entry is 0 (the one-launch step reads no diagonal)
  int F = 0;             // fixed-point scale 2^F
  int64_t nnz = 0;
  // columns on the fly (code 121)
  int slots_state = 0;     // 0 not tried, 1 built and checked, -1 not applicable
  bool use_slots = false;  // the products take the slot form (code 121) instead of the stored columns
  int nrun = 0;            // run slots, a multiple of 4 (padding slots never match)
  int nslot = 0;           // rank slots, a multiple of 4
  int kk = 0;              // run-table row length: max over fields of k + 1
  int ndtab = 0;
  DBuf<uint4> runs;
  DBuf<FxSlot> slots;
  DBuf<int2> dtab;
  DBuf<uint32_t> basis32;  // the sector's basis in 32 bits
  DBuf<uint32_t> rtab;     // byte tables of Rank32
  Rank32 rank{};
  // the columns as the product reads them: 32-row slices, entry k of row 32 s + l
  // at sell_off[s] + 128 (k / 4) + 4 l + k % 4 (fxsum.cu), the row's count in sell_len
  int64_t sell_cols = 0;  // stored slots, padding included
  mutable int step_fused = 0;  // the last Lanczos step on this form: 1 one launch (fxstep.cuh), -1 two
  // the block layout (code 122, fxblock.cu): rows grouped by the high part of their state
  int blk_state = 0;       // 0 not tried, 1 built and checked, -1 not applicable
  bool use_blk = false;    // the one-launch step (and the plain product) take the block form
  int blk_lowbits = 0, blk_lstride = 0, blk_hstride = 0, blk_ncross = 0;
  uint32_t blk_cross[24];  // crossing transitions: support, input pattern, flip
  DBuf<uint32_t> blk_state32;  // the basis in 32 bits
  DBuf<int32_t> blk_off;       // first row of each high part's block (-1: none)
  DBuf<uint16_t> blk_rank;     // rank of each low part among those of its popcount
  DBuf<uint8_t> blk_ldeg;      // targets of each low part ...
  DBuf<uint16_t> blk_ladj;     // ... as positions in the block
  DBuf<uint8_t> blk_hdeg;      // target blocks of each high part ...
  DBuf<int32_t> blk_hadj;      // ... as their first rows
  // the staged one-launch step: groups of whole blocks (rows [x, y)), contiguous runs of groups per CTA
  int blk_part_state = 0;      // 0 not tried, 1 built, -1 the step does not fit
  int blk_nctas = 0, blk_threads = 0, blk_max_group = 0, blk_max_cta = 0;
  size_t blk_smem = 0;
  DBuf<int2> blk_groups;
  DBuf<int32_t> blk_cta_first;
  DBuf<int64_t> sell_off;
  DBuf<int32_t> sell_col;
  DBuf<uint8_t> sell_len;
};

#ifdef __CUDACC__
// x * 2^F rounded toward zero into a signed 128-bit integer; flags |x| >= 2^(126 - 7 - F).
__device__ __forceinline__ __int128 fx_from_double(double x, int F, int* ovf) {
  const unsigned long long bits = (unsigned long long)__double_as_longlong(x);
  const int e = (int)((bits >> 52) & 0x7ffu);
  if (e == 0) return 0;  // zero or subnormal: below the quantum
  const unsigned long long m = (bits & 0xfffffffffffffull) | (1ull << 52);
  const int sh = e - 1075 + F;  // x * 2^F = m * 2^sh
  unsigned __int128 v;
  if (sh >= 0) {
    if (sh > 126 - 7 - 53) {
      if (ovf) *ovf = 1;
      return 0;
    }
    v = (unsigned __int128)m << sh;
  } else if (sh > -64) {
    v = (unsigned __int128)(m >> (-sh));
  } else {
    v = 0;
  }
  const __int128 s = (__int128)v;
  return (bits >> 63) ? -s : s;
}
#endif

}  // namespace qd
