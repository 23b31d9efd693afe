// ham.cuh -- a lowered Hamiltonian held on the device.
//
// Layout in HBM:
//   rowptr  int64[dim+1]   CSR row pointers
//   colidx  int32[nnz]     columns, ascending within each row
//   vals_c  cplx[nnz]      complex128 values (bit-identical to the reference)
//   vals_r  double[nnz]    real part, only when every imaginary part is 0
//   diag_r  double[dim]    diagonal of the matrix-free form (diag_c if complex)
// The reference's CSC layout is produced on demand by transposing.
#pragma once

#include <memory>

#include "common.cuh"
#include "fxsum.cuh"
#include "sector.cuh"

namespace qd {

struct Workspace;
struct WorkspaceDeleter {
  void operator()(Workspace* w) const;
};
struct ArnoldiBuffers;
struct ArnoldiDeleter {
  void operator()(ArnoldiBuffers* b) const;
};
struct ArnoldiGround;
struct ArnoldiGroundDeleter {
  void operator()(ArnoldiGround* b) const;
};

struct GateDev {
  int kind, site, site_b, string;
  cplx u[4];  // u[b*2 + o] = amplitude from input bit b to output bit o = U(b, o)
};

struct TermDev {
  cplx coeff;
  int gate_offset;
  int ngates;
  int nbit;  // bit gates in this product (each doubles the leaves)
  int pad;
};

// Matrix-free form: the operator compiled into "entries", one per (term,
// input pattern on the term's support) that changes the state.  Row r
// (state s) receives amp * sign * x[rank(c)] from every entry with
// (s & sup) == outb, where c = s ^ flip and sign = (-1)^popcount(c & jw)
// (the Jordan-Wigner parity of the bits outside the support).  Entries that
// keep the state are summed once into the stored diagonal.
struct MfEntry {
  uint64_t sup;   // support bits of the term
  uint64_t outb;  // output pattern (support bits of the row state)
  uint64_t flip;  // input ^ output
  uint64_t jw;    // bits outside the support whose parity flips the sign
  cplx amp;       // coefficient * leaf sum (sign from jw excluded)
};

// Ranking of a product sector by byte tables: for field f, byte b of its
// value v, and cb set bits below that byte, tab[off_f + (b * 256 + byte) *
// (k_f + 1) + cb] is the byte's share of the colex rank.
struct MfRank {
  int nf;
  int pad;
  int lo[4], width[4], k[4], is_free[4], nb[4];
  int64_t stride[4];
  int64_t off[4];
  const int64_t* tab;
};

constexpr int kMfMaxSupport = 6;
constexpr int kMfMaxEntries = 512;

}  // namespace qd

struct qd_ham {
  qd::Ctx* ctx = nullptr;
  qd_sector* sec = nullptr;
  int64_t dim = 0;
  int64_t nnz = 0;
  int flags = 0;
  int max_row_nnz = 0;
  double norm_inf = -1.0;  // max row sum of |H| (ham_norm_inf), -1 until computed
  int spmv_variant = 110;  // CSR product kernel the solvers launch (krylov.cuh SpmvVariant)
  qd::DBuf<int64_t> rowptr;
  qd::DBuf<int32_t> colidx;
  qd::DBuf<cplx> vals_c;
  qd::DBuf<double> vals_r;
  qd::DBuf<float> vals_f;  // fp32 copy of vals_r for the mixed-precision SpMV
  qd::DBuf<int32_t> row_order;  // rows by decreasing length inside 256-row windows (kernel 111)
  // the batched solver's check for one common off-diagonal FP32 value (batch.cu): run once,
  // dropped when the matrix changes; bun_d holds d_r - c per row (0 where the row stores no
  // diagonal), then c, then the flag (1 when the value is common) as an int
  bool bun_checked = false;
  qd::DBuf<float> bun_d;
  // uniform-coupling form with exact fixed-point sums (fxsum.cuh)
  int fx_state = 0;          // 0 not tried, 1 built, -1 not applicable
  bool fx_allowed = true;    // the Lanczos product uses it when built (kernel code 120)
  std::unique_ptr<qd::FxForm> fx;
  int mfx_state = 0;                 // the same form built from the terms alone (matrix-free Lanczos)
  std::unique_ptr<qd::FxForm> mfx;
  // matrix-free form (qd_ham_build_matrix_free)
  bool has_mf = false;
  bool mf_real = false;      // every amplitude and diagonal entry is real
  bool mf_tables = false;    // product sector ranked by byte tables (else sector_rank)
  int mf_nent = 0;
  qd::DBuf<qd::MfEntry> mf_ent;
  qd::DBuf<double> diag_r;   // real diagonal (mf_real)
  qd::DBuf<cplx> diag_c;     // complex diagonal
  qd::DBuf<int64_t> mf_tab;
  qd::DBuf<uint32_t> mf_tab32;  // the tables in 32 bits (registers of at most 32 bits)
  qd::MfRank mf_rank{};
  std::vector<qd_term> host_terms;
  std::vector<qd_gate> host_gates;
  bool from_terms = false;  // the values are the lowering of host_terms (not a sum or a multiple of matrices)
  bool one_shot = false;    // solved once (a served request): launch directly instead of capturing a graph
  std::unique_ptr<qd::Workspace, qd::WorkspaceDeleter> ws;  // solver buffers, reused across calls
  std::unique_ptr<qd::ArnoldiBuffers, qd::ArnoldiDeleter> arnoldi;
  std::unique_ptr<qd::ArnoldiGround, qd::ArnoldiGroundDeleter> arnoldi_gs;  // Arnoldi ground-state solve
  double arnoldi_gs_ritz = 0.0;  // its last lowest eigenvalue (the error of a grown solve)
};

namespace qd {
void ham_lower(qd_ham* H, const qd_term* terms, int nterms, const qd_gate* gates, int ngates);
void ham_finish(qd_ham* H);
void ham_add(const qd_ham* A, const qd_ham* B, qd_ham* out);
void ham_copy(const qd_ham* A, qd_ham* out);
void ham_scale(qd_ham* H, cplx s);
void ham_transpose(Ctx* ctx, int64_t n, const int64_t* ptr, const int32_t* idx, const cplx* vals,
                   int64_t nnz, int64_t* out_ptr, int32_t* out_idx, cplx* out_vals);
void ham_build_matrix_free(qd_ham* H);
void compile_terms(const qd_ham* H, std::vector<MfEntry>& off, std::vector<MfEntry>& dia);
void build_tables(const qd_sector* S, MfRank& rk, std::vector<int64_t>& tab);
bool ham_build_fx_slots(qd_ham* H);
bool ham_build_fx_block(qd_ham* H);
bool ham_build_mf_fx_block(qd_ham* H);
bool ham_build_mf_fx(qd_ham* H);
bool ham_lower_pull(qd_ham* H);
void mf_apply_c(qd_ham* H, const cplx* x, cplx* y);
bool ham_build_fx(qd_ham* H);
void launch_fx(Ctx* ctx, const qd_ham* H, const FxForm& f, const double* x, const __int128* X, double* y,
               const double* scale_dev, const int* stop, int step);
void launch_fx_shadow(Ctx* ctx, int64_t n, const double* x, __int128* X, int F, int* ovf);
void ham_ensure_row_order(qd_ham* H);
double ham_norm_inf(qd_ham* H);
double ham_gershgorin_halfwidth(qd_ham* H);
}  // namespace qd
