// ham.cuh -- a lowered Hamiltonian held on the device.
//
// Layout in HBM:
//   rowptr  int64[dim+1]   CSR row pointers
//   colidx  int32[nnz]     columns, ascending within each row
//   vals_c  cplx[nnz]      complex128 values (bit-identical to the reference)
//   vals_r  double[nnz]    real part, only when every imaginary part is 0
//   diag_r  double[dim]    real diagonal (matrix-free path)
// The reference's CSC layout is produced on demand by transposing.
#pragma once

#include <memory>

#include "common.cuh"
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

// Matrix-free description: the Hamiltonian split into a diagonal (stored)
// and off-diagonal "flip" terms, each acting on a small support.
struct MfTerm {
  uint64_t support;   // bits the term changes or reads
  uint64_t jw_mask;   // bits outside the support whose parity flips the sign
  int nsup;           // number of support bits (<= kMfMaxSupport)
  int ntrans;         // transitions stored at trans_offset
  int trans_offset;
  int pad;
};

struct MfTrans {
  uint32_t in_local;   // local input configuration (support bits compressed)
  uint32_t out_local;  // local output configuration
  cplx amp;            // coefficient * product of gate amplitudes (sign from jw_mask excluded)
};

constexpr int kMfMaxSupport = 6;

}  // namespace qd

struct qd_ham {
  qd::Ctx* ctx = nullptr;
  qd_sector* sec = nullptr;
  int64_t dim = 0;
  int64_t nnz = 0;
  int flags = 0;
  int max_row_nnz = 0;
  int spmv_variant = 110;  // CSR product kernel the solvers launch (krylov.cuh SpmvVariant)
  qd::DBuf<int64_t> rowptr;
  qd::DBuf<int32_t> colidx;
  qd::DBuf<cplx> vals_c;
  qd::DBuf<double> vals_r;
  qd::DBuf<float> vals_f;  // fp32 copy of vals_r for the mixed-precision SpMV
  qd::DBuf<int32_t> row_order;  // rows by decreasing length inside 256-row windows (kernel 111)
  // matrix-free form
  bool has_mf = false;
  qd::DBuf<double> diag_r;
  qd::DBuf<qd::MfTerm> mf_terms;
  qd::DBuf<qd::MfTrans> mf_trans;
  int mf_nterms = 0;
  double mf_uniform_amp = 0.0;  // when every off-diagonal transition has this real amplitude
  std::vector<qd_term> host_terms;
  std::vector<qd_gate> host_gates;
  std::unique_ptr<qd::Workspace, qd::WorkspaceDeleter> ws;  // solver buffers, reused across calls
  std::unique_ptr<qd::ArnoldiBuffers, qd::ArnoldiDeleter> arnoldi;
};

namespace qd {
void ham_lower(qd_ham* H, const qd_term* terms, int nterms, const qd_gate* gates, int ngates);
void ham_transpose(Ctx* ctx, int64_t n, const int64_t* ptr, const int32_t* idx, const cplx* vals,
                   int64_t nnz, int64_t* out_ptr, int32_t* out_idx, cplx* out_vals);
void ham_build_matrix_free(qd_ham* H);
void ham_ensure_row_order(qd_ham* H);
}  // namespace qd
