// hamops.cu -- sums and multiples of lowered matrices.
//
// The reference adds lowered SpMatrix values with Eigen's sparse sum: the
// result's pattern is the union of the operands' patterns and each value is
// op(a, b) = a + b, an entry present in one operand only taking a + 0
// (Model::getHamiltonianMatrix, lattice.hpp:339-354; McManager::incrMatrix,
// mc_manager.hpp:72-79).  A multiple scales every stored value by s
// (McManager::normMatrix, mc_manager.hpp:81-83).  Explicit zeros stay.
#include <algorithm>

#include "ham.cuh"
#include "krylov.cuh"
#include "scan.cuh"

namespace qd {

// Union of two ascending column lists: count (pass 0) or write (pass 1).
__global__ void ham_add_kernel(int64_t n, const int64_t* ap, const int32_t* ac, const cplx* av, const int64_t* bp,
                               const int32_t* bc, const cplx* bv, int pass, int64_t* counts, const int64_t* op,
                               int32_t* oc, cplx* ov) {
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
    int64_t i = ap[r], j = bp[r];
    const int64_t ie = ap[r + 1], je = bp[r + 1];
    int64_t o = pass ? op[r] : 0;
    while (i < ie || j < je) {
      const int32_t ci = (i < ie) ? ac[i] : INT32_MAX, cj = (j < je) ? bc[j] : INT32_MAX;
      int32_t c;
      cplx v;
      if (ci == cj) {
        c = ci;
        if (pass) v = mkc(__dadd_rn(av[i].re, bv[j].re), __dadd_rn(av[i].im, bv[j].im));
        ++i;
        ++j;
      } else if (ci < cj) {
        c = ci;
        if (pass) v = mkc(__dadd_rn(av[i].re, 0.0), __dadd_rn(av[i].im, 0.0));
        ++i;
      } else {
        c = cj;
        if (pass) v = mkc(__dadd_rn(0.0, bv[j].re), __dadd_rn(0.0, bv[j].im));
        ++j;
      }
      if (pass) {
        oc[o] = c;
        ov[o] = v;
      }
      ++o;
    }
    if (!pass) counts[r] = o;
  }
}

// v = v * s with one rounding per product and per sum, as std::complex does.
__global__ void ham_scale_kernel(int64_t nnz, cplx* v, cplx s) {
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < nnz; k += (int64_t)gridDim.x * blockDim.x) {
    const cplx a = v[k];
    v[k] = mkc(__dadd_rn(__dmul_rn(a.re, s.re), -__dmul_rn(a.im, s.im)),
               __dadd_rn(__dmul_rn(a.re, s.im), __dmul_rn(a.im, s.re)));
  }
}

static int ops_grid(Ctx* ctx, int64_t n) {
  return (int)std::max<int64_t>(1, std::min<int64_t>(ceil_div(n, 256), (int64_t)ctx->num_sms * 8));
}

void ham_add(const qd_ham* A, const qd_ham* B, qd_ham* H) {
  Ctx* ctx = A->ctx;
  const int64_t n = A->dim;
  H->dim = n;
  DBuf<int64_t> counts(n + 1);
  QD_CUDA(cudaMemsetAsync(counts.p, 0, (n + 1) * sizeof(int64_t), ctx->stream));
  if (n > 0) {
    ham_add_kernel<<<ops_grid(ctx, n), 256, 0, ctx->stream>>>(n, A->rowptr.p, A->colidx.p, A->vals_c.p, B->rowptr.p,
                                                             B->colidx.p, B->vals_c.p, 0, counts.p, nullptr, nullptr,
                                                             nullptr);
    QD_CHECK_LAUNCH();
    QD_LAUNCHED(ctx);
  }
  H->rowptr.alloc(n + 2);
  exclusive_scan_i64(ctx, counts.p, H->rowptr.p, n + 1);
  int64_t nnz = 0;
  QD_CUDA(cudaMemcpyAsync(&nnz, H->rowptr.p + n, sizeof(int64_t), cudaMemcpyDeviceToHost, ctx->stream));
  QD_CUDA(cudaStreamSynchronize(ctx->stream));
  H->nnz = nnz;
  H->colidx.alloc(nnz + 16);
  H->vals_c.alloc(nnz + 16);
  QD_CUDA(cudaMemsetAsync(H->colidx.p, 0, (nnz + 16) * sizeof(int32_t), ctx->stream));
  QD_CUDA(cudaMemsetAsync(H->vals_c.p, 0, (nnz + 16) * sizeof(cplx), ctx->stream));
  if (n > 0 && nnz > 0) {
    ham_add_kernel<<<ops_grid(ctx, n), 256, 0, ctx->stream>>>(n, A->rowptr.p, A->colidx.p, A->vals_c.p, B->rowptr.p,
                                                             B->colidx.p, B->vals_c.p, 1, nullptr, H->rowptr.p,
                                                             H->colidx.p, H->vals_c.p);
    QD_CHECK_LAUNCH();
    QD_LAUNCHED(ctx);
  }
  ham_finish(H);
}

void ham_copy(const qd_ham* A, qd_ham* H) {
  Ctx* ctx = A->ctx;
  const int64_t n = A->dim, nnz = A->nnz;
  H->dim = n;
  H->nnz = nnz;
  H->rowptr.alloc(n + 2);
  H->colidx.alloc(nnz + 16);
  H->vals_c.alloc(nnz + 16);
  QD_CUDA(cudaMemcpyAsync(H->rowptr.p, A->rowptr.p, (n + 1) * sizeof(int64_t), cudaMemcpyDeviceToDevice,
                          ctx->stream));
  QD_CUDA(cudaMemcpyAsync(H->colidx.p, A->colidx.p, (nnz + 16) * sizeof(int32_t), cudaMemcpyDeviceToDevice,
                          ctx->stream));
  QD_CUDA(cudaMemcpyAsync(H->vals_c.p, A->vals_c.p, (nnz + 16) * sizeof(cplx), cudaMemcpyDeviceToDevice,
                          ctx->stream));
  H->host_terms = A->host_terms;
  H->host_gates = A->host_gates;
  H->from_terms = A->from_terms;
  H->spmv_variant = A->spmv_variant;
  ham_finish(H);
}

void ham_scale(qd_ham* H, cplx s) {
  Ctx* ctx = H->ctx;
  if (H->nnz > 0) {
    ham_scale_kernel<<<ops_grid(ctx, H->nnz), 256, 0, ctx->stream>>>(H->nnz, H->vals_c.p, s);
    QD_CHECK_LAUNCH();
    QD_LAUNCHED(ctx);
  }
  // every form derived from the values goes
  H->ws.reset();
  H->arnoldi.reset();
  H->arnoldi_gs.reset();
  H->fx.reset();
  H->fx_state = 0;
  H->mfx.reset();
  H->mfx_state = 0;
  H->fx_allowed = true;
  H->has_mf = false;
  H->mf_ent = DBuf<MfEntry>();
  H->diag_r = DBuf<double>();
  H->diag_c = DBuf<cplx>();
  H->norm_inf = -1.0;
  H->from_terms = false;
  ham_finish(H);
}

}  // namespace qd
