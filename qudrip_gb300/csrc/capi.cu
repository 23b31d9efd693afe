// capi.cu -- the extern "C" boundary declared in include/qudrip_gb300.h.
#include <cstdarg>
#include <cstring>
#include <string>

#include "batch.cuh"
#include "kbatch.cuh"
#include "traj.cuh"
#include "evolve.cuh"
#include "ham.cuh"
#include "krylov.cuh"
#include "sector.cuh"

namespace qd {

static thread_local std::string g_last_error;

void set_error(const char* fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_last_error = buf;
}

void clear_error() { g_last_error.clear(); }

void WorkspaceDeleter::operator()(Workspace* w) const { delete w; }

void sector_build(qd_sector* S);
void sector_rank_device(qd_sector* S, const uint64_t* d_states, int64_t n, int64_t* d_ranks);

}  // namespace qd

struct qd_ctx : qd::Ctx {};

struct qd_state {
  qd::Ctx* ctx = nullptr;
  int64_t dim = 0;
  int nt = 0;
  int64_t ld = 0;
  qd::DBuf<cplx> data;  // nt columns of ld entries
  cplx* col(int t) { return data.p + (int64_t)t * ld; }
};

using namespace qd;

extern "C" {

int qd_api_version(void) { return QD_API_VERSION; }

const char* qd_status_string(qd_status s) {
  switch (s) {
    case QD_OK: return "ok";
    case QD_ERR_INVALID: return "invalid argument";
    case QD_ERR_OOM: return "device out of memory";
    case QD_ERR_CUDA: return "CUDA error";
    case QD_ERR_BREAKDOWN: return "Krylov breakdown";
    case QD_ERR_TIMEOUT: return "device wait timed out";
    case QD_ERR_UNSUPPORTED: return "unsupported";
    case QD_ERR_OVERFLOW: return "overflow";
    case QD_ERR_NOT_HERMITIAN: return "operator is not Hermitian";
    case QD_ERR_BUSY: return "busy";
    default: return "unknown status";
  }
}

const char* qd_last_error(void) { return g_last_error.c_str(); }

// ------------------------------------------------------------------ context
qd_status qd_ctx_create(int device, qd_ctx** out) {
  return guard([&] {
    QD_REQUIRE(out != nullptr, QD_ERR_INVALID, "qd_ctx_create: null output");
    int ndev = 0;
    QD_CUDA(cudaGetDeviceCount(&ndev));
    QD_REQUIRE(device >= 0 && device < ndev, QD_ERR_INVALID, "qd_ctx_create: device %d of %d", device, ndev);
    QD_CUDA(cudaSetDevice(device));
    auto* c = new qd_ctx();
    c->device = device;
    cudaError_t e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
      delete c;
      QD_CUDA(e);
    }
    QD_CUDA(cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, device));
    for (auto& ev : c->events) QD_CUDA(cudaEventCreate(&ev));
    *out = c;
  });
}

qd_status qd_ctx_destroy(qd_ctx* ctx) {
  return guard([&] {
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    for (auto& ev : ctx->events)
      if (ev) cudaEventDestroy(ev);
    cudaStreamDestroy(ctx->stream);
    delete ctx;
  });
}

qd_status qd_ctx_sync(qd_ctx* ctx) {
  return guard([&] {
    QD_REQUIRE(ctx, QD_ERR_INVALID, "null context");
    QD_CUDA(cudaStreamSynchronize(ctx->stream));
  });
}

qd_status qd_ctx_stream(qd_ctx* ctx, void** stream_out) {
  return guard([&] {
    QD_REQUIRE(ctx && stream_out, QD_ERR_INVALID, "null argument");
    *stream_out = (void*)ctx->stream;
  });
}

qd_status qd_ctx_launch_count(qd_ctx* ctx, int64_t* count) {
  return guard([&] {
    QD_REQUIRE(ctx && count, QD_ERR_INVALID, "null argument");
    *count = ctx->launches;
  });
}

qd_status qd_ctx_record(qd_ctx* ctx, int slot) {
  return guard([&] {
    QD_REQUIRE(ctx && slot >= 0 && slot < 16, QD_ERR_INVALID, "bad event slot");
    QD_CUDA(cudaEventRecord(ctx->events[slot], ctx->stream));
  });
}

qd_status qd_ctx_elapsed(qd_ctx* ctx, int a, int b, float* ms) {
  return guard([&] {
    QD_REQUIRE(ctx && ms && a >= 0 && a < 16 && b >= 0 && b < 16, QD_ERR_INVALID, "bad event slot");
    QD_CUDA(cudaEventSynchronize(ctx->events[b]));
    QD_CUDA(cudaEventElapsedTime(ms, ctx->events[a], ctx->events[b]));
  });
}

qd_status qd_host_alloc(int64_t bytes, void** out) {
  return guard([&] {
    QD_REQUIRE(out && bytes > 0, QD_ERR_INVALID, "bad argument");
    QD_CUDA(cudaHostAlloc(out, (size_t)bytes, cudaHostAllocDefault));
  });
}

qd_status qd_host_free(void* p) {
  return guard([&] {
    if (p) QD_CUDA(cudaFreeHost(p));
  });
}

// ------------------------------------------------------------------ sectors
qd_status qd_sector_create(qd_ctx* ctx, int nbits, const qd_constraint* cons, int ncons, int tight,
                           qd_sector** out) {
  return guard([&] {
    QD_REQUIRE(ctx && out, QD_ERR_INVALID, "qd_sector_create: null argument");
    QD_REQUIRE(nbits >= 1 && nbits <= kMaxBits, QD_ERR_INVALID, "nbits must be in 1..%d", kMaxBits);
    QD_REQUIRE(ncons >= 0 && (ncons == 0 || cons), QD_ERR_INVALID, "bad constraint array");
    QD_REQUIRE(tight >= 0, QD_ERR_INVALID, "tight must be >= 0");
    for (int i = 0; i < ncons; ++i) {
      QD_REQUIRE(cons[i].nterms >= 1 && cons[i].nterms <= 4, QD_ERR_INVALID, "constraint %d: 1..4 terms", i);
      for (int k = 0; k < cons[i].nterms; ++k) {
        const qd_cq_term& t = cons[i].term[k];
        QD_REQUIRE(t.kind == QD_CQ_NSET || t.kind == QD_CQ_ND, QD_ERR_INVALID, "constraint %d: bad kind", i);
        QD_REQUIRE(t.kind != QD_CQ_ND || (t.nsite >= 1 && 2 * t.nsite <= 64), QD_ERR_INVALID,
                   "constraint %d: Nd needs 1 <= nsite <= 32", i);
      }
    }
    DeviceGuard dg(ctx->device);
    auto* S = new qd_sector();
    S->ctx = ctx;
    S->nbits = nbits;
    S->tight = tight;
    S->cons.assign(cons, cons + ncons);
    try {
      sector_build(S);
    } catch (...) {
      delete S;
      throw;
    }
    *out = S;
  });
}

qd_status qd_sector_destroy(qd_sector* sec) {
  return guard([&] {
    if (!sec) return;
    DeviceGuard dg(sec->ctx->device);
    cudaStreamSynchronize(sec->ctx->stream);
    delete sec;
  });
}

qd_status qd_sector_dim(const qd_sector* sec, int64_t* dim) {
  return guard([&] {
    QD_REQUIRE(sec && dim, QD_ERR_INVALID, "null argument");
    *dim = sec->view.dim;
  });
}

qd_status qd_sector_rank_kind(const qd_sector* sec, int* kind) {
  return guard([&] {
    QD_REQUIRE(sec && kind, QD_ERR_INVALID, "null argument");
    *kind = sec->view.rank_kind;
  });
}

qd_status qd_sector_basis(qd_sector* sec, uint64_t* host_states) {
  return guard([&] {
    QD_REQUIRE(sec && (host_states || sec->view.dim == 0), QD_ERR_INVALID, "null argument");
    DeviceGuard dg(sec->ctx->device);
    if (sec->view.dim == 0) return;
    QD_CUDA(cudaMemcpyAsync(host_states, sec->basis.p, sec->view.dim * 8, cudaMemcpyDeviceToHost,
                            sec->ctx->stream));
    QD_CUDA(cudaStreamSynchronize(sec->ctx->stream));
  });
}

qd_status qd_sector_rank(qd_sector* sec, const uint64_t* host_states, int64_t n, int64_t* host_ranks) {
  return guard([&] {
    QD_REQUIRE(sec && n >= 0 && (n == 0 || (host_states && host_ranks)), QD_ERR_INVALID, "bad argument");
    if (n == 0) return;
    DeviceGuard dg(sec->ctx->device);
    DBuf<uint64_t> s(n);
    DBuf<int64_t> r(n);
    QD_CUDA(cudaMemcpyAsync(s.p, host_states, n * 8, cudaMemcpyHostToDevice, sec->ctx->stream));
    sector_rank_device(sec, s.p, n, r.p);
    QD_CUDA(cudaMemcpyAsync(host_ranks, r.p, n * 8, cudaMemcpyDeviceToHost, sec->ctx->stream));
    QD_CUDA(cudaStreamSynchronize(sec->ctx->stream));
  });
}

// ------------------------------------------------------------------ Hamiltonians
qd_status qd_ham_lower(qd_sector* sec, const qd_term* terms, int nterms, const qd_gate* gates, int ngates,
                       qd_ham** out) {
  return guard([&] {
    QD_REQUIRE(sec && out, QD_ERR_INVALID, "qd_ham_lower: null argument");
    QD_REQUIRE(nterms >= 0 && (nterms == 0 || terms), QD_ERR_INVALID, "bad term array");
    QD_REQUIRE(ngates >= 0 && (ngates == 0 || gates), QD_ERR_INVALID, "bad gate array");
    DeviceGuard dg(sec->ctx->device);
    auto* H = new qd_ham();
    H->ctx = sec->ctx;
    H->sec = sec;
    try {
      ham_lower(H, terms, nterms, gates, ngates);
    } catch (...) {
      delete H;
      throw;
    }
    *out = H;
  });
}

qd_status qd_ham_add(const qd_ham* a, const qd_ham* b, qd_ham** out) {
  return guard([&] {
    QD_REQUIRE(a && b && out, QD_ERR_INVALID, "qd_ham_add: null argument");
    QD_REQUIRE(a->sec == b->sec, QD_ERR_INVALID, "qd_ham_add: the operands live on different sectors");
    DeviceGuard dg(a->ctx->device);
    auto* H = new qd_ham();
    H->ctx = a->ctx;
    H->sec = a->sec;
    try {
      ham_add(a, b, H);
    } catch (...) {
      delete H;
      throw;
    }
    *out = H;
  });
}

qd_status qd_ham_copy(const qd_ham* a, qd_ham** out) {
  return guard([&] {
    QD_REQUIRE(a && out, QD_ERR_INVALID, "qd_ham_copy: null argument");
    DeviceGuard dg(a->ctx->device);
    auto* H = new qd_ham();
    H->ctx = a->ctx;
    H->sec = a->sec;
    try {
      ham_copy(a, H);
    } catch (...) {
      delete H;
      throw;
    }
    *out = H;
  });
}

qd_status qd_ham_scale(qd_ham* ham, double re, double im) {
  return guard([&] {
    QD_REQUIRE(ham, QD_ERR_INVALID, "qd_ham_scale: null argument");
    DeviceGuard dg(ham->ctx->device);
    ham_scale(ham, mkc(re, im));
  });
}

qd_status qd_ham_destroy(qd_ham* ham) {
  return guard([&] {
    if (!ham) return;
    DeviceGuard dg(ham->ctx->device);
    cudaStreamSynchronize(ham->ctx->stream);
    delete ham;
  });
}

qd_status qd_ham_get_info(qd_ham* ham, qd_ham_info* info) {
  return guard([&] {
    QD_REQUIRE(ham && info, QD_ERR_INVALID, "null argument");
    std::memset(info, 0, sizeof(*info));
    info->dim = ham->dim;
    info->nnz = ham->nnz;
    info->flags = ham->flags;
    info->max_row_nnz = ham->max_row_nnz;
    info->has_matrix_free = ham->has_mf ? 1 : 0;
    info->product_kernel = ham->spmv_variant;
    if ((ham->flags & QD_HAM_REAL) && ham->fx_allowed && ham_build_fx(ham))
      info->product_kernel = (ham->fx->use_blk && ham->fx->blk_state > 0)
                                 ? kSpmvFxBlock
                                 : ((ham->fx->use_slots && ham->fx->slots_state > 0) ? kSpmvFxSlots : kSpmvFx);
    if (ham->fx && ham->fx->step_fused) info->step_launches = ham->fx->step_fused > 0 ? 1 : 2;
  });
}

qd_status qd_ham_build_matrix_free(qd_ham* ham) {
  return guard([&] {
    QD_REQUIRE(ham, QD_ERR_INVALID, "null argument");
    DeviceGuard dg(ham->ctx->device);
    ham_build_matrix_free(ham);
  });
}

qd_status qd_ham_apply_matrix_free(qd_ham* ham, qd_state* x, int t_in, qd_state* y, int t_out) {
  return guard([&] {
    QD_REQUIRE(ham && x && y, QD_ERR_INVALID, "null argument");
    QD_REQUIRE(x->dim == ham->dim && y->dim == ham->dim, QD_ERR_INVALID, "dimension mismatch");
    QD_REQUIRE(t_in >= 0 && t_in < x->nt && t_out >= 0 && t_out < y->nt, QD_ERR_INVALID, "bad column");
    QD_REQUIRE(x->col(t_in) != y->col(t_out), QD_ERR_INVALID, "in-place product");
    DeviceGuard dg(ham->ctx->device);
    mf_apply_c(ham, x->col(t_in), y->col(t_out));
    QD_CUDA(cudaStreamSynchronize(ham->ctx->stream));
  });
}

qd_status qd_ham_download_csr(qd_ham* ham, int64_t* rowptr, int32_t* colidx, double* vals) {
  return guard([&] {
    QD_REQUIRE(ham && rowptr, QD_ERR_INVALID, "null argument");
    DeviceGuard dg(ham->ctx->device);
    cudaStream_t s = ham->ctx->stream;
    QD_CUDA(cudaMemcpyAsync(rowptr, ham->rowptr.p, (ham->dim + 1) * 8, cudaMemcpyDeviceToHost, s));
    if (ham->nnz > 0) {
      QD_REQUIRE(colidx && vals, QD_ERR_INVALID, "null argument");
      QD_CUDA(cudaMemcpyAsync(colidx, ham->colidx.p, ham->nnz * 4, cudaMemcpyDeviceToHost, s));
      QD_CUDA(cudaMemcpyAsync(vals, ham->vals_c.p, ham->nnz * sizeof(cplx), cudaMemcpyDeviceToHost, s));
    }
    QD_CUDA(cudaStreamSynchronize(s));
  });
}

qd_status qd_ham_download_csc(qd_ham* ham, int64_t* colptr, int32_t* rowidx, double* vals) {
  return guard([&] {
    QD_REQUIRE(ham && colptr, QD_ERR_INVALID, "null argument");
    DeviceGuard dg(ham->ctx->device);
    cudaStream_t s = ham->ctx->stream;
    DBuf<int64_t> cp(ham->dim + 1);
    DBuf<int32_t> ri(ham->nnz + 1);
    DBuf<cplx> cv(ham->nnz + 1);
    ham_transpose(ham->ctx, ham->dim, ham->rowptr.p, ham->colidx.p, ham->vals_c.p, ham->nnz, cp.p, ri.p, cv.p);
    QD_CUDA(cudaMemcpyAsync(colptr, cp.p, (ham->dim + 1) * 8, cudaMemcpyDeviceToHost, s));
    if (ham->nnz > 0) {
      QD_REQUIRE(rowidx && vals, QD_ERR_INVALID, "null argument");
      QD_CUDA(cudaMemcpyAsync(rowidx, ri.p, ham->nnz * 4, cudaMemcpyDeviceToHost, s));
      QD_CUDA(cudaMemcpyAsync(vals, cv.p, ham->nnz * sizeof(cplx), cudaMemcpyDeviceToHost, s));
    }
    QD_CUDA(cudaStreamSynchronize(s));
  });
}

// ------------------------------------------------------------------ states
qd_status qd_state_create(qd_ctx* ctx, int64_t dim, int nt, qd_state** out) {
  return guard([&] {
    QD_REQUIRE(ctx && out, QD_ERR_INVALID, "null argument");
    QD_REQUIRE(dim >= 1 && nt >= 1, QD_ERR_INVALID, "state needs dim >= 1 and nt >= 1");
    DeviceGuard dg(ctx->device);
    auto* st = new qd_state();
    st->ctx = ctx;
    st->dim = dim;
    st->nt = nt;
    st->ld = (dim + 31) / 32 * 32;
    try {
      st->data.alloc((size_t)st->ld * nt);
      QD_CUDA(cudaMemsetAsync(st->data.p, 0, st->data.bytes(), ctx->stream));  // Matrix::Zero (state.hpp:29)
      QD_CUDA(cudaStreamSynchronize(ctx->stream));
    } catch (...) {
      delete st;
      throw;
    }
    *out = st;
  });
}

qd_status qd_state_destroy(qd_state* st) {
  return guard([&] {
    if (!st) return;
    DeviceGuard dg(st->ctx->device);
    cudaStreamSynchronize(st->ctx->stream);
    delete st;
  });
}

qd_status qd_state_upload(qd_state* st, int t, const double* host_complex) {
  return guard([&] {
    QD_REQUIRE(st && host_complex && t >= 0 && t < st->nt, QD_ERR_INVALID, "bad argument");
    DeviceGuard dg(st->ctx->device);
    QD_CUDA(cudaMemcpyAsync(st->col(t), host_complex, st->dim * sizeof(cplx), cudaMemcpyHostToDevice,
                            st->ctx->stream));
    QD_CUDA(cudaStreamSynchronize(st->ctx->stream));
  });
}

qd_status qd_state_download(qd_state* st, int t, double* host_complex) {
  return guard([&] {
    QD_REQUIRE(st && host_complex && t >= 0 && t < st->nt, QD_ERR_INVALID, "bad argument");
    DeviceGuard dg(st->ctx->device);
    QD_CUDA(cudaMemcpyAsync(host_complex, st->col(t), st->dim * sizeof(cplx), cudaMemcpyDeviceToHost,
                            st->ctx->stream));
    QD_CUDA(cudaStreamSynchronize(st->ctx->stream));
  });
}

qd_status qd_state_copy(qd_state* src, int t_src, qd_state* dst, int t_dst) {
  return guard([&] {
    QD_REQUIRE(src && dst && src->dim == dst->dim, QD_ERR_INVALID, "bad argument");
    QD_REQUIRE(t_src >= 0 && t_src < src->nt && t_dst >= 0 && t_dst < dst->nt, QD_ERR_INVALID, "bad column");
    QD_REQUIRE(src->ctx == dst->ctx, QD_ERR_INVALID, "states of different contexts");
    DeviceGuard dg(src->ctx->device);
    QD_CUDA(cudaMemcpyAsync(dst->col(t_dst), src->col(t_src), src->dim * sizeof(cplx), cudaMemcpyDeviceToDevice,
                            src->ctx->stream));
  });
}

qd_status qd_state_device_ptr(qd_state* st, int t, void** dptr) {
  return guard([&] {
    QD_REQUIRE(st && dptr && t >= 0 && t < st->nt, QD_ERR_INVALID, "bad argument");
    *dptr = (void*)st->col(t);
  });
}

qd_status qd_ham_apply(qd_ham* ham, qd_state* x, int t_in, qd_state* y, int t_out) {
  return guard([&] {
    QD_REQUIRE(ham && x && y, QD_ERR_INVALID, "null argument");
    QD_REQUIRE(x->dim == ham->dim && y->dim == ham->dim, QD_ERR_INVALID, "dimension mismatch");
    QD_REQUIRE(t_in >= 0 && t_in < x->nt && t_out >= 0 && t_out < y->nt, QD_ERR_INVALID, "bad column");
    QD_REQUIRE(!(x == y && t_in == t_out), QD_ERR_INVALID, "qd_ham_apply cannot work in place");
    DeviceGuard dg(ham->ctx->device);
    ham_apply_c(ham, x->col(t_in), y->col(t_out));
    QD_CUDA(cudaStreamSynchronize(ham->ctx->stream));
  });
}

qd_status qd_state_eval(qd_state* psi, int t, qd_ham* ham, double* re_im) {
  return guard([&] {
    QD_REQUIRE(psi && ham && re_im && t >= 0 && t < psi->nt, QD_ERR_INVALID, "bad argument");
    // the reference only prints on a dimension mismatch (state.hpp:35-39); here it is an error
    QD_REQUIRE(psi->dim == ham->dim, QD_ERR_INVALID, "State::eval: dimension mismatch (%lld vs %lld)",
               (long long)psi->dim, (long long)ham->dim);
    DeviceGuard dg(ham->ctx->device);
    const cplx e = state_eval(ham, psi->col(t));
    re_im[0] = e.re;
    re_im[1] = e.im;
  });
}

qd_status qd_obs_eval(qd_state* psi, int t, int nobs, qd_ham* const* obs, double* re_im) {
  return guard([&] {
    QD_REQUIRE(psi && obs && re_im && nobs >= 1 && t >= 0 && t < psi->nt, QD_ERR_INVALID, "bad argument");
    for (int i = 0; i < nobs; ++i)
      QD_REQUIRE(obs[i] && obs[i]->dim == psi->dim && obs[i]->ctx == psi->ctx, QD_ERR_INVALID,
                 "observable %d: null, other dimension or other context", i);
    DeviceGuard dg(psi->ctx->device);
    obs_eval_many(obs, nobs, psi->col(t), reinterpret_cast<cplx*>(re_im));
  });
}

// ------------------------------------------------------------------ Lanczos
qd_status qd_lanczos_ground(qd_ham* ham, qd_state* psi, int t, const qd_lanczos_opts* opts, double* evals_out,
                            qd_lanczos_result* res) {
  return guard([&] {
    QD_REQUIRE(ham && psi && opts && res, QD_ERR_INVALID, "null argument");
    QD_REQUIRE(t >= 0 && t < psi->nt, QD_ERR_INVALID, "bad column");
    QD_REQUIRE(psi->dim == ham->dim, QD_ERR_INVALID, "dimension mismatch");
    QD_REQUIRE(opts->spmv == QD_SPMV_CSR || opts->spmv == QD_SPMV_MATRIX_FREE, QD_ERR_INVALID, "bad spmv kind");
    QD_REQUIRE(opts->ritz == QD_RITZ_STORED_BASIS || opts->ritz == QD_RITZ_SECOND_PASS, QD_ERR_INVALID,
               "bad ritz mode");
    DeviceGuard dg(ham->ctx->device);
    std::memset(res, 0, sizeof(*res));
    lanczos_ground(ham, psi->col(t), *opts, evals_out, res);
  });
}

qd_status qd_ham_time_spmv(qd_ham* ham, int spmv, int iters, double* avg_ms, double* bytes_per_launch) {
  return guard([&] {
    QD_REQUIRE(ham && avg_ms && bytes_per_launch && iters >= 1, QD_ERR_INVALID, "bad argument");
    const bool plain = spmv == QD_SPMV_CSR || spmv == QD_SPMV_MATRIX_FREE || spmv == kSpmvFx || spmv == kSpmvFxSlots ||
                       spmv == kSpmvFxBlock ||
                       (spmv >= kSpmvTile && spmv <= kSpmvLast);
    const bool fused = spmv >= 2000 + kSpmvTile && spmv <= 2000 + kSpmvLast;
    const bool vec = spmv == 3001 || spmv == 3002;
    QD_REQUIRE(plain || fused || vec, QD_ERR_UNSUPPORTED, "qd_ham_time_spmv: unknown kernel code %d", spmv);
    DeviceGuard dg(ham->ctx->device);
    if (spmv % 1000 == kSpmvRowSorted) ham_ensure_row_order(ham);
    time_spmv(ham, spmv, iters, avg_ms, bytes_per_launch);
  });
}

qd_status qd_arnoldi_evolve(qd_ham* ham, qd_state* psi, int t_in, int t_out, double h, int m, int* act_dim) {
  return guard([&] {
    QD_REQUIRE(ham && psi, QD_ERR_INVALID, "null argument");
    QD_REQUIRE(psi->dim == ham->dim, QD_ERR_INVALID, "dimension mismatch");
    QD_REQUIRE(t_in >= 0 && t_in < psi->nt && t_out >= 0 && t_out < psi->nt, QD_ERR_INVALID, "bad column");
    DeviceGuard dg(ham->ctx->device);
    arnoldi_evolve(ham, psi->col(t_in), psi->col(t_out), h, m, act_dim);
  });
}

qd_status qd_lanczos_extend(qd_ham* ham, qd_state* psi, int t, const qd_lanczos_opts* opts, double* evals_out,
                            qd_lanczos_result* res) {
  return guard([&] {
    QD_REQUIRE(ham && psi && opts && res, QD_ERR_INVALID, "null argument");
    QD_REQUIRE(t >= 0 && t < psi->nt, QD_ERR_INVALID, "bad column");
    QD_REQUIRE(psi->dim == ham->dim, QD_ERR_INVALID, "dimension mismatch");
    DeviceGuard dg(ham->ctx->device);
    std::memset(res, 0, sizeof(*res));
    lanczos_extend(ham, psi->col(t), *opts, evals_out, res);
  });
}

static void arnoldi_ground_call(qd_ham* ham, qd_state* psi, int t, const qd_lanczos_opts* opts, double* evals_out,
                                qd_lanczos_result* res, bool extend) {
  QD_REQUIRE(ham && psi && opts && res, QD_ERR_INVALID, "null argument");
  QD_REQUIRE(t >= 0 && t < psi->nt, QD_ERR_INVALID, "bad column");
  QD_REQUIRE(psi->dim == ham->dim, QD_ERR_INVALID, "dimension mismatch");
  DeviceGuard dg(ham->ctx->device);
  const double prev = (extend && ham->arnoldi_gs) ? ham->arnoldi_gs_ritz : 0.0;
  std::memset(res, 0, sizeof(*res));
  arnoldi_ground(ham, psi->col(t), opts->krylov_dim, opts->add_dim, extend, evals_out, res);
  res->err = std::fabs(res->ritz_value - prev);
  ham->arnoldi_gs_ritz = res->ritz_value;
}

qd_status qd_arnoldi_ground(qd_ham* ham, qd_state* psi, int t, const qd_lanczos_opts* opts, double* evals_out,
                            qd_lanczos_result* res) {
  return guard([&] { arnoldi_ground_call(ham, psi, t, opts, evals_out, res, false); });
}

qd_status qd_arnoldi_extend(qd_ham* ham, qd_state* psi, int t, const qd_lanczos_opts* opts, double* evals_out,
                            qd_lanczos_result* res) {
  return guard([&] { arnoldi_ground_call(ham, psi, t, opts, evals_out, res, true); });
}

qd_status qd_hermitian_lanczos_ground(qd_ham* ham, qd_state* psi, int t, int kry_dim, double* evals_out,
                                      qd_lanczos_result* res) {
  return guard([&] {
    QD_REQUIRE(ham && psi && res, QD_ERR_INVALID, "null argument");
    QD_REQUIRE(t >= 0 && t < psi->nt, QD_ERR_INVALID, "bad column");
    QD_REQUIRE(psi->dim == ham->dim, QD_ERR_INVALID, "dimension mismatch");
    DeviceGuard dg(ham->ctx->device);
    std::memset(res, 0, sizeof(*res));
    hermitian_lanczos_ground(ham, psi->col(t), kry_dim, evals_out, res);
  });
}

qd_status qd_lanczos_evolve(qd_ham* ham, qd_state* psi, int t_in, int t_out, double h, int m, int nsteps,
                            int* act_dim) {
  return guard([&] {
    QD_REQUIRE(ham && psi, QD_ERR_INVALID, "null argument");
    QD_REQUIRE(psi->dim == ham->dim, QD_ERR_INVALID, "dimension mismatch");
    QD_REQUIRE(t_in >= 0 && t_in < psi->nt && t_out >= 0 && t_out < psi->nt, QD_ERR_INVALID, "bad column");
    QD_REQUIRE(m >= 2 && m <= 33, QD_ERR_UNSUPPORTED, "Krylov dimension m must be in 2..33");
    DeviceGuard dg(ham->ctx->device);
    QD_REQUIRE(nsteps >= 1, QD_ERR_INVALID, "nsteps must be positive");
    lanczos_evolve(ham, psi->col(t_in), psi->col(t_out), h, m, nsteps, act_dim, nullptr);
  });
}

qd_status qd_batch_lanczos(qd_ctx* ctx, int ninst, qd_ham* const* hams, const double* const* v0s, int steps,
                           double* out) {
  return guard([&] {
    QD_REQUIRE(ctx && hams && v0s && out, QD_ERR_INVALID, "null argument");
    DeviceGuard dg(ctx->device);
    batch_lanczos(ctx, hams, v0s, ninst, steps, out);
  });
}

qd_status qd_krylov_evolve_batch(qd_ham* ham, const double* d_X, int64_t ldx, int nvec, double h, int m,
                                 double* d_Y, int64_t ldy, int* act_dims) {
  return guard([&] {
    QD_REQUIRE(ham && d_Y && nvec >= 1, QD_ERR_INVALID, "bad argument");
    QD_REQUIRE(ldy >= ham->dim && (!d_X || ldx >= ham->dim), QD_ERR_INVALID, "leading dimension below dim");
    QD_REQUIRE(d_X || nvec <= ham->dim, QD_ERR_INVALID, "more unit vectors than the dimension");
    DeviceGuard dg(ham->ctx->device);
    krylov_batch(ham, reinterpret_cast<const cplx*>(d_X), ldx, nvec, h, m, reinterpret_cast<cplx*>(d_Y), nullptr,
                 ldy, act_dims);
  });
}

qd_status qd_traj_run(qd_ham* heff, const qd_traj_desc* desc, const double* psi0, double* obs_mean,
                      double* obs_stderr, qd_traj_stats* stats) {
  return guard([&] {
    QD_REQUIRE(heff && desc && psi0 && (obs_mean || desc->nobs == 0), QD_ERR_INVALID, "null argument");
    QD_REQUIRE(desc->chan_bits && (desc->nobs == 0 || (desc->obs_a && desc->obs_b)), QD_ERR_INVALID,
               "null channel or observable array");
    DeviceGuard dg(heff->ctx->device);
    int64_t jumps = 0;
    double t[2] = {0, 0};
    int path[2] = {0, 0};
    traj_run(heff, *desc, psi0, obs_mean, obs_stderr, &jumps, t, path);
    if (stats) {
      std::memset(stats, 0, sizeof(*stats));
      stats->jumps = jumps;
      stats->setup_ms = t[0];
      stats->ensemble_ms = t[1];
      stats->path = path[0];
      stats->products = path[1];
    }
  });
}

qd_status qd_ham_set_spmv_kernel(qd_ham* ham, int kernel) {
  return guard([&] {
    QD_REQUIRE(ham && ((kernel >= kSpmvTile && kernel <= kSpmvLast) || kernel == kSpmvFx || kernel == kSpmvFxSlots ||
                       kernel == kSpmvFxBlock),
               QD_ERR_INVALID, "unknown product kernel");
    DeviceGuard dg(ham->ctx->device);
    if (kernel == kSpmvFx || kernel == kSpmvFxSlots || kernel == kSpmvFxBlock) {
      QD_REQUIRE(ham_build_fx(ham), QD_ERR_UNSUPPORTED, "the fixed-point form does not apply to this operator");
      QD_REQUIRE(kernel != kSpmvFxSlots || ham_build_fx_slots(ham), QD_ERR_UNSUPPORTED,
                 "the columns of this operator cannot be computed on the fly (code 121)");
      QD_REQUIRE(kernel != kSpmvFxBlock || ham_build_fx_block(ham), QD_ERR_UNSUPPORTED,
                 "this sector or operator has no block layout (code 122)");
      ham->fx->use_slots = (kernel == kSpmvFxSlots);
      ham->fx->use_blk = (kernel == kSpmvFxBlock);
      ham->fx_allowed = true;
      return;
    }
    if (kernel == kSpmvRowSorted) ham_ensure_row_order(ham);
    ham->spmv_variant = kernel;
    ham->fx_allowed = false;
  });
}

qd_status qd_ham_autotune(qd_ham* ham, int iters, int* chosen, double* best_ms) {
  return guard([&] {
    QD_REQUIRE(ham && iters >= 1, QD_ERR_INVALID, "bad argument");
    DeviceGuard dg(ham->ctx->device);
    double best = 1e300, bytes = 0;
    int pick = ham->spmv_variant;
    ham_ensure_row_order(ham);
    for (int v = kSpmvTile; v <= kSpmvLast; ++v) {
      double ms = 0;
      time_spmv(ham, v, iters, &ms, &bytes);
      if (ms < best) {
        best = ms;
        pick = v;
      }
    }
    ham->spmv_variant = pick;
    ham->fx_allowed = false;
    if ((ham->flags & QD_HAM_REAL) && ham_build_fx(ham)) {
      // the fixed-point forms as the recurrence launches them (fused with the step's inner products,
      // which a CSR kernel leaves to a separate pass): a conservative comparison for them
      const bool slots0 = ham->fx->use_slots, blk0 = ham->fx->use_blk;
      int fx_pick = 0;
      for (int v = kSpmvFx; v <= kSpmvFxBlock; ++v) {
        if (v == kSpmvFxSlots && !ham_build_fx_slots(ham)) continue;
        if (v == kSpmvFxBlock && !ham_build_fx_block(ham)) continue;
        double ms = 0;
        ham->fx_allowed = true;
        ham->fx->use_slots = (v == kSpmvFxSlots);
        ham->fx->use_blk = (v == kSpmvFxBlock);
        time_spmv(ham, QD_SPMV_CSR, iters, &ms, &bytes);
        if (ms < best) {
          best = ms;
          pick = v;
          fx_pick = v;
        }
      }
      ham->fx_allowed = fx_pick != 0;
      ham->fx->use_slots = fx_pick ? (fx_pick == kSpmvFxSlots) : slots0;
      ham->fx->use_blk = fx_pick ? (fx_pick == kSpmvFxBlock) : blk0;
    }
    if (chosen) *chosen = pick;
    if (best_ms) *best_ms = best;
  });
}

}  // extern "C"
