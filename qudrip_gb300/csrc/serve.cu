// serve.cu -- the request loop: ground-state and real-time-evolution requests
// admitted by device-memory footprint onto worker lanes.
//
// No counterpart in the reference (each of its programs runs one solve per
// process).  Design:
//   * A lane is a non-blocking CUDA stream (its own Ctx) driven by one host
//     thread.  Small lanes (high stream priority) take requests whose sector
//     dimension is at most small_dim; large lanes take any request; batch
//     lanes (mixed form) take every waiting small ground state with a real
//     start vector at once, once at least batch_min of them wait, and run
//     them in one persistent launch (batch_lanczos, one CTA per instance);
//     below that the small lanes serve them one by one at once.  Requests on different lanes
//     overlap on the GPU; a request that arrives while others run is taken by
//     the next lane that frees up (continuous batching, not a queue in front
//     of a single solver).
//   * Admission is in arrival order and by footprint: a request is taken only
//     when its estimated device bytes fit the budget next to everything
//     admitted before it; once its Hamiltonian is lowered the estimate is
//     replaced by the bytes actually held.  The sector, the CSR Hamiltonian
//     and the Krylov basis stay resident until the request completes.
//   * Lane threads allocate from the stream-ordered pool on their own stream
//     (AllocStreamScope), so one lane's allocations and frees do not
//     serialise the other lanes' kernels.
//   * Every solve is deterministic and independent of the other requests
//     (per-request buffers, fixed reduction orders; a batched instance is one
//     CTA whatever the batch), so a result is the same alone and in the mix.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

#include "batch.cuh"
#include "evolve.cuh"
#include "ham.cuh"
#include "krylov.cuh"
#include "philox.cuh"
#include "sector.cuh"

namespace qd {

void sector_build(qd_sector* S);

// ---------------------------------------------------------------- seeded start vectors
constexpr uint32_t kSeedStream = 0x53544152u;

__host__ __device__ inline double seeded_element(uint64_t seed, int64_t i) {
  double u1, u2;
  philox_uniform2(seed, kSeedStream, (uint32_t)(i >> 1), u1, u2);
  return 2.0 * ((i & 1) ? u2 : u1) - 1.0;
}

__global__ void seeded_start_kernel(int64_t n, uint64_t seed, cplx* out) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = mkc(seeded_element(seed, i), 0.0);
}

// ---------------------------------------------------------------- requests
struct ServeReq {
  uint64_t id = 0;
  qd_request d{};
  std::vector<qd_constraint> cons;
  std::vector<qd_term> terms;
  std::vector<qd_gate> gates;
  std::vector<double> psi0;  // interleaved complex, empty when seeded
  bool real_start = true;
  int64_t dim_est = 0;
  int64_t bytes_est = 0;
  int64_t bytes_held = 0;
  double t_submit = 0.0, t_admit = 0.0;
};

enum LaneKind { kLaneSmall = 0, kLaneLarge = 1, kLaneBatch = 2 };

struct Lane {
  Ctx ctx;
  LaneKind kind = kLaneLarge;
  std::thread th;
};

// Sector dimension from the constraints when they are independent particle
// counts (one Nset term of weight 1 per constraint, disjoint masks, tight 0):
// the product of binomials times 2^(free bits).  Otherwise 2^nbits (a bound).
static int64_t estimate_dim(const ServeReq& r) {
  auto binom = [](int n, int k) -> double {
    if (k < 0 || k > n) return 0.0;
    double b = 1.0;
    for (int i = 1; i <= k; ++i) b = b * (n - k + i) / i;
    return b;
  };
  const int nb = r.d.nbits;
  double full = std::ldexp(1.0, std::min(nb, 62));
  if (r.d.tight != 0) return (int64_t)full;
  uint64_t used = 0;
  double dim = 1.0;
  for (const qd_constraint& c : r.cons) {
    if (c.nterms != 1 || c.term[0].kind != QD_CQ_NSET || c.term[0].coef != 1) return (int64_t)full;
    const uint64_t m = c.term[0].mask;
    if (m & used) return (int64_t)full;
    used |= m;
    dim *= binom(__builtin_popcountll(m), (int)c.target);
  }
  dim *= std::ldexp(1.0, nb - __builtin_popcountll(used));
  return (int64_t)std::min(dim, full);
}

// Device bytes a request may need at its peak: the lowering's triplet buffer
// (32 slots of 24 bytes per row at the first capacity), the CSR arrays for up
// to min(terms, 64) entries per row, the basis and its index, and the Krylov
// vectors of the solver.
static int64_t estimate_bytes(const ServeReq& r, int64_t dim) {
  const int64_t per_row_nnz = std::min<int64_t>(std::max<int64_t>(r.d.nterms, 1), 64);
  const int64_t lowering = dim * 32 * 24;
  const int64_t csr = dim * per_row_nnz * (16 + 8 + 4 + 4) + dim * 16;
  const int64_t basis = dim * 16;
  const int64_t kry = (r.d.kind == QD_REQ_GROUND) ? (int64_t)(r.d.krylov_dim + 4) * dim * 16
                                                  : (int64_t)(r.d.krylov_dim + 4) * dim * 16 * 2;
  return std::max(lowering, csr) + basis + kry + (8 << 20);
}

template <typename T>
static int64_t dbytes(const DBuf<T>& b) {
  return (int64_t)b.bytes();
}

static int64_t held_bytes(const qd_sector* S, const qd_ham* H) {
  int64_t b = 0;
  if (S) b += dbytes(S->basis) + dbytes(S->binom) + dbytes(S->dir);
  if (H) {
    b += dbytes(H->rowptr) + dbytes(H->colidx) + dbytes(H->vals_c) + dbytes(H->vals_r) + dbytes(H->vals_f) +
         dbytes(H->row_order) + dbytes(H->diag_r) + dbytes(H->bun_d);
    if (H->ws) {
      const Workspace& W = *H->ws;
      b += dbytes(W.partials_d) + dbytes(W.gpart_d) + dbytes(W.partials_c) + dbytes(W.gpart_c) +
           dbytes(W.partials_td) + dbytes(W.gpart_td) + dbytes(W.partials_tc) + dbytes(W.gpart_tc) +
           dbytes(W.tickets) + dbytes(W.lz_d.V) + dbytes(W.lz_c.V) + dbytes(W.lz_d.w) + dbytes(W.lz_c.w);
    }
    if (H->arnoldi) b += dbytes(H->arnoldi->V) + dbytes(H->arnoldi->w) + dbytes(H->arnoldi->partials);
  }
  return b;
}

}  // namespace qd

struct qd_server {
  qd::Ctx* parent = nullptr;
  qd_server_opts o{};
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<qd::ServeReq*> pending;
  std::deque<qd_result> done;
  std::vector<std::unique_ptr<qd::Lane>> lanes;
  bool stop = false;
  bool has_batch = false;
  int64_t in_use = 0, peak = 0;
  int64_t submitted = 0, completed = 0, failed = 0, batches = 0, batched = 0;
  int64_t active = 0, max_active = 0;
  uint64_t next_id = 1;
  std::chrono::steady_clock::time_point t0 = std::chrono::steady_clock::now();
  double now() const {
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  }
};

namespace qd {

static bool batchable(const qd_server* S, const ServeReq* r) {
  return S->has_batch && r->d.kind == QD_REQ_GROUND && r->dim_est <= S->o.batch_dim && r->d.psi_out == nullptr &&
         r->real_start && r->d.krylov_dim <= 256;
}

// Small lanes take every small request, batchable ground states included (a lone
// small ground state is served at once instead of waiting for a batch); batch
// lanes take batchable ground states only once batch_min of them wait (take()).
static bool eligible(const qd_server* S, const ServeReq* r, LaneKind k) {
  const bool small = r->dim_est <= S->o.small_dim;
  switch (k) {
    case kLaneBatch: return batchable(S, r);
    case kLaneSmall: return small;
    default: return !batchable(S, r);
  }
}

// Takes requests for a lane under the lock: the oldest eligible one that fits
// the budget (a batch lane takes every such request, up to batch_max, with the
// oldest one's Krylov dimension).
static std::vector<ServeReq*> take(qd_server* S, LaneKind k) {
  std::vector<ServeReq*> got;
  const int cap = (k == kLaneBatch) ? std::max(1, S->o.batch_max) : 1;
  if (k == kLaneBatch) {
    int waiting = 0;
    for (const ServeReq* r : S->pending) waiting += batchable(S, r) ? 1 : 0;
    if (waiting < std::max(1, S->o.batch_min)) return got;
  }
  int kdim = -1;
  for (auto it = S->pending.begin(); it != S->pending.end() && (int)got.size() < cap;) {
    ServeReq* r = *it;
    if (eligible(S, r, k) && (kdim < 0 || r->d.krylov_dim == kdim) &&
        (S->in_use + r->bytes_est <= S->o.hbm_budget || S->active == 0)) {
      if (kdim < 0) kdim = r->d.krylov_dim;
      S->in_use += r->bytes_est;
      r->bytes_held = r->bytes_est;
      S->peak = std::max(S->peak, S->in_use);
      S->active++;
      S->max_active = std::max(S->max_active, S->active);
      r->t_admit = S->now();
      got.push_back(r);
      it = S->pending.erase(it);
    } else {
      ++it;
    }
  }
  return got;
}

// Replaces a request's reserved bytes by what it holds now.
static void recharge(qd_server* S, ServeReq* r, int64_t held) {
  std::lock_guard<std::mutex> lk(S->mu);
  S->in_use += held - r->bytes_held;
  r->bytes_held = held;
  S->peak = std::max(S->peak, S->in_use);
}

static void finish(qd_server* S, ServeReq* r, qd_result& res) {
  std::lock_guard<std::mutex> lk(S->mu);
  res.id = r->id;
  res.tag = r->d.tag;
  res.kind = r->d.kind;
  res.t_submit = r->t_submit;
  res.t_admit = r->t_admit;
  res.t_done = S->now();
  res.bytes = r->bytes_held;
  S->in_use -= r->bytes_held;
  S->active--;
  S->completed++;
  if (res.status != QD_OK) S->failed++;
  S->done.push_back(res);
  delete r;
  S->cv_done.notify_all();
  S->cv_work.notify_all();
}

struct Built {
  qd_sector* sec = nullptr;
  qd_ham* H = nullptr;
  ~Built() {
    delete H;
    delete sec;
  }
};

static void build_request(Ctx* ctx, ServeReq* r, Built& b) {
  b.sec = new qd_sector();
  b.sec->ctx = ctx;
  b.sec->nbits = r->d.nbits;
  b.sec->tight = r->d.tight;
  b.sec->cons = r->cons;
  sector_build(b.sec);
  QD_REQUIRE(b.sec->view.dim >= 1, QD_ERR_INVALID, "empty sector");
  QD_REQUIRE(r->psi0.empty() || (int64_t)r->psi0.size() == 2 * b.sec->view.dim, QD_ERR_INVALID,
             "start state has %lld elements, the sector %lld", (long long)(r->psi0.size() / 2),
             (long long)b.sec->view.dim);
  b.H = new qd_ham();
  b.H->ctx = ctx;
  b.H->sec = b.sec;
  b.H->one_shot = true;
  ham_lower(b.H, r->terms.data(), (int)r->terms.size(), r->gates.data(), (int)r->gates.size());
}

// One request with the grid-wide solvers on this lane's stream.
static bool trace_on() {
  static const bool on = std::getenv("QD_SERVE_TRACE") != nullptr;
  return on;
}

static void run_single(qd_server* S, Lane* L, ServeReq* r, Built* prebuilt) {
  qd_result res;
  std::memset(&res, 0, sizeof(res));
  res.path = QD_PATH_GRID;
  Ctx* ctx = &L->ctx;
  const double t0 = S->now();
  double t_built = t0, t_solved = t0;
  try {
    Built own;
    Built& b = prebuilt ? *prebuilt : own;
    if (!b.H) build_request(ctx, r, b);
    if (trace_on()) {
      QD_CUDA(cudaStreamSynchronize(ctx->stream));
      t_built = S->now();
    }
    qd_ham* H = b.H;
    const int64_t n = H->dim;
    res.dim = n;
    res.nnz = H->nnz;
    DBuf<cplx> psi(n);
    if (!r->psi0.empty()) {
      QD_CUDA(cudaMemcpyAsync(psi.p, r->psi0.data(), n * sizeof(cplx), cudaMemcpyHostToDevice, ctx->stream));
    } else {
      const int g = (int)std::min<int64_t>(ceil_div(n, 256), (int64_t)ctx->num_sms * 8);
      seeded_start_kernel<<<g, 256, 0, ctx->stream>>>(n, r->d.seed, psi.p);
      QD_CHECK_LAUNCH();
      QD_LAUNCHED(ctx);
    }
    if (r->d.kind == QD_REQ_GROUND) {
      qd_lanczos_opts lo;
      std::memset(&lo, 0, sizeof(lo));
      lo.krylov_dim = r->d.krylov_dim;
      lo.spmv = QD_SPMV_CSR;
      lo.ritz = QD_RITZ_STORED_BASIS;
      qd_lanczos_result lr;
      std::memset(&lr, 0, sizeof(lr));
      lanczos_ground(H, psi.p, lo, nullptr, &lr);
      res.ritz = lr.ritz_value;
      res.act_dim = lr.act_dim;
      res.matvecs = lr.matvecs;
    } else {
      const bool fast = (S->o.mode == QD_SERVE_MIXED) && (H->flags & QD_HAM_HERMITIAN);
      int act = 0;
      if (fast) {
        // Integrate to T = nsteps * dt with the mixed form's own Krylov step:
        // m = 32 and h = T / n with n = ceil(T w / 8), w the half-width of
        // H's Gershgorin interval.  The Krylov space of H and of H - cI are
        // the same and exp(-ih(H - cI)) = exp(ihc) exp(-ihH), so the error
        // bound (e ||h(H - cI)|| / 2m)^m holds for the centre c, with
        // ||H - cI|| <= w <= ||H||_inf: ||h(H - cI)|| <= 8 = m / 4 keeps it
        // below 1e-15 per step.  The requested (dt, m) is kept when it is the
        // coarser of the two.
        const double T = r->d.dt * r->d.nsteps;
        const double hn = ham_gershgorin_halfwidth(H);
        int nint = std::max(1, (int)std::ceil(std::fabs(T) * hn / 8.0));
        double h = r->d.dt;
        int m = r->d.krylov_dim, steps = r->d.nsteps;
        if (nint < r->d.nsteps && std::isfinite(hn)) {
          h = T / nint;
          m = 32;
          steps = nint;
        }
        int64_t mv = 0;
        lanczos_evolve(H, psi.p, psi.p, h, m, steps, &act, &mv);
        res.matvecs += mv;
      } else {
        for (int s = 0; s < r->d.nsteps; ++s) {
          arnoldi_evolve(H, psi.p, psi.p, r->d.dt, r->d.krylov_dim, &act);
          res.matvecs += act;
        }
      }
      res.act_dim = act;
    }
    if (trace_on()) {
      QD_CUDA(cudaStreamSynchronize(ctx->stream));
      t_solved = S->now();
    }
    recharge(S, r, held_bytes(b.sec, H) + (int64_t)psi.bytes());
    double n2 = 0.0;
    cplx e = mkc(0.0, 0.0);
    state_norm2_eval(H, psi.p, &n2, &e);
    res.norm = std::sqrt(n2);
    res.energy = e.re / n2;
    res.matvecs += 1;
    if (r->d.psi_out) {
      QD_REQUIRE(r->d.psi_out_len >= n, QD_ERR_INVALID, "psi_out holds %lld elements, the result %lld",
                 (long long)r->d.psi_out_len, (long long)n);
      QD_CUDA(cudaMemcpyAsync(r->d.psi_out, psi.p, n * sizeof(cplx), cudaMemcpyDeviceToHost, ctx->stream));
    }
    QD_CUDA(cudaStreamSynchronize(ctx->stream));
    res.status = QD_OK;
  } catch (const Error& e) {
    res.status = e.code;
    cudaStreamSynchronize(ctx->stream);
  } catch (...) {
    res.status = QD_ERR_INVALID;
    cudaStreamSynchronize(ctx->stream);
  }
  if (trace_on())
    std::fprintf(stderr, "[qd serve] id=%llu kind=%d lane=%d dim=%lld build=%.2fms solve=%.2fms rest=%.2fms\n",
                 (unsigned long long)r->id, r->d.kind, (int)L->kind, (long long)res.dim, 1e3 * (t_built - t0),
                 1e3 * (t_solved - t_built), 1e3 * (S->now() - t_solved));
  finish(S, r, res);
}

// Small real ground states in one persistent launch (one CTA per instance).
static void run_batch(qd_server* S, Lane* L, std::vector<ServeReq*>& rs) {
  Ctx* ctx = &L->ctx;
  std::vector<std::unique_ptr<Built>> built(rs.size());
  std::vector<int> ok;
  for (size_t i = 0; i < rs.size(); ++i) {
    built[i].reset(new Built());
    try {
      build_request(ctx, rs[i], *built[i]);
      if (built[i]->H->flags & QD_HAM_REAL) {
        ok.push_back((int)i);
      } else {
        run_single(S, L, rs[i], built[i].get());  // complex Hamiltonian: FP64 solver on this lane
        rs[i] = nullptr;
      }
    } catch (const Error& e) {
      qd_result res;
      std::memset(&res, 0, sizeof(res));
      res.status = e.code;
      res.path = QD_PATH_BATCH;
      cudaStreamSynchronize(ctx->stream);
      finish(S, rs[i], res);
      rs[i] = nullptr;
    }
  }
  if (ok.empty()) return;
  const double t_built = S->now();
  std::vector<qd_ham*> hams;
  std::vector<std::vector<double>> v0(ok.size());
  std::vector<const double*> v0p;
  for (size_t q = 0; q < ok.size(); ++q) {
    ServeReq* r = rs[ok[q]];
    qd_ham* H = built[ok[q]]->H;
    hams.push_back(H);
    v0[q].resize(H->dim);
    if (!r->psi0.empty())
      for (int64_t i = 0; i < H->dim; ++i) v0[q][i] = r->psi0[2 * i];
    else
      for (int64_t i = 0; i < H->dim; ++i) v0[q][i] = seeded_element(r->d.seed, i);
    v0p.push_back(v0[q].data());
    recharge(S, r, held_bytes(built[ok[q]]->sec, H) + H->dim * (int64_t)(r->d.krylov_dim + 4) * 4);
  }
  std::vector<double> out(ok.size() * 8, 0.0);
  int status = QD_OK;
  try {
    batch_lanczos(ctx, hams.data(), v0p.data(), (int)ok.size(), rs[ok[0]]->d.krylov_dim, out.data());
  } catch (const Error& e) {
    status = e.code;
    cudaStreamSynchronize(ctx->stream);
  }
  {
    std::lock_guard<std::mutex> lk(S->mu);
    S->batches++;
    S->batched += (int64_t)ok.size();
  }
  if (trace_on())
    std::fprintf(stderr, "[qd serve] batch of %zu: builds done at %.2fms, solved at %.2fms\n", ok.size(),
                 1e3 * t_built, 1e3 * S->now());
  for (size_t q = 0; q < ok.size(); ++q) {
    qd_result res;
    std::memset(&res, 0, sizeof(res));
    res.status = status;
    res.path = QD_PATH_BATCH;
    res.dim = hams[q]->dim;
    res.nnz = hams[q]->nnz;
    res.ritz = out[q * 8 + 0];
    res.energy = out[q * 8 + 1];
    res.norm = std::sqrt(std::max(out[q * 8 + 2], 0.0));
    res.act_dim = (int)out[q * 8 + 3];
    res.matvecs = res.act_dim + 1;
    finish(S, rs[ok[q]], res);
  }
}

static void lane_main(qd_server* S, Lane* L) {
  cudaSetDevice(L->ctx.device);
  AllocStreamScope scope(L->ctx.stream);
  for (;;) {
    std::vector<ServeReq*> got;
    {
      std::unique_lock<std::mutex> lk(S->mu);
      for (;;) {
        if (S->stop) return;
        got = take(S, L->kind);
        if (!got.empty()) break;
        S->cv_work.wait(lk);
      }
    }
    if (L->kind == kLaneBatch)
      run_batch(S, L, got);
    else
      run_single(S, L, got[0], nullptr);
  }
}

}  // namespace qd

using namespace qd;

extern "C" {

qd_status qd_seeded_start(uint64_t seed, int64_t dim, double* host_out) {
  return guard([&] {
    QD_REQUIRE(dim >= 0 && (dim == 0 || host_out), QD_ERR_INVALID, "bad argument");
    for (int64_t i = 0; i < dim; ++i) host_out[i] = seeded_element(seed, i);
  });
}

qd_status qd_server_create(qd_ctx* ctx_, const qd_server_opts* opts, qd_server** out) {
  Ctx* ctx = reinterpret_cast<Ctx*>(ctx_);
  return guard([&] {
    QD_REQUIRE(ctx && out, QD_ERR_INVALID, "null argument");
    DeviceGuard dg(ctx->device);
    std::unique_ptr<qd_server> S(new qd_server());
    S->parent = ctx;
    if (opts) S->o = *opts;
    qd_server_opts& o = S->o;
    QD_REQUIRE(o.mode == QD_SERVE_PLAIN || o.mode == QD_SERVE_MIXED, QD_ERR_INVALID, "bad mode");
    if (o.small_lanes <= 0) o.small_lanes = 4;
    if (o.large_lanes <= 0) o.large_lanes = 3;
    if (o.batch_lanes <= 0) o.batch_lanes = 2;
    if (o.mode == QD_SERVE_PLAIN) o.batch_lanes = 0;
    if (o.batch_max <= 0) o.batch_max = 64;
    if (o.batch_min <= 0) o.batch_min = 4;
    if (o.small_dim <= 0) o.small_dim = 65536;
    if (o.batch_dim <= 0) o.batch_dim = 3432;
    QD_REQUIRE(o.small_lanes + o.large_lanes + o.batch_lanes <= 64, QD_ERR_INVALID, "at most 64 lanes");
    if (o.hbm_budget <= 0) {
      size_t fr = 0, tot = 0;
      QD_CUDA(cudaMemGetInfo(&fr, &tot));
      o.hbm_budget = (int64_t)(0.8 * (double)fr);
    }
    S->has_batch = o.batch_lanes > 0;
    // keep freed blocks in the stream-ordered pool instead of returning them
    cudaMemPool_t pool;
    QD_CUDA(cudaDeviceGetDefaultMemPool(&pool, ctx->device));
    uint64_t keep = ~0ull;
    QD_CUDA(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep));
    int prio_lo = 0, prio_hi = 0;
    QD_CUDA(cudaDeviceGetStreamPriorityRange(&prio_lo, &prio_hi));
    auto add = [&](LaneKind k, int n) {
      for (int i = 0; i < n; ++i) {
        std::unique_ptr<Lane> L(new Lane());
        L->kind = k;
        L->ctx.device = ctx->device;
        L->ctx.num_sms = ctx->num_sms;
        const int prio = (k == kLaneLarge) ? prio_lo : prio_hi;
        QD_CUDA(cudaStreamCreateWithPriority(&L->ctx.stream, cudaStreamNonBlocking, prio));
        for (auto& ev : L->ctx.events) QD_CUDA(cudaEventCreate(&ev));
        S->lanes.push_back(std::move(L));
      }
    };
    add(kLaneSmall, o.small_lanes);
    add(kLaneLarge, o.large_lanes);
    add(kLaneBatch, o.batch_lanes);
    qd_server* raw = S.get();
    for (auto& L : S->lanes) L->th = std::thread(lane_main, raw, L.get());
    *out = S.release();
  });
}

qd_status qd_server_submit(qd_server* S, const qd_request* q, uint64_t* id) {
  return guard([&] {
    QD_REQUIRE(S && q, QD_ERR_INVALID, "null argument");
    QD_REQUIRE(q->kind == QD_REQ_GROUND || q->kind == QD_REQ_EVOLVE, QD_ERR_INVALID, "bad request kind");
    QD_REQUIRE(q->nbits >= 1 && q->nbits <= kMaxBits, QD_ERR_INVALID, "nbits must be in 1..%d", kMaxBits);
    QD_REQUIRE(q->ncons >= 0 && (q->ncons == 0 || q->cons), QD_ERR_INVALID, "bad constraint array");
    QD_REQUIRE(q->nterms >= 0 && (q->nterms == 0 || q->terms), QD_ERR_INVALID, "bad term array");
    QD_REQUIRE(q->ngates >= 0 && (q->ngates == 0 || q->gates), QD_ERR_INVALID, "bad gate array");
    if (q->kind == QD_REQ_GROUND)
      QD_REQUIRE(q->krylov_dim >= 1 && q->krylov_dim <= 4096, QD_ERR_INVALID, "krylov_dim must be in 1..4096");
    else
      QD_REQUIRE(q->krylov_dim >= 2 && q->krylov_dim <= 33 && q->nsteps >= 1 && std::isfinite(q->dt),
                 QD_ERR_INVALID, "evolution needs m in 2..33, nsteps >= 1 and a finite dt");
    QD_REQUIRE(!q->psi0 || q->psi0_len >= 1, QD_ERR_INVALID, "psi0_len must be positive");
    for (int i = 0; i < q->ncons; ++i)
      QD_REQUIRE(q->cons[i].nterms >= 1 && q->cons[i].nterms <= 4, QD_ERR_INVALID, "constraint %d: 1..4 terms", i);
    auto* r = new ServeReq();
    r->d = *q;
    r->cons.assign(q->cons, q->cons + q->ncons);
    r->terms.assign(q->terms, q->terms + q->nterms);
    r->gates.assign(q->gates, q->gates + q->ngates);
    if (q->psi0) {
      r->psi0.assign(q->psi0, q->psi0 + 2 * q->psi0_len);
      for (int64_t i = 0; i < q->psi0_len; ++i)
        if (r->psi0[2 * i + 1] != 0.0) {
          r->real_start = false;
          break;
        }
    }
    r->d.cons = nullptr;
    r->d.terms = nullptr;
    r->d.gates = nullptr;
    r->d.psi0 = nullptr;
    r->dim_est = q->psi0 ? q->psi0_len : estimate_dim(*r);
    r->bytes_est = estimate_bytes(*r, r->dim_est);
    std::lock_guard<std::mutex> lk(S->mu);
    r->id = S->next_id++;
    r->t_submit = S->now();
    S->submitted++;
    S->pending.push_back(r);
    if (id) *id = r->id;
    S->cv_work.notify_all();
  });
}

qd_status qd_server_poll(qd_server* S, qd_result* out, int max, int* n, int timeout_ms) {
  return guard([&] {
    QD_REQUIRE(S && n && (max == 0 || out) && max >= 0, QD_ERR_INVALID, "bad argument");
    std::unique_lock<std::mutex> lk(S->mu);
    if (S->done.empty() && timeout_ms > 0)
      S->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), [&] { return !S->done.empty(); });
    int k = 0;
    while (k < max && !S->done.empty()) {
      out[k++] = S->done.front();
      S->done.pop_front();
    }
    *n = k;
  });
}

qd_status qd_server_now(qd_server* S, double* seconds) {
  return guard([&] {
    QD_REQUIRE(S && seconds, QD_ERR_INVALID, "null argument");
    *seconds = S->now();
  });
}

qd_status qd_server_get_stats(qd_server* S, qd_server_stats* st) {
  return guard([&] {
    QD_REQUIRE(S && st, QD_ERR_INVALID, "null argument");
    std::lock_guard<std::mutex> lk(S->mu);
    st->submitted = S->submitted;
    st->completed = S->completed;
    st->failed = S->failed;
    st->queued = (int64_t)S->pending.size();
    st->active = S->active;
    st->max_active = S->max_active;
    st->batches = S->batches;
    st->batched = S->batched;
    st->bytes_in_use = S->in_use;
    st->bytes_peak = S->peak;
    st->budget = S->o.hbm_budget;
  });
}

qd_status qd_server_destroy(qd_server* S) {
  return guard([&] {
    if (!S) return;
    {
      std::lock_guard<std::mutex> lk(S->mu);
      S->stop = true;
      S->cv_work.notify_all();
    }
    for (auto& L : S->lanes)
      if (L->th.joinable()) L->th.join();
    for (ServeReq* r : S->pending) delete r;
    S->pending.clear();
    cudaSetDevice(S->parent->device);
    for (auto& L : S->lanes) {
      cudaStreamSynchronize(L->ctx.stream);
      for (auto& ev : L->ctx.events)
        if (ev) cudaEventDestroy(ev);
      cudaStreamDestroy(L->ctx.stream);
    }
    delete S;
  });
}

}  // extern "C"
