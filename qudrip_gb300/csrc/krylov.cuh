// krylov.cuh -- solver workspaces (reused across calls on one Hamiltonian).
#pragma once

#include <type_traits>

#include "fxstep.cuh"
#include "ham.cuh"
#include "spmv.cuh"
#include "vec.cuh"

namespace qd {



inline double real_part(double v) { return v; }
inline double real_part(cplx v) { return v.re; }

// Device buffers of one Lanczos recurrence and its captured CUDA graph.
template <typename VV>
struct LanczosBuffers {
  int64_t n = 0;
  int kdim = 0;
  int64_t ld = 0;  // leading dimension of the stored basis
  DBuf<VV> V;      // (kdim + 1) x ld basis vectors
  DBuf<VV> w;
  DBuf<VV> alpha, beta;
  DBuf<Tri<VV>> dots;  // per step: <V2, w>, <V1, w>, <V1, V2>
  DBuf<double> nrm, nrm2, y, scl;  // scl[k] = 1 / ||V[k]|| (basis stored unnormalised)
  DBuf<int> stop;
  DBuf<__int128> X;  // fixed-point copies of the two newest basis vectors (uniform-coupling product)
  DBuf<int> ovf;         // [0] a vector left the fixed-point range, [1] a bounded device wait ran out
  DBuf<unsigned> epoch;  // launch parity of the one-launch steps (fxstep.cuh, fxblock.cu)
  DBuf<double> mbox;     // their alpha and beta mailbox (kMboxDoubles entries)
  cudaGraphExec_t exec = nullptr;
  int kind = 0;  // product the captured graph launches (0 CSR, 1 matrix-free, 2 fixed-point, +4 one-launch step)
  int done = 0;  // Lanczos steps run on the stored basis (incremental solves continue from here)
  void ensure_fx(cudaStream_t s) {  // stream-ordered: a legacy-stream call would wait for every lane
    if (!X.p) {
      X.alloc((size_t)2 * ld);
      ovf.alloc(2);
      epoch.alloc(4);
      mbox.alloc(kMboxDoubles);  // both set empty by each run's first launch
    }
  }
  int64_t graph_kernels = 0;

  void ensure(int64_t n_, int kdim_) {
    if (n_ == n && kdim_ == kdim) return;
    drop_graph();
    n = n_;
    kdim = kdim_;
    ld = (n + 31) / 32 * 32;
    V.alloc((size_t)(kdim + 1) * ld);
    w.alloc(ld);
    alpha.alloc(kdim + 2);
    beta.alloc(kdim + 2);
    dots.alloc(kdim + 2);
    nrm.alloc(kdim + 2);
    nrm2.alloc(kdim + 2);
    y.alloc(kdim + 2);
    scl.alloc(kdim + 2);
    stop.alloc(1);
    X = DBuf<__int128>();
  }
  void drop_graph() {
    if (exec) cudaGraphExecDestroy(exec);
    exec = nullptr;
  }
  // Capture `body` (a fixed launch sequence) once, replay it afterwards.
  template <typename F>
  void run_graph(Ctx* ctx, F&& body) {
    if (!exec) {
      cudaGraph_t g = nullptr;
      const int64_t before = ctx->launches;
      QD_CUDA(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
      try {
        body();
      } catch (...) {
        cudaStreamEndCapture(ctx->stream, &g);
        if (g) cudaGraphDestroy(g);
        throw;
      }
      QD_CUDA(cudaStreamEndCapture(ctx->stream, &g));
      graph_kernels = ctx->launches - before;
      ctx->launches = before;
      const cudaError_t e = cudaGraphInstantiate(&exec, g, 0);
      cudaGraphDestroy(g);
      QD_CUDA(e);
    }
    QD_CUDA(cudaGraphLaunch(exec, ctx->stream));
    ctx->launches += graph_kernels;
  }
  ~LanczosBuffers() { drop_graph(); }
};

struct EvolveGraph;
struct EvolveGraphDeleter {
  void operator()(EvolveGraph* g) const;
};

struct Workspace {
  Ctx* ctx;
  std::unique_ptr<EvolveGraph, EvolveGraphDeleter> evolve;  // cached Krylov-step graph
  // the last Lanczos ground-state run: vector type (1 real, 2 complex), value
  // type (1 real, 2 complex), product kind -- what a continuation must reuse
  int lz_vv = 0, lz_mv = 0, lz_mf = 0, lz_fxk = 0;
  DBuf<double> partials_d, gpart_d;
  DBuf<cplx> partials_c, gpart_c;
  DBuf<Tri<double>> partials_td, gpart_td;
  DBuf<Tri<cplx>> partials_tc, gpart_tc;
  DBuf<unsigned> tickets;
  LanczosBuffers<double> lz_d;
  LanczosBuffers<cplx> lz_c;
  // H psi and the result of state_eval, kept between calls (a device allocation
  // and free per call would wait for the whole device)
  DBuf<cplx> eval_y, eval_out;
  DBuf<double> eval_real;  // the uniform-coupling form's value and its imaginary-part flag
  DBuf<int> eval_flag;
  DBuf<double> start_nrm2;  // ||v0||^2 of the last ground-state solve (read by its first kernels)
  DBuf<int> start_has_im;

  explicit Workspace(Ctx* c);
  GridRed<double> red_d(int slot);
  GridRed<double> red_d_flat(int slot);
  GridRed<cplx> red_c(int slot);
  template <typename VV>
  GridRed<Tri<VV>> red_tri(int slot) {
    unsigned* t = tickets.p + (size_t)slot * (1 + kRedMaxGroups);
    if constexpr (std::is_same<VV, double>::value) return GridRed<Tri<double>>{partials_td.p, t, gpart_td.p};
    else return GridRed<Tri<cplx>>{partials_tc.p, t, gpart_tc.p};
  }
  template <typename VV>
  GridRed<VV> red_c_or_d(int slot) {
    if constexpr (std::is_same<VV, double>::value) return red_d(slot);
    else return red_c(slot);
  }
};

Workspace& ham_workspace(qd_ham* H);
void ham_apply_c(qd_ham* H, const cplx* x, cplx* y);
cplx state_eval(qd_ham* H, const cplx* psi);
double state_norm2(qd_ham* H, const cplx* psi);
void state_norm2_eval(qd_ham* H, const cplx* psi, double* n2, cplx* e);
void obs_eval_many(qd_ham* const* obs, int nobs, const cplx* psi, cplx* out_host);
void lanczos_ground(qd_ham* H, cplx* psi, const qd_lanczos_opts& o, double* evals_out, qd_lanczos_result* res);
void lanczos_extend(qd_ham* H, cplx* psi, const qd_lanczos_opts& o, double* evals_out, qd_lanczos_result* res);
void time_spmv(qd_ham* H, int spmv, int iters, double* avg_ms, double* bytes_per_launch);
void lanczos_evolve(qd_ham* H, const cplx* psi_in, cplx* psi_out, double h, int m, int nsteps, int* act_out,
                    int64_t* matvecs_out);
void hermitian_lanczos_ground(qd_ham* H, cplx* psi, int kdim, double* evals_out, qd_lanczos_result* res);
void launch_fx_dots(Ctx* ctx, const qd_ham* H, const FxForm& f, const double* x, const __int128* X,
                    const double* V2, double* y, const double* s1, const double* s2, const int* stop, int step,
                    double* beta, double* alpha, Tri<double>* dots, GridRed<Tri<double>> red);
void launch_fx_slots(Ctx* ctx, const qd_ham* H, const FxForm& f, const double* x, const __int128* X, double* y,
                     const double* scale_dev, const int* stop, int step);
void launch_fx_slots_dots(Ctx* ctx, const qd_ham* H, const FxForm& f, const double* x, const __int128* X,
                          const double* V2, double* y, const double* s1, const double* s2, const int* stop, int step,
                          double* beta, double* alpha, Tri<double>* dots, GridRed<Tri<double>> red, int grid);
struct FxStepArgs;
// One Lanczos step of the uniform-coupling form in one cooperative launch
// (fxstep.cuh); false when it does not fit on the device at once.
bool launch_fx_step(Ctx* ctx, const qd_ham* H, const FxForm& f, FxStepArgs a);
// <psi|H psi> on the uniform-coupling form when psi's imaginary part is 0 (false, with *value
// undefined, when it is not)
bool fx_eval_real(Ctx* ctx, const qd_ham* H, const FxForm& f, const cplx* psi, GridRed<double> red, double* out_dev,
                  int* flag_dev, double* value);
bool launch_fx_slots_step(Ctx* ctx, const qd_ham* H, const FxForm& f, const FxStepArgs& a, int grid);
bool launch_fx_block_step(Ctx* ctx, const qd_ham* H, const FxForm& f, FxStepArgs a, int grid);
void launch_fx_block_dots(Ctx* ctx, const qd_ham* H, const FxForm& f, const double* x, const __int128* X,
                          const double* V2, double* y, const double* s1, const double* s2, const int* stop, int step,
                          double* beta, double* alpha, Tri<double>* dots, GridRed<Tri<double>> red, int grid);
void launch_fx_block(Ctx* ctx, const qd_ham* H, const FxForm& f, const double* x, const __int128* X, double* y);
template <typename VV>
void launch_mf(Ctx* ctx, qd_ham* H, const VV* x, VV* y, double scale, const double* scale_dev, const int* stop,
               int step);

}  // namespace qd
