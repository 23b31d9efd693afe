/*
 * qudrip_gb300.h -- C ABI of the GB300 (sm_103a) exact-diagonalization engine.
 *
 * This is the drop-in boundary for QuDrip's exact-diagonalization path.  The
 * reference has no FFI: its boundary is the C++ template API of
 * include/{index,conservation,operator,operator_abel,state,sparse_algorithm}.hpp.
 * Every entry point below names the reference interface it replaces
 * (file:line inside the QuDrip project).  The C++ drop-in header
 * include/qudrip_gpu.hpp rebuilds the reference's own names on top of these.
 *
 * Conventions
 *   - Every function returns a qd_status; QD_OK is 0.  Nothing aborts.
 *   - Host arrays belong to the caller; device memory belongs to the handles.
 *   - Complex numbers are interleaved (re, im) doubles, i.e. C99 double
 *     complex / std::complex<double> layout.
 *   - A qd_ctx owns one CUDA stream; handles made from one context must not be
 *     used from two host threads at once.  Contexts are independent.
 */
#ifndef QUDRIP_GB300_H
#define QUDRIP_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define QD_API_VERSION 1

typedef int qd_status;
enum {
  QD_OK = 0,
  QD_ERR_INVALID = 1,     /* bad argument, size or handle */
  QD_ERR_OOM = 2,         /* device allocation failed */
  QD_ERR_CUDA = 3,        /* a CUDA runtime call failed */
  QD_ERR_BREAKDOWN = 4,   /* Krylov breakdown (norm < 1e-10); reported, not fatal */
  QD_ERR_TIMEOUT = 5,     /* a bounded device-side wait gave up */
  QD_ERR_UNSUPPORTED = 6, /* valid request the engine does not implement */
  QD_ERR_OVERFLOW = 7,    /* a per-column leaf table or an index type overflowed */
  QD_ERR_NOT_HERMITIAN = 8,
  QD_ERR_BUSY = 9         /* server slot / admission refused for now */
};

typedef struct qd_ctx qd_ctx;
typedef struct qd_sector qd_sector;
typedef struct qd_ham qd_ham;
typedef struct qd_state qd_state;

/* ------------------------------------------------------------------ */
/* Context                                                            */
/* ------------------------------------------------------------------ */
qd_status qd_ctx_create(int device, qd_ctx **out);
qd_status qd_ctx_destroy(qd_ctx *ctx);
qd_status qd_ctx_sync(qd_ctx *ctx);
/* The CUDA stream (cudaStream_t) all work of this context is issued on. */
qd_status qd_ctx_stream(qd_ctx *ctx, void **stream_out);
/* Number of kernels this context launched since creation (diagnostics). */
qd_status qd_ctx_launch_count(qd_ctx *ctx, int64_t *count);
/* Timing on the context's stream: record event `slot` (0..15); elapsed ms
 * between two recorded slots (waits for the later one). */
qd_status qd_ctx_record(qd_ctx *ctx, int slot);
qd_status qd_ctx_elapsed(qd_ctx *ctx, int slot_a, int slot_b, float *ms);
/* Page-locked host memory for fast host<->device copies. */
qd_status qd_host_alloc(int64_t bytes, void **out);
qd_status qd_host_free(void *p);
const char *qd_status_string(qd_status s);
/* Last error message recorded on this host thread (empty if none). */
const char *qd_last_error(void);
int qd_api_version(void);

/* ------------------------------------------------------------------ */
/* Conserved quantities and sectors                                   */
/*   replaces getQbits (index.hpp:80-94,300), getNset/getNup/getNdo   */
/*   (conservation.hpp:89-115,233-246), getNd/getNh (117-157,248-256),*/
/*   Constrain/LooseConstrain/Evaluate (conservation.hpp:200-231) and */
/*   SubIndex (index.hpp:187-261)                                     */
/* ------------------------------------------------------------------ */
enum { QD_CQ_NSET = 0, QD_CQ_ND = 1 };

typedef struct {
  int32_t kind;  /* QD_CQ_NSET: popcount(state & mask)                       */
                 /* QD_CQ_ND:   popcount(((s>>nsite)^m) & (s^m)), m = hole ?  */
                 /*             low nsite bits : 0 (doublons / holons)       */
  int32_t nsite; /* QD_CQ_ND only */
  int32_t hole;  /* QD_CQ_ND only: 0 = doublon count, 1 = holon count */
  int32_t coef;  /* integer weight of this quantity in the constraint sum */
  uint64_t mask; /* QD_CQ_NSET only */
} qd_cq_term;

/* One `cq = target` argument of Constrain: sum_k coef_k * Q_k == target
 * (|difference| <= tight). */
typedef struct {
  int32_t nterms; /* 1..4 */
  int32_t reserved;
  int64_t target;
  qd_cq_term term[4];
} qd_constraint;

/* Sector of an nbits-qubit register (nbits <= 62).  The basis is every
 * state that satisfies all constraints, in ascending integer order; ncons == 0
 * gives the full 2^nbits space (dim must fit in int32). tight is
 * LooseConstrain's tolerance (0 for Constrain). */
qd_status qd_sector_create(qd_ctx *ctx, int nbits, const qd_constraint *cons,
                           int ncons, int tight, qd_sector **out);
qd_status qd_sector_destroy(qd_sector *sec);
qd_status qd_sector_dim(const qd_sector *sec, int64_t *dim);
/* 1 if ranks come from the combinatorial number system (product of
 * popcount constraints on disjoint contiguous bit fields), 0 if from a search
 * of the sorted basis. */
qd_status qd_sector_rank_kind(const qd_sector *sec, int *kind);
/* Copy the basis (dim states, ascending) to host memory. */
qd_status qd_sector_basis(qd_sector *sec, uint64_t *host_states);
/* rank of each state; states outside the sector get dim (the reference's
 * SubIndex returns range(), index.hpp:234-240). */
qd_status qd_sector_rank(qd_sector *sec, const uint64_t *host_states, int64_t n,
                         int64_t *host_ranks);

/* ------------------------------------------------------------------ */
/* Operator trees                                                     */
/*   replaces bitOp / getBoseGate / getFermiGate (operators/bit.hpp), */
/*   hopBitOp / getHopFermiGate / getHopBoseGate (operators/hopbit.hpp)*/
/*   Operator products (operator.hpp:68-132) and OperatorSum          */
/*   (operator_abel.hpp:9-158)                                        */
/* ------------------------------------------------------------------ */
enum { QD_GATE_BIT = 0, QD_GATE_HOP = 1 };

typedef struct {
  int32_t kind;   /* QD_GATE_BIT or QD_GATE_HOP */
  int32_t site;   /* BIT: the site; HOP: creation site a of gate(a, b) */
  int32_t site_b; /* HOP: annihilation site b of gate(a, b); a == b is n_a */
  int32_t string; /* +1 bosonic gate, -1 fermionic (Jordan-Wigner) gate */
  /* BIT only: the 2x2 matrix given with `gate << U`, row-major,
   * u[2*(2*i+j)] + i*u[2*(2*i+j)+1] = U(i, j).  The amplitude from input bit
   * b to output bit o is U(b, o), i.e. the gate applies U transposed, exactly
   * as elOpBase::operator<< (operator.hpp:24-29) with bitOp::branch
   * (operators/bit.hpp:62-63). */
  double u[8];
} qd_gate;

typedef struct {
  double coeff_re, coeff_im;
  int32_t gate_offset; /* first gate of this product in the gate array */
  int32_t ngates;      /* gates g[off] * g[off+1] * ...; applied right to left */
} qd_term;

/* ------------------------------------------------------------------ */
/* Lowering `OperatorSum >> index`                                     */
/*   replaces Operator::operator>> / full_branch (operator.hpp:135-267) */
/*   and OperatorSum::operator>> (operator_abel.hpp:25-34)            */
/* The result is bit-identical to the reference's Eigen CSC matrix:    */
/* same sparsity pattern (explicit zeros from cross-term cancellation   */
/* kept, leaves with |value| <= 1e-10 dropped before duplicate sums)    */
/* and the same complex128 values.  It is held on the device as CSR,    */
/* built row by row from transitions compiled per term when every term  */
/* acts on at most 6 sites, else by walking each column's operator tree  */
/* (environment QD_LOWER_TREE=1 forces the tree walk; both give the same */
/* matrix).                                                            */
/* ------------------------------------------------------------------ */
enum { QD_HAM_REAL = 1, QD_HAM_HERMITIAN = 2 };

typedef struct {
  int64_t dim;
  int64_t nnz;
  int32_t flags;       /* QD_HAM_REAL | QD_HAM_HERMITIAN */
  int32_t max_row_nnz;
  int32_t has_matrix_free; /* 1 if qd_ham_build_matrix_free succeeded */
  int32_t product_kernel;  /* product the real Lanczos path launches (codes of qd_ham_set_spmv_kernel) */
  int32_t step_launches;   /* kernel launches per Lanczos step of the last real solve on the      */
                           /* uniform-coupling form: 1 (product, dots, update and norm in one    */
                           /* cooperative launch) or 2 (QD_LANCZOS_STEP=split, or a step too big */
                           /* to be resident at once); 0 before such a solve                    */
} qd_ham_info;

qd_status qd_ham_lower(qd_sector *sec, const qd_term *terms, int nterms,
                       const qd_gate *gates, int ngates, qd_ham **out);
qd_status qd_ham_destroy(qd_ham *ham);
qd_status qd_ham_get_info(qd_ham *ham, qd_ham_info *info);

/* *out = a + b for two matrices on the same sector: the union of their
 * patterns, each value a + b (a + 0 where only one has the entry), explicit
 * zeros kept -- Eigen's sparse sum of two lowered SpMatrix values, as
 * Model::getHamiltonianMatrix (lattice.hpp:339-354) and McManager::incrMatrix
 * (mc_manager.hpp:72-79) use it.  The result has no operator terms, so it has
 * no matrix-free form (qd_ham_build_matrix_free answers QD_ERR_UNSUPPORTED). */
qd_status qd_ham_add(const qd_ham *a, const qd_ham *b, qd_ham **out);
/* *out = an independent copy of a (the value semantics of SpMatrix). */
qd_status qd_ham_copy(const qd_ham *a, qd_ham **out);
/* ham *= (re + i im), value by value with the rounding of a std::complex
 * product (McManager::normMatrix, mc_manager.hpp:81-83); the derived forms
 * (fixed-point, matrix-free, cached solver graphs) are dropped. */
qd_status qd_ham_scale(qd_ham *ham, double re, double im);

/* Matrix-free form: replaces Operator::map_acc / OperatorSum::map_acc
 * (operator.hpp:215-232, operator_abel.hpp:36-49).  Compiles the operator
 * tree into per-support transitions (terms of at most 6 sites, at most 512
 * state-changing transitions in all) and a stored diagonal; products then read
 * only the basis, the diagonal and the vectors.  Solvers take it with
 * qd_lanczos_opts.spmv = QD_SPMV_MATRIX_FREE (built on demand).  For real
 * operators with one value on every off-diagonal entry, the matrix-free
 * Lanczos recurrence runs the exact fixed-point slot form (kernel code 121)
 * built from the transitions alone (no stored matrix is read), bit-identical
 * to the stored-matrix recurrence; other operators take the FP64 product. */
qd_status qd_ham_build_matrix_free(qd_ham *ham);
/* y(:, t_out) = H x(:, t_in) through the matrix-free form (x != y). */
qd_status qd_ham_apply_matrix_free(qd_ham *ham, qd_state *x, int t_in,
                                   qd_state *y, int t_out);
/* Reference layout: column pointers (dim+1), row indices sorted within each
 * column, complex values (2*nnz doubles). */
qd_status qd_ham_download_csc(qd_ham *ham, int64_t *colptr, int32_t *rowidx,
                              double *vals);
qd_status qd_ham_download_csr(qd_ham *ham, int64_t *rowptr, int32_t *colidx,
                              double *vals);

/* ------------------------------------------------------------------ */
/* States                                                             */
/*   replaces State / getState / operator() / eval (state.hpp:9-104)  */
/* A state is nt complex128 columns of length dim on the device.       */
/* ------------------------------------------------------------------ */
qd_status qd_state_create(qd_ctx *ctx, int64_t dim, int nt, qd_state **out);
qd_status qd_state_destroy(qd_state *st);
qd_status qd_state_upload(qd_state *st, int t, const double *host_complex);
qd_status qd_state_download(qd_state *st, int t, double *host_complex);
/* dst(:, t_dst) = src(:, t_src) on the device (same dim). */
qd_status qd_state_copy(qd_state *src, int t_src, qd_state *dst, int t_dst);
/* Device address of column t (complex128, dim entries). */
qd_status qd_state_device_ptr(qd_state *st, int t, void **dptr);
/* y(:, t_out) = H * x(:, t_in)   (Eigen `H * psi`) */
qd_status qd_ham_apply(qd_ham *ham, qd_state *x, int t_in, qd_state *y,
                       int t_out);
/* psi(:,t)^dagger * H * psi(:,t), unnormalised, as State::eval
 * (state.hpp:33-45). */
qd_status qd_state_eval(qd_state *psi, int t, qd_ham *ham, double *re_im);
/* <psi(:,t)|O_i|psi(:,t)> for nobs operators of psi's sector and context
 * (replaces the loop of McManager::incrAllObs, mc_manager.hpp:88-106):
 * re_im receives 2*nobs doubles; the fused products run back to back with
 * one copy of the results. */
qd_status qd_obs_eval(qd_state *psi, int t, int nobs, qd_ham *const *obs, double *re_im);

/* ------------------------------------------------------------------ */
/* Lanczos ground state                                               */
/*   replaces Arnoldi::getLanczosSolver(...).getGroundState            */
/*   (sparse_algorithm.hpp:395-425, 458-473, 475-604)                  */
/* ------------------------------------------------------------------ */
enum { QD_SPMV_CSR = 0, QD_SPMV_MATRIX_FREE = 1 };
enum { QD_RITZ_STORED_BASIS = 0, QD_RITZ_SECOND_PASS = 1 };

typedef struct {
  int32_t krylov_dim; /* kry_dim of getLanczosSolver(index, kry_dim) */
  int32_t spmv;       /* QD_SPMV_CSR or QD_SPMV_MATRIX_FREE */
  int32_t ritz;       /* QD_RITZ_STORED_BASIS (default) or QD_RITZ_SECOND_PASS */
  int32_t add_dim;    /* getGroundState's add_dim: 0 or -1 runs krylov_dim steps; k in
                         1..krylov_dim-1 runs k steps now and keeps the solve open for
                         qd_lanczos_extend (updateKrylovRepr, sparse_algorithm.hpp:521-546) */
} qd_lanczos_opts;

typedef struct {
  int32_t act_dim;    /* Krylov dimension reached (act_dim() of the solver) */
  int32_t breakdown;  /* 1 if the recurrence stopped at norm < 1e-10 */
  int32_t matvecs;    /* sparse matrix-vector products performed */
  int32_t reserved;
  double ritz_value;  /* lowest eigenvalue of the Krylov matrix */
  double err;         /* error(): norm of eigenvalue change (first call: |lambda_0|) */
} qd_lanczos_result;

/* psi(:, t) is the start vector on entry and the (unnormalised) Ritz vector on
 * exit, exactly as getGroundState overwrites psi(tstp).  evals_out (may be
 * NULL) receives act_dim ascending Krylov eigenvalues. */
qd_status qd_lanczos_ground(qd_ham *ham, qd_state *psi, int t,
                            const qd_lanczos_opts *opts, double *evals_out,
                            qd_lanczos_result *res);

/* A later getGroundState(H, psi, tstp, add_dim) on the same solver:
 * continues the last qd_lanczos_ground on this operator (same krylov_dim and
 * product kind) for opts->add_dim more steps (0 or -1: up to krylov_dim) from
 * its stored basis, then writes the Ritz vector of the grown space to
 * psi(:, t) and the eigenvalues to evals_out.  A solve that broke down, or
 * whose buffers a Krylov evolution on the operator reused, does not grow. */
qd_status qd_lanczos_extend(qd_ham *ham, qd_state *psi, int t, const qd_lanczos_opts *opts,
                            double *evals_out, qd_lanczos_result *res);

/* ------------------------------------------------------------------ */
/* Krylov real-time step                                              */
/*   replaces ArnoldiSolver<T,0>::evolve (sparse_algorithm.hpp:548-562)*/
/*   with expandBasis<0> (:372-393) and MatrixExp (matrix.hpp:20)     */
/* psi(:, t_out) = V exp(-i K h) e_0 with m-1 Arnoldi products from      */
/* psi(:, t_in) normalised; unit norm for Hermitian H.  t_out may equal  */
/* t_in.  act_dim (may be NULL) receives the Krylov dimension used.      */
/* m (the solver's kry_dim) must be in 2..33.                           */
/* ------------------------------------------------------------------ */
qd_status qd_arnoldi_evolve(qd_ham *ham, qd_state *psi, int t_in, int t_out,
                            double h, int m, int *act_dim);

/* ------------------------------------------------------------------ */
/* Arnoldi ground state (non-Hermitian solver, incremental)            */
/*   replaces Arnoldi::getSolver(index, kry_dim).getGroundState(H, psi,*/
/*   tstp, add_dim) -- ArnoldiSolver<T,0>: getGroundState             */
/*   (sparse_algorithm.hpp:564-585), updateKrylovRepr (:521-546),     */
/*   expandBasis<0> (:372-393), getState<herm 0> (:447-453)           */
/* The basis grows by full orthogonalisation of H v_{k-1} against every */
/* previous vector (two classical Gram-Schmidt passes; the reference's  */
/* modified Gram-Schmidt up to rounding); the breaking step (norm <     */
/* 1e-10) counts.  As the reference's SelfAdjointEigenSolver, the       */
/* eigensolve reads the Arnoldi matrix's lower triangle: the real parts */
/* of <v_i, H v_i> and the sub-diagonal norms.  psi(:, t) is the start  */
/* vector on entry and the Ritz vector V z_0 on exit; evals_out (may be */
/* NULL, krylov_dim doubles) receives act_dim ascending eigenvalues.    */
/* opts->krylov_dim is kry_dim, opts->add_dim the steps of this call    */
/* (0 or -1: up to kry_dim); spmv and ritz are ignored (CSR products).  */
/* res->err is |lambda_0| (a fresh solve) or, after qd_arnoldi_extend,  */
/* |lambda_0 - previous lambda_0|; front ends compute error() over the  */
/* convergeEV eigenvalues from evals_out.                               */
/* ------------------------------------------------------------------ */
qd_status qd_arnoldi_ground(qd_ham *ham, qd_state *psi, int t, const qd_lanczos_opts *opts,
                            double *evals_out, qd_lanczos_result *res);
/* A later getGroundState(H, psi, tstp, add_dim) on the same solver: grows
 * the last qd_arnoldi_ground on this operator (same krylov_dim) by
 * opts->add_dim steps from its stored basis and writes the new Ritz vector;
 * a space that reached krylov_dim or closed by breakdown does not grow. */
qd_status qd_arnoldi_extend(qd_ham *ham, qd_state *psi, int t, const qd_lanczos_opts *opts,
                            double *evals_out, qd_lanczos_result *res);

/* ------------------------------------------------------------------ */
/* Batched mixed-precision Lanczos ground states                      */
/*   many independent getGroundState solves (sparse_algorithm.hpp:    */
/*   564-585) in one persistent launch                                 */
/* Each instance: real Hamiltonian `hams[i]` (same context), host start  */
/* vector v0s[i] (dim doubles), `steps` Lanczos steps with FP32 products  */
/* and basis, FP64 accumulation of inner products, one full             */
/* reorthogonalisation pass per step, a device tridiagonal solve and one  */
/* FP64 Rayleigh-quotient refinement.  out: 8 doubles per instance --     */
/* lowest Krylov eigenvalue, refined energy, psi^T psi, act_dim,          */
/* breakdown flag, the instance's start and end on the device clock    */
/* (%globaltimer, ns), and the number of CTAs that computed it.         */
/* ------------------------------------------------------------------ */
qd_status qd_batch_lanczos(qd_ctx *ctx, int ninst, qd_ham *const *hams,
                           const double *const *v0s, int steps, double *out);

/* ------------------------------------------------------------------ */
/* Batched Krylov real-time steps                                     */
/*   ArnoldiSolver<T,0>::evolve (sparse_algorithm.hpp:548-562) for     */
/*   nvec columns at once, one persistent launch, FP64                 */
/* Y[:, b] = V exp(-i K h) e_0 for X[:, b] (device complex128, leading  */
/* dimension ldx; X == NULL means the unit vectors e_0 .. e_{nvec-1},   */
/* i.e. the first nvec columns of exp(-i H h)).  Y is device complex128 */
/* with leading dimension ldy.  act_dims (host, may be NULL) receives    */
/* each column's Krylov dimension.  m <= 32.                            */
/* ------------------------------------------------------------------ */
qd_status qd_krylov_evolve_batch(qd_ham *ham, const double *d_X, int64_t ldx,
                                 int nvec, double h, int m, double *d_Y,
                                 int64_t ldy, int *act_dims);

/* ------------------------------------------------------------------ */
/* Quantum-jump trajectories                                           */
/*   the jump loop of programs/hubbard_diss.cpp:439-482 (weights        */
/*   :520-529, no-jump generator :514-517, channel search :565-577)    */
/* heff must be the no-jump generator H - (i/2) gamma sum_j n_j of the  */
/* jump operators L_j = sqrt(gamma) n_{chan_bits[j]}.  Every trajectory  */
/* starts from psi0 (host complex128), runs nsteps steps of length dt,   */
/* draws its random numbers from Philox4x32-10 keyed by (seed,           */
/* trajectory, step), and records <n_{obs_a[k]} n_{obs_b[k]}> after      */
/* every step.  obs_mean and obs_stderr receive (nsteps+1) x nobs        */
/* doubles (row = step).  Where heff has dim <= 5120 on at most 32 bits  */
/* and one off-diagonal value +-c, each trajectory runs in one SM's      */
/* shared memory (complex64 vectors, exp(-i heff dt) by a truncated      */
/* Taylor series whose degree and sub-steps follow the series' remainder */
/* bound, at most m-1 products per sub-step); otherwise every step is an */
/* FP64 Arnoldi exponential with m vectors per trajectory.  The          */
/* environment variable QD_TRAJ_ARNOLDI=1 selects the second form.       */
/* ------------------------------------------------------------------ */
typedef struct {
  int32_t ntraj;
  int32_t nsteps;
  double dt;
  double gamma;
  uint64_t seed;
  int32_t m;
  int32_t nchan;              /* <= 32 */
  const int32_t *chan_bits;   /* nchan bit indices */
  int32_t nobs;               /* <= 16 */
  int32_t reserved;
  const int32_t *obs_a;
  const int32_t *obs_b;
} qd_traj_desc;

typedef struct {
  int64_t jumps;        /* jumps over all trajectories */
  double setup_ms;      /* building and uploading the resident form */
  double ensemble_ms;   /* the nsteps steps of all trajectories */
  int32_t path;         /* 0: resident Taylor kernel, 1: FP64 Arnoldi steps */
  int32_t products;     /* sparse products per trajectory step (Taylor terms x sub-steps, or m - 1) */
} qd_traj_stats;

qd_status qd_traj_run(qd_ham *heff, const qd_traj_desc *desc, const double *psi0,
                      double *obs_mean, double *obs_stderr, qd_traj_stats *stats);

/* Average device time of the sparse product kernel the solvers use on this
 * Hamiltonian (iters back-to-back launches on the context stream, timed with
 * CUDA events), and the kernel's algorithmic HBM bytes per launch:
 * CSR: nnz*(value + 4) + (dim+1)*8 + dim*(x + y) bytes; 120: nnz_offdiag*4 +
 * (dim+1)*4 + dim*(8 diagonal + 8 x + 16 fixed-point x + 8 y); 121: dim*(4
 * state + 8 diagonal + 8 x + 16 fixed-point x + 8 y); 1 (matrix-free):
 * dim*(8 basis + diagonal + x + y), or, where one value c is on every
 * off-diagonal entry, the 121 slot form built from the terms alone with its
 * fused inner products, dim*(4 + 8 + 8 + 16 + 8 + 8).  Code 0 times what the
 * Lanczos path launches (for 120 and 121 with the fused inner products: + 8 v2
 * per row).
 * Diagnostic codes:
 * 2000 + kernel times the product with the fused Lanczos dot epilogue; 3001
 * and 3002 time the two Lanczos vector kernels alone (real Hamiltonians). */
qd_status qd_ham_time_spmv(qd_ham *ham, int spmv, int iters, double *avg_ms,
                           double *bytes_per_launch);

/* Product kernels the Lanczos recurrence launches.  CSR: 100 warp tile (lane
 * per row), 101 balanced warp tile (equal nnz per lane), 102/103/104 two/four/
 * eight lanes per row, 105 thread per row, 106/107 thread per row with 4/8
 * loads in flight (108/109 streaming loads), 110 thread per row with an
 * exact-count tail (the default CSR kernel), 111 as 110 in length order.
 * 120: the uniform-coupling form -- when every off-diagonal entry of a real
 * operator has one value c, the diagonal and the columns are kept without
 * values and each row's off-diagonal sum is accumulated exactly in 128-bit
 * fixed point from a fixed-point copy of the vector, rounded once to FP64.
 * It is the default wherever it applies (real start vector); choosing any
 * other code turns it off.  121: the same form with the columns computed on
 * the fly from the operator's terms instead of read (product sectors of at
 * most 32 bits; kept only after a build-time check that every row's columns
 * equal its stored ones, so 121 and 120 give bit-identical solves).  All
 * give the same products up to rounding. */
qd_status qd_ham_set_spmv_kernel(qd_ham *ham, int kernel);
/* Time every product kernel on this Hamiltonian (120 and 121 included where
 * they apply, timed as the recurrence launches them, with its inner products)
 * and keep the fastest for the solvers (the autotuner); returns the choice
 * and its average ms. */
qd_status qd_ham_autotune(qd_ham *ham, int iters, int *chosen, double *best_ms);

/* <psi|H|psi> for a CSR Hamiltonian, with no device allocation at all.
 * No counterpart in the reference: it serves callers that must not call
 * cudaMalloc (an application that owns the device memory pool, or an
 * allocation-free request path).  The caller passes device buffers it owns:
 * d_rowptr (dim+1), d_colidx and d_vals (nnz complex128, interleaved), d_psi
 * (dim complex128) and d_result (2 doubles, written on `stream`).  The work
 * runs on `stream` on the current device.  Scratch is a fixed 32 KB array in
 * the library's device image, so dim is limited to 4,194,304 rows (larger
 * sizes are rejected with QD_ERR_INVALID).  The first call on each device
 * looks that array up; make it before any stream capture.  Calls that overlap
 * on one device race on the shared scratch. */
qd_status qd_csr_expect_noalloc(const int64_t *d_rowptr, const int32_t *d_colidx,
                                const double *d_vals, int64_t dim,
                                const double *d_psi, double *d_result,
                                void *stream);

/* ------------------------------------------------------------------ */
/* Hermitian Lanczos ground state                                     */
/*   replaces Hermitian::LanczosSolver::getGroundState                */
/*   (sparse_algorithm.hpp:287-301) with getKrylovReprAd (:72-122)    */
/*   and getKrylovGS (:206-238)                                       */
/* Two-vector recurrence (no stored basis), stop once ||r||^2 <= 1e-10; */
/* the ground-state vector is rebuilt by a second pass and written to    */
/* psi(:, t).  Up to kry_dim + 1 Lanczos coefficients, as the reference's */
/* loop; evals_out (NULL or kry_dim + 1 doubles) receives res->act_dim     */
/* eigenvalues of the tridiagonal matrix; one product per step and pass. */
/* ------------------------------------------------------------------ */
qd_status qd_hermitian_lanczos_ground(qd_ham *ham, qd_state *psi, int t, int kry_dim,
                                      double *evals_out, qd_lanczos_result *res);

/* ------------------------------------------------------------------ */
/* Short-recurrence Krylov real-time step (Hermitian operators)       */
/*   same result as qd_arnoldi_evolve (ArnoldiSolver<T,0>::evolve,    */
/*   sparse_algorithm.hpp:548-562) up to rounding: for Hermitian H the */
/*   Arnoldi projection is tridiagonal, so the three-term recurrence   */
/*   builds the same Krylov space with two vector passes per product.  */
/* nsteps steps of length h from psi(:, t_in) into psi(:, t_out), each   */
/* with m - 1 products and the breakdown rule of expandBasis<0>; the     */
/* small exponential exp(-i h T) e_0 is evaluated on the device, so a     */
/* step is one CUDA graph launch with no host round trip.  act_dim gets  */
/* the last step's Krylov dimension.  QD_ERR_NOT_HERMITIAN for other H.  */
/* ------------------------------------------------------------------ */
qd_status qd_lanczos_evolve(qd_ham *ham, qd_state *psi, int t_in, int t_out,
                            double h, int m, int nsteps, int *act_dim);

/* ------------------------------------------------------------------ */
/* Seeded start vectors                                               */
/* Element i = 2u - 1 with u the (i mod 2)-th uniform double of        */
/* Philox4x32-10 (key = seed, counter = (i / 2, 0x53544152, 0, 0)).     */
/* Host-only; the request loop draws the same vector on the device.   */
/* ------------------------------------------------------------------ */
qd_status qd_seeded_start(uint64_t seed, int64_t dim, double *host_out);

/* ------------------------------------------------------------------ */
/* Request loop (serving)                                             */
/*   no counterpart in the reference, which runs one solve per        */
/*   process (programs/*.cpp).  A server owns worker lanes on the      */
/*   context's device, each a CUDA stream driven by a host thread.     */
/* Requests carry an operator description (sector constraints, terms,  */
/* gates -- what qd_sector_create / qd_ham_lower take) and are admitted */
/* in arrival order as lanes free up and as their estimated device      */
/* footprint fits the byte budget; the sector, the lowered Hamiltonian  */
/* and the Krylov basis stay resident on the device for the request's   */
/* lifetime, and requests on different lanes overlap on the GPU.        */
/* Ground state: Lanczos (krylov_dim steps) from the start vector,      */
/* result = Ritz vector.  Evolution: nsteps Krylov steps of length dt   */
/* with dimension m = krylov_dim.                                      */
/* QD_SERVE_PLAIN runs every request with the FP64 reference            */
/* algorithms (qd_lanczos_ground, qd_arnoldi_evolve).  QD_SERVE_MIXED   */
/* batches ground states with dim <= batch_dim and a real start vector  */
/* into one persistent launch per lane pass (qd_batch_lanczos: FP32     */
/* products and basis, FP64 accumulation and refinement), and evolves   */
/* Hermitian operators to T = nsteps * dt with qd_lanczos_evolve and its */
/* own step: m = 32, h = T / ceil(T ||H||_inf / 8) (Krylov error bound    */
/* below 1e-15 per step), or the requested (dt, m) when that is coarser. */
/* ------------------------------------------------------------------ */
enum { QD_REQ_GROUND = 0, QD_REQ_EVOLVE = 1 };
enum { QD_SERVE_PLAIN = 0, QD_SERVE_MIXED = 1 };
enum { QD_PATH_GRID = 0, QD_PATH_BATCH = 1 };

typedef struct qd_server qd_server;

typedef struct qd_server_opts {
  int32_t mode;         /* QD_SERVE_PLAIN or QD_SERVE_MIXED */
  int32_t small_lanes;  /* lanes for requests with dim <= small_dim (default 4) */
  int32_t large_lanes;  /* lanes for any request (default 3) */
  int32_t batch_lanes;  /* QD_SERVE_MIXED: lanes for batched ground states (default 2) */
  int32_t batch_max;    /* requests per batched launch (default 64) */
  int32_t batch_min;    /* QD_SERVE_MIXED: a batch lane starts once this many batchable ground states
                           wait (default 4); fewer go to the small lanes one by one */
  int64_t small_dim;    /* default 65536 */
  int64_t hbm_budget;   /* bytes admitted requests may hold; 0 = 80% of free memory */
  int64_t batch_dim;    /* QD_SERVE_MIXED: ground states with dim <= batch_dim are batched (default 3432) */
  int32_t reserved[2];
} qd_server_opts;

typedef struct qd_request {
  int32_t kind;                /* QD_REQ_GROUND or QD_REQ_EVOLVE */
  int32_t nbits;
  int32_t ncons;
  int32_t tight;
  const qd_constraint *cons;
  const qd_term *terms;
  const qd_gate *gates;
  int32_t nterms;
  int32_t ngates;
  int32_t krylov_dim;          /* ground: Lanczos steps (1..256); evolve: m (2..33) */
  int32_t nsteps;              /* evolve: number of steps of length dt */
  double dt;
  const double *psi0;          /* complex128[psi0_len] start state, copied at submit; NULL: seeded */
  int64_t psi0_len;            /* must equal the sector dimension when psi0 is given */
  uint64_t seed;               /* qd_seeded_start(seed, dim) when psi0 is NULL */
  double *psi_out;             /* complex128 result state, written before the result is posted; or NULL */
  int64_t psi_out_len;         /* capacity of psi_out in complex elements */
  uint64_t tag;                /* returned unchanged in the result */
} qd_request;

typedef struct qd_result {
  uint64_t id;
  uint64_t tag;
  int32_t status;              /* QD_OK or the failing status */
  int32_t kind;
  int32_t path;                /* QD_PATH_GRID or QD_PATH_BATCH */
  int32_t act_dim;             /* Krylov dimension of the (last) solve */
  int64_t dim;
  int64_t nnz;
  int64_t matvecs;
  int64_t bytes;               /* device bytes the request held */
  double energy;               /* Re <psi|H|psi> / <psi|psi> of the result state */
  double ritz;                 /* ground: lowest Ritz value; evolve: 0 */
  double norm;                 /* ||result state|| */
  double t_submit, t_admit, t_done;  /* seconds on the server clock */
} qd_result;

typedef struct qd_server_stats {
  int64_t submitted, completed, failed, queued, active, max_active;
  int64_t batches, batched;    /* batched launches and the requests they carried */
  int64_t bytes_in_use, bytes_peak, budget;
} qd_server_stats;

qd_status qd_server_create(qd_ctx *ctx, const qd_server_opts *opts, qd_server **out);
/* Copies the request description and start state; psi_out must stay valid
 * until the request's result has been polled. */
qd_status qd_server_submit(qd_server *srv, const qd_request *req, uint64_t *id);
/* Up to max finished results; waits up to timeout_ms for the first one. */
qd_status qd_server_poll(qd_server *srv, qd_result *out, int max, int *n, int timeout_ms);
qd_status qd_server_now(qd_server *srv, double *seconds);
qd_status qd_server_get_stats(qd_server *srv, qd_server_stats *st);
/* Finishes the running requests, drops the queued ones, joins the lanes. */
qd_status qd_server_destroy(qd_server *srv);

#ifdef __cplusplus
}
#endif
#endif /* QUDRIP_GB300_H */
