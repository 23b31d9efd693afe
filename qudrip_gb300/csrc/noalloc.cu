// noalloc.cu -- <psi|H|psi> for a CSR Hamiltonian without any device allocation.
//
// Who needs this: callers that are not allowed to allocate device memory.
// Typical cases are a host application that owns the whole device memory
// pool and forbids foreign cudaMalloc calls, and a latency-critical request
// path where an allocation could stall or fragment memory in the middle of
// serving.  Such callers hand in device buffers they already own (the CSR
// arrays, the state and a two-double output) and this entry point only
// launches a kernel on their stream.
//
// The reduction scratch (one partial sum per block plus a ticket counter)
// lives in the file-scope array g_noalloc_scratch below.  Every GPU that loads
// the library holds it (about 32 KB) until the process exits.  Host code may
// not use the array's name as a device address, so the first call on each
// device looks the address up with cudaGetSymbolAddress while that device is
// current; make that first call before any stream capture.  All calls on one
// device share that device's array: the ticket is cleared at the start of
// every call, and calls that overlap on the GPU (for example on two streams
// of the same device) race on it -- serialise them.
#include <mutex>

#include "vec.cuh"

namespace qd {

constexpr int kNoAllocThreads = 256;
constexpr int kNoAllocRowsPerThread = 8;
constexpr int kNoAllocRowsPerBlock = kNoAllocThreads * kNoAllocRowsPerThread;  // 2048
constexpr int kNoAllocMaxBlocks = 2048;
constexpr int64_t kNoAllocMaxDim = (int64_t)kNoAllocMaxBlocks * kNoAllocRowsPerBlock;  // 4,194,304 rows

struct NoAllocScratch {
  cplx partials[kNoAllocMaxBlocks];
  unsigned int ticket;
};

static __device__ __align__(256) NoAllocScratch g_noalloc_scratch;

__global__ void __launch_bounds__(kNoAllocThreads) expect_noalloc_kernel(int64_t dim, const int64_t* rowptr,
                                                                         const int32_t* colidx, const cplx* vals,
                                                                         const cplx* psi, NoAllocScratch* scratch,
                                                                         cplx* result) {
  cplx acc = mkc(0.0, 0.0);
  const int64_t base = (int64_t)blockIdx.x * kNoAllocRowsPerBlock;
  for (int i = 0; i < kNoAllocRowsPerThread; ++i) {
    const int64_t r = base + (int64_t)i * kNoAllocThreads + threadIdx.x;
    if (r >= dim) break;
    cplx hr = mkc(0.0, 0.0);
    for (int64_t k = rowptr[r]; k < rowptr[r + 1]; ++k) hr = vfma(vals[k], ld_ro(psi + colidx[k]), hr);
    acc = vdotfma(psi[r], hr, acc);  // conj(psi_r) (H psi)_r
  }
  grid_sum(acc, GridRed<cplx>{scratch->partials, &scratch->ticket}, result);
}

static std::mutex g_noalloc_mutex;
static NoAllocScratch* g_noalloc_addr[64] = {};

}  // namespace qd

using namespace qd;

extern "C" qd_status qd_csr_expect_noalloc(const int64_t* d_rowptr, const int32_t* d_colidx, const double* d_vals,
                                          int64_t dim, const double* d_psi, double* d_result, void* stream) {
  return guard([&] {
    QD_REQUIRE(d_rowptr && d_colidx && d_vals && d_psi && d_result, QD_ERR_INVALID,
               "qd_csr_expect_noalloc: null device pointer");
    QD_REQUIRE(dim >= 1, QD_ERR_INVALID, "qd_csr_expect_noalloc: dim must be >= 1");
    QD_REQUIRE(dim <= kNoAllocMaxDim, QD_ERR_INVALID,
               "qd_csr_expect_noalloc: dim %lld exceeds the fixed scratch limit of %lld rows",
               (long long)dim, (long long)kNoAllocMaxDim);
    int dev = 0;
    QD_CUDA(cudaGetDevice(&dev));
    QD_REQUIRE(dev >= 0 && dev < 64, QD_ERR_UNSUPPORTED, "qd_csr_expect_noalloc: device %d out of range", dev);
    NoAllocScratch* scratch = nullptr;
    {
      std::lock_guard<std::mutex> lk(g_noalloc_mutex);
      if (!g_noalloc_addr[dev]) {
        void* p = nullptr;
        QD_CUDA(cudaGetSymbolAddress(&p, g_noalloc_scratch));  // the current device's copy
        g_noalloc_addr[dev] = static_cast<NoAllocScratch*>(p);
      }
      scratch = g_noalloc_addr[dev];
    }
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    QD_CUDA(cudaMemsetAsync(&scratch->ticket, 0, sizeof(unsigned int), s));
    const unsigned grid = (unsigned)((dim + kNoAllocRowsPerBlock - 1) / kNoAllocRowsPerBlock);
    expect_noalloc_kernel<<<grid, kNoAllocThreads, 0, s>>>(dim, d_rowptr, d_colidx,
                                                           reinterpret_cast<const cplx*>(d_vals),
                                                           reinterpret_cast<const cplx*>(d_psi), scratch,
                                                           reinterpret_cast<cplx*>(d_result));
    QD_CHECK_LAUNCH();
  });
}
