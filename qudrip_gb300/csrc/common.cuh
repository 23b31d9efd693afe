// common.cuh -- shared infrastructure of the GB300 engine: status handling,
// device allocation bookkeeping, exact (non-contracted) complex arithmetic.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>

#include "../../include/qudrip_gb300.h"

namespace qd {

// ---------------------------------------------------------------- errors
void set_error(const char* fmt, ...);
void clear_error();

struct Error {
  qd_status code;
};

#define QD_CUDA(call)                                                                  \
  do {                                                                                 \
    cudaError_t e__ = (call);                                                          \
    if (e__ != cudaSuccess) {                                                          \
      ::qd::set_error("%s:%d %s: %s", __FILE__, __LINE__, #call, cudaGetErrorString(e__)); \
      throw ::qd::Error{e__ == cudaErrorMemoryAllocation ? QD_ERR_OOM : QD_ERR_CUDA};  \
    }                                                                                  \
  } while (0)

#define QD_REQUIRE(cond, code, ...)   \
  do {                                \
    if (!(cond)) {                    \
      ::qd::set_error(__VA_ARGS__);   \
      throw ::qd::Error{code};        \
    }                                 \
  } while (0)

#define QD_LAUNCHED(ctx) ((ctx)->launches++)

#define QD_CHECK_LAUNCH()                                                              \
  do {                                                                                 \
    cudaError_t e__ = cudaGetLastError();                                              \
    if (e__ != cudaSuccess) {                                                          \
      ::qd::set_error("%s:%d kernel launch: %s", __FILE__, __LINE__, cudaGetErrorString(e__)); \
      throw ::qd::Error{QD_ERR_CUDA};                                                  \
    }                                                                                  \
  } while (0)

// Wrap a C-ABI body: converts thrown qd::Error into a status code.
template <typename F>
qd_status guard(F&& f) {
  try {
    clear_error();
    f();
    return QD_OK;
  } catch (const Error& e) {
    return e.code;
  } catch (...) {
    set_error("unexpected host exception");
    return QD_ERR_INVALID;
  }
}

// ---------------------------------------------------------------- device buffers
// Stream on which this thread's DBuf allocations are ordered.  Null (the
// default) means cudaMalloc / cudaFree.  Request-loop worker threads set their
// lane's stream, so their allocations come from the stream-ordered pool
// (cudaMallocAsync / cudaFreeAsync), which does not serialise the other
// lanes' kernels the way cudaMalloc / cudaFree do.
inline cudaStream_t& alloc_stream() {
  static thread_local cudaStream_t s = nullptr;
  return s;
}
struct AllocStreamScope {
  cudaStream_t prev;
  explicit AllocStreamScope(cudaStream_t s) : prev(alloc_stream()) { alloc_stream() = s; }
  ~AllocStreamScope() { alloc_stream() = prev; }
};

// Owning device buffer; never copied.
template <typename T>
struct DBuf {
  T* p = nullptr;
  size_t n = 0;
  cudaStream_t s = nullptr;  // stream the buffer was allocated on (stream-ordered pool), or null
  DBuf() = default;
  explicit DBuf(size_t count) { alloc(count); }
  DBuf(const DBuf&) = delete;
  DBuf& operator=(const DBuf&) = delete;
  DBuf(DBuf&& o) noexcept : p(o.p), n(o.n), s(o.s) {
    o.p = nullptr;
    o.n = 0;
    o.s = nullptr;
  }
  DBuf& operator=(DBuf&& o) noexcept {
    if (this != &o) {
      release();
      p = o.p;
      n = o.n;
      s = o.s;
      o.p = nullptr;
      o.n = 0;
      o.s = nullptr;
    }
    return *this;
  }
  ~DBuf() { release(); }
  void alloc(size_t count) {
    release();
    if (count == 0) count = 1;
    s = alloc_stream();
    if (s)
      QD_CUDA(cudaMallocAsync((void**)&p, count * sizeof(T), s));
    else
      QD_CUDA(cudaMalloc((void**)&p, count * sizeof(T)));
    n = count;
  }
  void release() {
    if (p) {
      if (s)
        cudaFreeAsync(p, s);
      else
        cudaFree(p);
    }
    p = nullptr;
    n = 0;
    s = nullptr;
  }
  size_t bytes() const { return n * sizeof(T); }
};

// ---------------------------------------------------------------- context
struct Ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  int num_sms = 0;
  int64_t launches = 0;
  cudaEvent_t events[16] = {};
};

struct DeviceGuard {
  int prev = -1;
  explicit DeviceGuard(int dev) {
    cudaGetDevice(&prev);
    if (prev != dev) cudaSetDevice(dev);
  }
  ~DeviceGuard() {
    int cur = -1;
    cudaGetDevice(&cur);
    if (prev >= 0 && cur != prev) cudaSetDevice(prev);
  }
};

inline int64_t ceil_div(int64_t a, int64_t b) { return (a + b - 1) / b; }

}  // namespace qd

// ---------------------------------------------------------------- device math
// Complex arithmetic with one rounding per product and per sum (the
// __d*_rn intrinsics are never contracted into FMA).  This reproduces the
// reference's std::complex<double> results bit for bit.
struct __align__(16) cplx {
  double re, im;
};

__host__ __device__ inline cplx mkc(double r, double i) {
  cplx c;
  c.re = r;
  c.im = i;
  return c;
}

#ifdef __CUDACC__
__device__ __forceinline__ cplx cmul_rn(cplx a, cplx b) {
  return mkc(__dsub_rn(__dmul_rn(a.re, b.re), __dmul_rn(a.im, b.im)),
             __dadd_rn(__dmul_rn(a.re, b.im), __dmul_rn(a.im, b.re)));
}
__device__ __forceinline__ cplx cadd_rn(cplx a, cplx b) {
  return mkc(__dadd_rn(a.re, b.re), __dadd_rn(a.im, b.im));
}
__device__ __forceinline__ cplx rmul_rn(double r, cplx b) {
  return mkc(__dmul_rn(r, b.re), __dmul_rn(r, b.im));
}
#endif
