// scan.cu -- exclusive prefix sum of int64 arrays: each block scans a tile of
// kTile elements, the tile totals are scanned recursively, then added back.
#include "scan.cuh"

namespace qd {

constexpr int kScanBlock = 512;
constexpr int kPerThread = 4;
constexpr int kTile = kScanBlock * kPerThread;

__global__ void tile_scan_kernel(const int64_t* in, int64_t* out, int64_t n, int64_t* tile_sums) {
  __shared__ int64_t warp_tot[kScanBlock / 32];
  const int64_t base = (int64_t)blockIdx.x * kTile + (int64_t)threadIdx.x * kPerThread;
  int64_t v[kPerThread];
  int64_t local = 0;
#pragma unroll
  for (int i = 0; i < kPerThread; ++i) {
    v[i] = (base + i < n) ? in[base + i] : 0;
    local += v[i];
  }
  // inclusive warp scan of the per-thread totals
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int64_t incl = local;
  for (int o = 1; o < 32; o <<= 1) {
    const int64_t t = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += t;
  }
  if (lane == 31) warp_tot[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    int64_t w = (lane < kScanBlock / 32) ? warp_tot[lane] : 0;
    for (int o = 1; o < 32; o <<= 1) {
      const int64_t t = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += t;
    }
    if (lane < kScanBlock / 32) warp_tot[lane] = w;  // inclusive
  }
  __syncthreads();
  int64_t run = incl - local + (warp > 0 ? warp_tot[warp - 1] : 0);
#pragma unroll
  for (int i = 0; i < kPerThread; ++i) {
    if (base + i < n) out[base + i] = run;
    run += v[i];
  }
  if (threadIdx.x == kScanBlock - 1) tile_sums[blockIdx.x] = run;
}

__global__ void tile_add_kernel(int64_t* out, int64_t n, const int64_t* tile_offsets) {
  const int64_t base = (int64_t)blockIdx.x * kTile + (int64_t)threadIdx.x * kPerThread;
  const int64_t add = tile_offsets[blockIdx.x];
#pragma unroll
  for (int i = 0; i < kPerThread; ++i)
    if (base + i < n) out[base + i] += add;
}

void exclusive_scan_i64(Ctx* ctx, const int64_t* in, int64_t* out, int64_t n) {
  if (n <= 0) return;
  const int64_t ntiles = ceil_div(n, kTile);
  DBuf<int64_t> sums(ntiles);
  tile_scan_kernel<<<(unsigned)ntiles, kScanBlock, 0, ctx->stream>>>(in, out, n, sums.p);
  QD_CHECK_LAUNCH();
  QD_LAUNCHED(ctx);
  if (ntiles > 1) {
    exclusive_scan_i64(ctx, sums.p, sums.p, ntiles);
    tile_add_kernel<<<(unsigned)ntiles, kScanBlock, 0, ctx->stream>>>(out, n, sums.p);
    QD_CHECK_LAUNCH();
    QD_LAUNCHED(ctx);
  }
  // keep `sums` alive until the kernels that read it have run
  QD_CUDA(cudaStreamSynchronize(ctx->stream));
}

}  // namespace qd
