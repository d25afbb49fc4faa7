// ibm_residual_noalloc: r = b - A x and the norms ||r||_2, ||b||_2 for one
// 7-point operator, with no device allocation at all.
//
// Who needs this: callers that cannot call cudaMalloc. Typical ones hand all
// free device memory to their own pool allocator at start-up (so a foreign
// cudaMalloc fails or fragments their pool), run under a fixed device-memory
// budget where an out-of-memory error mid-run is not acceptable, or cannot
// accept the device-wide synchronisation that cudaFree implies. Every other
// entry point of this library works through a context, and creating a context
// allocates; this one needs none.
//
// Its only scratch is the file-scope array below: per-tile partial sums of the
// two norms and the counter that elects the block finishing the reduction.
// The array lives in the library's module and is held on every device that
// loads the library until the process exits. Its address in the current
// context is looked up with cudaGetSymbolAddress on every call made outside
// stream capture, so a device reset or another context made current on the
// device is followed; a call made while its stream is being captured reuses
// the address found by the last uncaptured call on that device. In host code
// the array's name is only a stand-in for the symbol, never a device address.
#include <cmath>
#include <mutex>

#include "ibm_common.cuh"

namespace ibm {
namespace {

constexpr long kNaMaxRows = IBM_NOALLOC_MAX_ROWS;
constexpr int kNaMaxTiles = (int)(kNaMaxRows / kTile);
constexpr int kNaMaxDevices = 64;
static_assert(kNaMaxRows % kTile == 0, "the row limit is a whole number of tiles");

struct NoAllocScratch {
  double part[2 * kNaMaxTiles];  // per tile: sum r^2, sum b^2
  unsigned ticket;               // tiles finished; cleared before every launch
};

}  // namespace

// 2 * 32768 doubles + the counter: 512 KiB + 256 B per device.
static __device__ __align__(256) NoAllocScratch g_noalloc_scratch;

namespace {

// One block per tile of kTile rows. The stencil is evaluated in the same order
// as the context path's operator apply (centre, -x, +x, -y, +y, -z, +z, one fma
// each), so r is bitwise equal to b - ibm_apply_operator(x). The norms are
// summed in a fixed order (rows within a thread, lanes, warps, tiles), so the
// result does not depend on which block finishes last.
__global__ void __launch_bounds__(kThreads)
    k_residual_noalloc(const double *__restrict__ vals, int nx, int ny, int nz, long n,
                       const double *__restrict__ x, const double *__restrict__ b, double *__restrict__ r,
                       double *__restrict__ norms, NoAllocScratch *sc) {
  __shared__ double srr[kWarps], sbb[kWarps];
  __shared__ int last;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const long sy = nx, sz = (long)nx * ny;
  double rr = 0.0, bb = 0.0;
#pragma unroll
  for (int t = 0; t < kRowsPerThread; ++t) {
    const long row = (long)blockIdx.x * kTile + t * kThreads + threadIdx.x;
    if (row < n) {
      int i, j, k;
      row_ijk((int)row, nx, ny, i, j, k);
      const double *c = vals + 7 * row;
      double acc = 0.0;
      acc = fma(c[0], x[row], acc);
      acc = fma(c[1], i > 0 ? x[row - 1] : 0.0, acc);
      acc = fma(c[2], i < nx - 1 ? x[row + 1] : 0.0, acc);
      acc = fma(c[3], j > 0 ? x[row - sy] : 0.0, acc);
      acc = fma(c[4], j < ny - 1 ? x[row + sy] : 0.0, acc);
      acc = fma(c[5], k > 0 ? x[row - sz] : 0.0, acc);
      acc = fma(c[6], k < nz - 1 ? x[row + sz] : 0.0, acc);
      const double bv = b[row];
      const double rv = bv - acc;
      r[row] = rv;
      rr = fma(rv, rv, rr);
      bb = fma(bv, bv, bb);
    }
  }
  rr = warp_sum(rr);
  bb = warp_sum(bb);
  if (lane == 0) {
    srr[warp] = rr;
    sbb[warp] = bb;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0.0, e = 0.0;
    for (int w = 0; w < kWarps; ++w) {
      a += srr[w];
      e += sbb[w];
    }
    sc->part[2 * blockIdx.x] = a;
    sc->part[2 * blockIdx.x + 1] = e;
    __threadfence();
    last = atomicAdd(&sc->ticket, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  double a = 0.0, e = 0.0;
  for (int q = threadIdx.x; q < (int)gridDim.x; q += kThreads) {
    a += __ldcg(&sc->part[2 * q]);
    e += __ldcg(&sc->part[2 * q + 1]);
  }
  a = warp_sum(a);
  e = warp_sum(e);
  __syncthreads();
  if (lane == 0) {
    srr[warp] = a;
    sbb[warp] = e;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double ta = 0.0, te = 0.0;
    for (int w = 0; w < kWarps; ++w) {
      ta += srr[w];
      te += sbb[w];
    }
    norms[0] = sqrt(ta);
    norms[1] = sqrt(te);
    sc->ticket = 0;
  }
}

std::mutex g_na_mutex;
NoAllocScratch *g_na_ptr[kNaMaxDevices] = {};

// The scratch address in the current context. Outside capture it is looked
// up again (cheap, and correct after cudaDeviceReset or with a non-primary
// context current); during capture the last address found on the device is
// used, since the lookup itself may load the module and is not a stream
// operation that capture records.
cudaError_t scratch_on_device(int dev, bool capturing, NoAllocScratch **out) {
  std::lock_guard<std::mutex> lock(g_na_mutex);
  if (!capturing || !g_na_ptr[dev]) {
    void *p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return e;
    g_na_ptr[dev] = (NoAllocScratch *)p;
  }
  *out = g_na_ptr[dev];
  return cudaSuccess;
}

// [a, a + na) and [b, b + nb) share a byte.
bool overlaps(const void *a, size_t na, const void *b, size_t nb) {
  const char *pa = (const char *)a, *pb = (const char *)b;
  return pa < pb + nb && pb < pa + na;
}

bool on_device(const void *p, int dev) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  if (a.type == cudaMemoryTypeManaged) return true;
  return a.type == cudaMemoryTypeDevice && a.device == dev;
}

}  // namespace
}  // namespace ibm

extern "C" int ibm_residual_noalloc(const double *vals, int nx, int ny, int nz, const double *x, const double *b,
                                    double *r, double *norms, void *stream) {
  using namespace ibm;
  if (!vals || !x || !b || !r || !norms || nx <= 0 || ny <= 0 || nz <= 0) return IBM_ERR_ARG;
  const long n = (long)nx * ny * nz;
  if (n > kNaMaxRows) return IBM_ERR_TOO_LARGE;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return IBM_ERR_CUDA;
  if (dev < 0 || dev >= kNaMaxDevices) return IBM_ERR_UNSUPPORTED;
  // r and norms are written while other blocks still read x and b (each row
  // reads its six neighbours): an output sharing memory with an input races.
  const size_t vb = (size_t)n * sizeof(double), nb = 2 * sizeof(double);
  if (overlaps(r, vb, x, vb) || overlaps(r, vb, b, vb) || overlaps(r, vb, vals, 7 * vb) ||
      overlaps(norms, nb, x, vb) || overlaps(norms, nb, b, vb) || overlaps(norms, nb, r, vb) ||
      overlaps(norms, nb, vals, 7 * vb))
    return IBM_ERR_ARG;
  for (const void *p : {(const void *)vals, (const void *)x, (const void *)b, (const void *)r, (const void *)norms})
    if (!on_device(p, dev)) return IBM_ERR_ARG;
  cudaStream_t st = (cudaStream_t)stream;
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(st, &cs) != cudaSuccess) return IBM_ERR_CUDA;
  NoAllocScratch *sc = nullptr;
  if (scratch_on_device(dev, cs != cudaStreamCaptureStatusNone, &sc) != cudaSuccess) return IBM_ERR_CUDA;
  if (cudaMemsetAsync(&sc->ticket, 0, sizeof(unsigned), st) != cudaSuccess) return IBM_ERR_CUDA;
  const int tiles = (int)((n + kTile - 1) / kTile);
  k_residual_noalloc<<<tiles, kThreads, 0, st>>>(vals, nx, ny, nz, n, x, b, r, norms, sc);
  return cudaGetLastError() == cudaSuccess ? IBM_OK : IBM_ERR_CUDA;
}
