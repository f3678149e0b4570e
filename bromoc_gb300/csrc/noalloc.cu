// Ion-ion pair energy and forces without any device allocation.
//
// Some callers cannot allocate device memory while they run: a host program
// that reserves all of its GPU memory once at start-up and treats any later
// allocation as a failure (a long production run under a fixed memory
// budget), or an embedding in which another runtime owns the device
// allocator and forbids outside cudaMalloc/cudaFree calls.  This entry point
// serves them: the caller passes device buffers for the inputs and outputs,
// and the partial forces and block energies the kernel needs as scratch live
// in one file-scope __device__ array that exists from the moment the library
// is loaded on a device until the process exits.
//
// Limits and rules of use:
//   - at most kMaxIons = 4096 ions per call (the scratch is sized for that:
//     16 source chunks x 3 components x 4096 doubles + block energies,
//     about 1.6 MB per device); larger systems are rejected with
//     BROMOC_E_CAPACITY and should use bromoc_gpu_energy;
//   - every call on a device shares the same scratch: two calls whose
//     kernels overlap on the GPU (different streams or host threads without
//     ordering between them) race on it and give wrong results;
//   - the scratch keeps the previous call's contents, so each call writes
//     every slot it later reads (nothing relies on zeroed memory) and clears
//     its error flag itself;
//   - the first call on a device looks up the scratch's device address with
//     cudaGetSymbolAddress (with that device current) and keeps it for the
//     life of the process; make that first call before any stream capture
//     begins.  A device reset (cudaDeviceReset) ends every context of this
//     library and leaves that address stale: the library is not used again
//     in a process after a reset;
//   - each call waits on its stream before it returns (it reads back the
//     error word), so its results are ready when it returns.
#include <cstdio>
#include <mutex>

#include "../../include/bromoc_gpu.h"
#include "launch.h"
#include "physics.cuh"

namespace {

using namespace bgpu;

constexpr int kMaxIons = 4096;
constexpr int kTile = 128;
constexpr int kMaxChunks = 16;
constexpr int kMaxTiles = kMaxIons / kTile;

struct StaticScratch {
  double fpart[kMaxChunks * 3 * kMaxIons];    // per-chunk partial forces
  double epart[kMaxTiles * kMaxChunks * 4];   // per-block energies
  int err;                                    // guard violations this call
};

static __device__ __align__(256) StaticScratch g_scratch;

// device address of g_scratch per device, looked up once
constexpr int kMaxDevices = 64;
StaticScratch *g_addr[kMaxDevices] = {};
std::mutex g_addr_mu;

__device__ __forceinline__ void hi_lo(double v, float &hi, float &lo) {
  hi = (float)v;
  lo = (float)(v - (double)hi);
}

// Block (tile, chunk): 128 mobile targets against the chunk's sources; the
// same pair laws and energy weighting as the context path (a mobile-mobile
// pair counts half on each side, a mobile-fixed pair once).
template <bool FP32>
__global__ void __launch_bounds__(kTile)
    k_pairs_static(KP p, int n, int nfix, int chunk, const double *__restrict__ x,
                   const double *__restrict__ y, const double *__restrict__ z,
                   const int *__restrict__ typei, StaticScratch *s) {
  __shared__ double sx[kTile], sy[kTile], sz[kTile];
  // FP32: each source's coordinates split once into hi + lo floats
  __shared__ float4 shi[FP32 ? kTile : 1], slo[FP32 ? kTile : 1];
  __shared__ int sc[kTile];
  __shared__ double red[(kTile / 32) * 4];
  __shared__ double tot[4];
  const int t = nfix + blockIdx.x * kTile + threadIdx.x;
  const bool tv = t < n;
  const int s0 = blockIdx.y * chunk, s1 = min(n, s0 + chunk);
  int row = 0;
  double xt = 0, yt = 0, zt = 0;
  bool ok = true;
  if (tv) {
    const int it = abs(typei[t]);
    if (it <= p.nold || it > p.ntype) {
      ok = false;
      atomicOr(&s->err, 1);
    } else {
      row = (p.nwtype[it] - 1) * p.nttyp;
    }
    xt = x[t];
    yt = y[t];
    zt = z[t];
  }
  float xh = 0, yh = 0, zh = 0, xl = 0, yl = 0, zl = 0;
  if (FP32) {
    hi_lo(xt, xh, xl);
    hi_lo(yt, yh, yl);
    hi_lo(zt, zh, zl);
  }
  double f[3] = {0, 0, 0}, e[4] = {0, 0, 0, 0};
  int terr = 0;
  for (int base = s0; base < s1; base += kTile) {
    const int src = base + threadIdx.x;
    __syncthreads();
    if (src < s1) {
      const int it = abs(typei[src]);
      const bool good = it > p.nold && it <= p.ntype;
      if (!good) atomicOr(&s->err, 1);
      sx[threadIdx.x] = x[src];
      sy[threadIdx.x] = y[src];
      sz[threadIdx.x] = z[src];
      if (FP32) {
        float4 h, l;
        hi_lo(sx[threadIdx.x], h.x, l.x);
        hi_lo(sy[threadIdx.x], h.y, l.y);
        hi_lo(sz[threadIdx.x], h.z, l.z);
        h.w = l.w = 0.f;
        shi[threadIdx.x] = h;
        slo[threadIdx.x] = l;
      }
      sc[threadIdx.x] = good ? ((p.nwtype[it] - 1) | ((src >= nfix) << 16)) : -1;
    }
    __syncthreads();
    const int m = min(kTile, s1 - base);
    if (tv && ok) {
      float ff[3] = {0.f, 0.f, 0.f}, ef[4] = {0.f, 0.f, 0.f, 0.f};
      for (int k = 0; k < m; ++k) {
        const int code = sc[k];
        if (base + k == t || code < 0) continue;
        const int is = p.pidx[row + (code & 0xffff)];
        if (FP32) {
          const float4 sh = shi[k], sl = slo[k];
          const float dx = (xh - sh.x) + (xl - sl.x), dy = (yh - sh.y) + (yl - sl.y),
                      dz = (zh - sh.z) + (zl - sl.z);
          const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
          const float de =
              law32(p, p.ppf[is], r2, (code >> 16) ? 0.5f : 1.0f, ef, terr, [&] {
                return r2_ff64(make_float4(xh, yh, zh, 0.f), make_float4(xl, yl, zl, 0.f),
                               sh, sl);
              });
          ff[0] = fmaf(de, dx, ff[0]);
          ff[1] = fmaf(de, dy, ff[1]);
          ff[2] = fmaf(de, dz, ff[2]);
        } else {
          const double dx = xt - sx[k], dy = yt - sy[k], dz = zt - sz[k];
          double dist;
          const double de = law64(p, p.pp[is], dx * dx + dy * dy + dz * dz,
                                  (code >> 16) ? 0.5 : 1.0, e, dist, terr);
          f[0] += de * dx;
          f[1] += de * dy;
          f[2] += de * dz;
        }
      }
      if (FP32) {
        for (int c = 0; c < 3; ++c) f[c] += ff[c];
        for (int c = 0; c < 4; ++c) e[c] += ef[c];
      }
    }
  }
  if (tv)
    for (int c = 0; c < 3; ++c)
      s->fpart[((size_t)blockIdx.y * 3 + c) * kMaxIons + t] = f[c];
  if (terr) atomicOr(&s->err, 2);
  block_sum<4>(e, red, tot);
  if (threadIdx.x == 0)
    for (int c = 0; c < 4; ++c)
      s->epart[((size_t)blockIdx.y * gridDim.x + blockIdx.x) * 4 + c] = tot[c];
}

// Forces: fixed ions get none (energy.mono.f90:181-185); mobile ions sum
// their chunk partials in chunk order.  Energies: fixed-order sum of the
// block slots by block 0.
__global__ void __launch_bounds__(256)
    k_pairs_static_out(int n, int nfix, int nchunk, int nslots, double *fx,
                       double *fy, double *fz, double *e, const StaticScratch *s) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    double f[3] = {0, 0, 0};
    if (i >= nfix)
      for (int c = 0; c < nchunk; ++c)
        for (int k = 0; k < 3; ++k) f[k] += s->fpart[((size_t)c * 3 + k) * kMaxIons + i];
    fx[i] = f[0];
    fy[i] = f[1];
    fz[i] = f[2];
  }
  if (blockIdx.x == 0 && threadIdx.x < 4) {
    double v = 0.0;
    for (int b = 0; b < nslots; ++b) v += s->epart[(size_t)b * 4 + threadIdx.x];
    e[threadIdx.x] = v;
  }
}

// Device address of g_scratch for the current device (looked up once).
int scratch_address(bromoc_ctx *ctx, StaticScratch **out) {
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices)
    return bromoc_ctx_fail(ctx, BROMOC_E_CUDA, "pair_energy_static: no current device");
  std::lock_guard<std::mutex> lock(g_addr_mu);
  if (!g_addr[dev]) {
    void *ptr = nullptr;
    const cudaError_t rc = cudaGetSymbolAddress(&ptr, g_scratch);
    if (rc != cudaSuccess || !ptr) {
      char msg[256];
      snprintf(msg, sizeof msg, "pair_energy_static: cudaGetSymbolAddress: %s",
               cudaGetErrorString(rc));
      return bromoc_ctx_fail(ctx, BROMOC_E_CUDA, msg);
    }
    g_addr[dev] = (StaticScratch *)ptr;
  }
  *out = g_addr[dev];
  return BROMOC_OK;
}

}  // namespace

extern "C" int bromoc_gpu_pair_energy_static(bromoc_ctx *ctx, int32_t n, int32_t nfix,
                                             const double *x, const double *y,
                                             const double *z, const int32_t *typei,
                                             double *fx, double *fy, double *fz,
                                             double *eterms4) {
  const KP *kp = nullptr;
  cudaStream_t stream = nullptr;
  int precision = 0;
  if (!ctx) return BROMOC_E_ARG;
  if (!bromoc_ctx_pair_view(ctx, &kp, &stream, &precision))
    return bromoc_ctx_fail(ctx, BROMOC_E_STATE,
                           "pair_energy_static: set_system, set_types and set_pairs first");
  if (kp->periodic)
    return bromoc_ctx_fail(ctx, BROMOC_E_STATE,
                           "pair_energy_static: the periodic mode is not supported");
  if (!eterms4 || (n > 0 && (!x || !y || !z || !typei || !fx || !fy || !fz)))
    return bromoc_ctx_fail(ctx, BROMOC_E_ARG, "pair_energy_static: null device buffer");
  if (n > kMaxIons)
    return bromoc_ctx_fail(ctx, BROMOC_E_CAPACITY,
                           "pair_energy_static: n exceeds the 4096-ion limit of its "
                           "static scratch; use bromoc_gpu_energy");
  if (n < 0 || nfix < 0 || nfix > n)
    return bromoc_ctx_fail(ctx, BROMOC_E_ARG, "pair_energy_static: bad n or nfix");
  StaticScratch *s = nullptr;
  int rc = scratch_address(ctx, &s);
  if (rc) return rc;
  // source chunks of a multiple of the tile, at most kMaxChunks (none for
  // n == 0, where the output kernel still writes zero energies)
  const int stiles = (n + kTile - 1) / kTile;
  const int per = (stiles + kMaxChunks - 1) / kMaxChunks;
  const int chunk = per * kTile;
  const int nchunk = n > 0 ? (n + chunk - 1) / chunk : 0;
  const int ttiles = (n - nfix + kTile - 1) / kTile;
  if (cudaMemsetAsync(&s->err, 0, sizeof(int), stream) != cudaSuccess)
    return bromoc_ctx_fail(ctx, BROMOC_E_CUDA, "pair_energy_static: clearing the flag");
  int nslots = 0;
  if (ttiles > 0) {
    dim3 g(ttiles, nchunk);
    if (precision == BROMOC_FP32)
      k_pairs_static<true><<<g, kTile, 0, stream>>>(*kp, n, nfix, chunk, x, y, z, typei, s);
    else
      k_pairs_static<false><<<g, kTile, 0, stream>>>(*kp, n, nfix, chunk, x, y, z, typei, s);
    nslots = ttiles * nchunk;
  }
  k_pairs_static_out<<<max(1, (n + 255) / 256), 256, 0, stream>>>(n, nfix, ttiles > 0 ? nchunk : 0,
                                                          nslots, fx, fy, fz, eterms4, s);
  int err = 0;
  if (cudaGetLastError() != cudaSuccess ||
      cudaMemcpyAsync(&err, &s->err, sizeof(int), cudaMemcpyDeviceToHost, stream) !=
          cudaSuccess ||
      cudaStreamSynchronize(stream) != cudaSuccess)
    return bromoc_ctx_fail(ctx, BROMOC_E_CUDA, "pair_energy_static: launch failed");
  if (err & 1)
    return bromoc_ctx_fail(ctx, BROMOC_E_ARG, "pair_energy_static: typei holds a non-ion type");
  if (err & 2)
    return bromoc_ctx_fail(ctx, BROMOC_E_DEVICE, "pair_energy_static: table index out of range");
  return BROMOC_OK;
}
