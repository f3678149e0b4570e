// Adjoint of a Brownian-dynamics segment with respect to the tabulated
// effective-potential tables (scope-table configuration C5).  No reference
// counterpart: the reference fits effective potentials with the IMC
// covariance method (imc-macro.f90) instead of differentiating dynamics.
//
// System: ions only, tabulated (EFPOT) ion-ion laws (polynom.f90:197-230),
// a box with hard walls (fixcoor.f90 clamp), dynamics0 with frozen noise
// (the Philox stream of the forward run).  Positions are float-float records
// as in the FP32 path; pair arithmetic is R = float (forward FP32) or
// R = double (the FP64 reference run of the gradient checks).
//
// Observable: the Gaussian-smoothed pair-distance histogram per ion-type
// pair, H_b = sum over the segment's configurations after each step and over
// pairs of K(r_b - r_ij), K(u) = exp(-u^2 / 2 s^2) / (sqrt(2 pi) s), on bin
// centres r_b = r0 + b dr, accumulated in 64-bit fixed point (deterministic).
// The host forms the loss from H; its derivative S_b = dL/dH_b comes back
// for the backward pass, where a pair at r contributes
// dL/dr = sum_b S_b K(r_b - r) (r_b - r) / s^2.
//
// Backward step t (x_{t+1} = box(x_t + clampbd(c F(x_t)) + s g_t)):
//   mu = boxmask_t (*) a_{t+1};  v = c (*) bdmask_t (*) mu
//   a_t = mu + J(x_t) v + dL/dx_t,   J = dF/dx (symmetric)
//   dL/dtheta += sum_{i<j} (dg_ij/dtheta) d_ij . (v_i - v_j)
// with g = -(dU/dr)/r.  theta = the reference-form table parameters:
// p2, p3 of every piece (dg/dp2 = -1/r, dg/dp3 = -2), the core constant sc0
// (12/r^14) and the tail constant sc2 (6/r^8); the host maps them onto the
// knots through the table builder, which is linear in the knots.
#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/bromoc_gpu.h"
#include "ff.cuh"
#include "launch.h"
#include "physics.cuh"

namespace bgpu {

constexpr int kAdjThreads = 64;     // targets per block == source tile
constexpr int kAdjMaxIonTypes = 4;  // per-thread tail accumulators
constexpr double kHistScale = 68719476736.0;  // 2^36 fixed point

enum AdjMode { kModeForce = 0, kModeBack = 1, kModeHist = 2 };

struct AdjArgs {
  const float4 *h, *l;       // positions (hi + type code, lo) of the configuration
  const void *v;             // backward: c bdmask mu, R[3][n]
  void *out;                 // R[nchunk][3][n]: partial forces / J v + dL/dx
  double *g_ep, *g_sc;       // backward: dL/d(p1,p2,p3) [3 cnt], dL/d(sc) [3 ntc]
  unsigned long long *hist;  // [ntypes2][nbins] fixed-point smoothed histogram
  const double *sbin;        // backward: dL/dH [ntypes2][nbins]
  int n, nchunk, chunk, nbins;
  float r0, dr, sigma;       // bin centres r0 + b dr, kernel width
  float rcut2;               // observable range (last centre + 5 sigma)^2, 0: none
  int theta;                 // backward: accumulate dL/dtheta
};

// local index of the unordered ion-type pair (a <= b), a, b in [0, nt)
__device__ __forceinline__ int tpair(int a, int b, int nt) {
  const int lo = min(a, b), hi = max(a, b);
  return lo * nt - lo * (lo - 1) / 2 + (hi - lo);
}

// g = -(dU/dr)/r, gp = dg/dr of the tabulated law of pair type is at r^2;
// region 0 table piece `piece`, 1 core, 2 tail.
template <typename R>
__device__ __forceinline__ void efp_adj(const KP &p, int is, R x2, R &g, R &gp, R &r,
                                        int &region, int &piece) {
  if constexpr (sizeof(R) == 8) {
    const PairParam &q = p.pp[is];
    r = sqrt(x2);
    const R ir = 1.0 / r, ir2 = ir * ir;
    if (x2 < q.dm2lo) {
      const R i6 = ir2 * ir2 * ir2;
      g = 12.0 * q.sc0 * i6 * i6 * ir2;
      gp = -14.0 * g * ir;
      region = 1;
    } else if (x2 > q.dm2hi) {
      const R i8 = ir2 * ir2 * ir2 * ir2;
      const R f = (q.flags & kChr) ? q.fct * ir2 * ir : 0.0;
      g = 6.0 * q.sc2 * i8 + f;
      gp = (-48.0 * q.sc2 * i8 - 3.0 * f) * ir;
      region = 2;
    } else {
      int i = (int)((r - q.dmi) * p.ires) + q.nxi;
      i = min(max(i, q.nxi), q.nxi + q.npieces - 1);
      const R p2 = p.ep[3 * i + 1], p3 = p.ep[3 * i + 2];
      g = -p2 * ir - 2.0 * p3;
      gp = (-2.0 * p3 - g) * ir;
      region = 0;
      piece = i;
    }
  } else {
    const PairParamF &q = p.ppf[is];
    const R ir = rsqrtf(x2), ir2 = ir * ir;
    r = x2 * ir;
    if (x2 < q.dm2lo) {
      const R i6 = ir2 * ir2 * ir2;
      g = 12.0f * q.sc0 * i6 * i6 * ir2;
      gp = -14.0f * g * ir;
      region = 1;
    } else if (x2 > q.dm2hi) {
      const R i8 = ir2 * ir2 * ir2 * ir2;
      const R f = (q.flags & kChr) ? q.fct * ir2 * ir : 0.0f;
      g = 6.0f * q.sc2 * i8 + f;
      gp = (-48.0f * q.sc2 * i8 - 3.0f * f) * ir;
      region = 2;
    } else {
      const int nxi = q.nxi, last = nxi + (q.flags >> 8) - 1;
      int i = (int)((r - q.dmi) * p.iresf) + nxi;
      i = min(max(i, nxi), last);
      const float4 c = p.ep32[i];
      const R t = r - c.w;
      g = -(c.y + 2.0f * c.z * t) * ir;
      gp = (-2.0f * c.z - g) * ir;
      region = 0;
      piece = i;
    }
  }
}

template <typename R>
__device__ __forceinline__ R to_r(float hi, float lo) {
  if constexpr (sizeof(R) == 8)
    return (double)hi + (double)lo;
  else
    return hi;
}

// Pair kernel of the adjoint engine.  Block (tx, cy): 64 targets x source
// chunk cy, sources staged in shared memory.  Per mode:
//   force: out = sum_j g d_ij                    (forces of the forward step)
//   back:  out = sum_j [g dv + (g'/r) (d.dv) d] + dL/dr d/r   (J v + dL/dx)
//          and dL/dtheta (i < j only), FP64 atomics per piece, per-thread
//          tail sums per source type
//   hist:  cloud-in-cell deposit of r_ij (i < j, r < rcut) into hist
template <typename R, int MODE>
__global__ void __launch_bounds__(kAdjThreads) k_adj_pairs(KP p, AdjArgs a) {
  __shared__ float4 sh[kAdjThreads], sl[kAdjThreads];
  __shared__ R sv[3][kAdjThreads];
  const R *vin = (const R *)a.v;
  const int n = a.n;
  const int t = blockIdx.x * kAdjThreads + threadIdx.x;
  const bool tv = t < n;
  const int s0 = blockIdx.y * a.chunk, s1 = min(n, s0 + a.chunk);
  float4 th = make_float4(0.f, 0.f, 0.f, 0.f), tl = th;
  R tvx = 0, tvy = 0, tvz = 0;
  if (tv) {
    th = a.h[t];
    tl = a.l[t];
    if (MODE == kModeBack) {
      tvx = vin[t];
      tvy = vin[n + t];
      tvz = vin[2 * n + t];
    }
  }
  const int tcode = __float_as_int(th.w) & 0xffff;
  const int ta = tcode - p.ndna;
  const int row = tcode * p.nttyp;
  R ox = 0, oy = 0, oz = 0;
  double tail[kAdjMaxIonTypes] = {0.0, 0.0, 0.0, 0.0};
  for (int base = s0; base < s1; base += kAdjThreads) {
    const int s = base + threadIdx.x;
    __syncthreads();
    if (s < s1) {
      sh[threadIdx.x] = a.h[s];
      sl[threadIdx.x] = a.l[s];
      if (MODE == kModeBack) {
        sv[0][threadIdx.x] = vin[s];
        sv[1][threadIdx.x] = vin[n + s];
        sv[2][threadIdx.x] = vin[2 * n + s];
      }
    }
    __syncthreads();
    const int cnt = min(kAdjThreads, s1 - base);
    R ttail[kAdjMaxIonTypes] = {0, 0, 0, 0};
    if (tv) {
      for (int k = 0; k < cnt; ++k) {
        const int s = base + k;
        if (s == t) continue;
        const float4 h = sh[k], l = sl[k];
        const R dx = (to_r<R>(th.x, tl.x) - to_r<R>(h.x, l.x)) +
                     (sizeof(R) == 8 ? R(0) : R(tl.x - l.x));
        const R dy = (to_r<R>(th.y, tl.y) - to_r<R>(h.y, l.y)) +
                     (sizeof(R) == 8 ? R(0) : R(tl.y - l.y));
        const R dz = (to_r<R>(th.z, tl.z) - to_r<R>(h.z, l.z)) +
                     (sizeof(R) == 8 ? R(0) : R(tl.z - l.z));
        const R x2 = dx * dx + dy * dy + dz * dz;
        const int scode = __float_as_int(h.w) & 0xffff;
        if (MODE == kModeHist) {
          if (t < s && x2 < (R)a.rcut2) {
            const R r = sqrt(x2);
            const int tp = tpair(ta, scode - p.ndna, p.nion_t);
            unsigned long long *hb = a.hist + (size_t)tp * a.nbins;
            const R sg = (R)a.sigma, ia = (R)(0.3989422804014327 / a.sigma);
            const int b0 = max(0, (int)ceil((r - 5 * sg - (R)a.r0) / (R)a.dr));
            const int b1 = min(a.nbins - 1, (int)floor((r + 5 * sg - (R)a.r0) / (R)a.dr));
            for (int b = b0; b <= b1; ++b) {
              const R u = ((R)a.r0 + b * (R)a.dr - r) / sg;
              const R k = ia * exp(-(R)0.5 * u * u);
              unsigned long long q;
              if constexpr (sizeof(R) == 8)
                q = (unsigned long long)(k * kHistScale + 0.5);
              else  // FP32 run: the fixed-point value formed on the FP32 pipe
                q = __float2ull_rn(k * (float)kHistScale);
              atomicAdd(hb + b, q);
            }
          }
          continue;
        }
        const int is = p.pidx[row + scode];
        R g, gp, r;
        int region, piece = 0;
        efp_adj<R>(p, is, x2, g, gp, r, region, piece);
        if (MODE == kModeForce) {
          ox += g * dx;
          oy += g * dy;
          oz += g * dz;
          continue;
        }
        // backward: J v, dL/dtheta, dL/dx of the observable
        const R vx = tvx - sv[0][k], vy = tvy - sv[1][k], vz = tvz - sv[2][k];
        const R q = dx * vx + dy * vy + dz * vz;
        const R ir = (R)1 / r;
        const R c = gp * ir * q;
        ox += g * vx + c * dx;
        oy += g * vy + c * dy;
        oz += g * vz + c * dz;
        if (a.theta && t < s) {
          if (region == 0) {
            atomicAdd(a.g_ep + 3 * piece + 1, (double)(-q * ir));
            atomicAdd(a.g_ep + 3 * piece + 2, (double)(-2 * q));
          } else if (region == 1) {
            const R ir2 = ir * ir, i6 = ir2 * ir2 * ir2;
            atomicAdd(a.g_sc + 3 * is, (double)(12 * i6 * i6 * ir2 * q));
          } else {
            const R ir2 = ir * ir;
            const int tb = scode - p.ndna;
            if (tb < kAdjMaxIonTypes) ttail[tb] += 6 * ir2 * ir2 * ir2 * ir2 * q;
          }
        }
        if (x2 < (R)a.rcut2) {  // observable: dL/dr d / r
          const int tp = tpair(ta, scode - p.ndna, p.nion_t);
          const double *sb = a.sbin + (size_t)tp * a.nbins;
          const R sg = (R)a.sigma, ia = (R)(0.3989422804014327 / a.sigma);
          const int b0 = max(0, (int)ceil((r - 5 * sg - (R)a.r0) / (R)a.dr));
          const int b1 = min(a.nbins - 1, (int)floor((r + 5 * sg - (R)a.r0) / (R)a.dr));
          R dldr = 0;
          for (int b = b0; b <= b1; ++b) {
            const R u = ((R)a.r0 + b * (R)a.dr - r) / sg;
            dldr += (R)sb[b] * ia * exp(-(R)0.5 * u * u) * u / sg;
          }
          ox += dldr * dx * ir;
          oy += dldr * dy * ir;
          oz += dldr * dz * ir;
        }
      }
    }
    if (MODE == kModeBack)
      for (int m = 0; m < kAdjMaxIonTypes; ++m) tail[m] += (double)ttail[m];
  }
  if (MODE == kModeBack && tv) {
    for (int m = 0; m < kAdjMaxIonTypes && m < p.nion_t; ++m)
      if (tail[m] != 0.0) {
        const int is = p.pidx[row + p.ndna + m];
        atomicAdd(a.g_sc + 3 * is + 2, tail[m]);
      }
  }
  if (MODE != kModeHist && tv) {
    R *o = (R *)a.out + (size_t)blockIdx.y * 3 * n;
    o[t] = ox;
    o[n + t] = oy;
    o[2 * n + t] = oz;
  }
}

// Forward step: forces from the chunk partials (fixed order), the BD move
// of dynamics0 with frozen noise, the box clamp, and the clamp masks of the
// step (bit k: bdmax clamp of component k; bit 3 + k: wall clamp).
template <typename R>
__global__ void k_adj_move(KP p, const float4 *h, const float4 *l, const R *part, int nchunk,
                           int n, float4 *hn, float4 *ln, uint8_t *mask, BoxF box,
                           uint64_t seed, uint64_t step) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  R F[3];
  for (int k = 0; k < 3; ++k) {
    R v = 0;
    for (int c = 0; c < nchunk; ++c) v += part[((size_t)c * 3 + k) * n + i];
    F[k] = v;
  }
  const int it = abs(p.typei[i]);
  R fact1, fact2;
  if constexpr (sizeof(R) == 8) {
    fact1 = p.fact1a[it];
    fact2 = p.fact2a[it];
  } else {
    fact1 = p.fact_f[it].x;
    fact2 = p.fact_f[it].y;
  }
  float g[3];
  bd_noise3_f(seed, step, (uint32_t)i, g);
  float4 h4 = h[i], l4 = l[i];
  float hh[3] = {h4.x, h4.y, h4.z}, ll[3] = {l4.x, l4.y, l4.z};
  int m = 0;
  const R bdmax = sizeof(R) == 8 ? (R)p.bdmax : (R)p.f.bdmax;
  for (int k = 0; k < 3; ++k) {
    R d = F[k] * fact1;
    if (fabs(d) > bdmax) {
      d = copysign(bdmax, d);
      m |= 1 << k;
    }
    const R disp = d + fact2 * (R)g[k];
    if constexpr (sizeof(R) == 8) {
      double x = (double)hh[k] + (double)ll[k] + disp;
      const double lo = k == 0 ? p.lx2m : (k == 1 ? p.ly2m : p.lz2m);
      const double hi = k == 0 ? p.lx2p : (k == 1 ? p.ly2p : p.lz2p);
      if (x < lo) {
        x = lo;
        m |= 8 << k;
      } else if (x > hi) {
        x = hi;
        m |= 8 << k;
      }
      hh[k] = (float)x;
      ll[k] = (float)(x - (double)hh[k]);
    } else {
      ff_add(hh[k], ll[k], (float)disp);
      if (ff_diff(hh[k], ll[k], box.bh[2 * k], box.bl[2 * k]) < 0.0f) {
        hh[k] = box.bh[2 * k];
        ll[k] = box.bl[2 * k];
        m |= 8 << k;
      } else if (ff_diff(hh[k], ll[k], box.bh[2 * k + 1], box.bl[2 * k + 1]) > 0.0f) {
        hh[k] = box.bh[2 * k + 1];
        ll[k] = box.bl[2 * k + 1];
        m |= 8 << k;
      }
    }
  }
  hn[i] = make_float4(hh[0], hh[1], hh[2], h4.w);
  ln[i] = make_float4(ll[0], ll[1], ll[2], 0.0f);
  if (mask) mask[i] = (uint8_t)m;
}

// Backward, before the pair sweep: mu = wallmask (*) a, v = c bdmask (*) mu.
template <typename R>
__global__ void k_adj_prep(KP p, const R *a, const uint8_t *mask, int n, R *mu, R *v) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int it = abs(p.typei[i]);
  R c;
  if constexpr (sizeof(R) == 8)
    c = p.fact1a[it];
  else
    c = p.fact_f[it].x;
  const int m = mask ? mask[i] : 0;
  for (int k = 0; k < 3; ++k) {
    const R u = (m & (8 << k)) ? (R)0 : a[(size_t)k * n + i];
    mu[(size_t)k * n + i] = u;
    v[(size_t)k * n + i] = (m & (1 << k)) ? (R)0 : c * u;
  }
}

// Backward, after the pair sweep: a = mu + sum of the chunk partials.
template <typename R>
__global__ void k_adj_combine(const R *mu, const R *part, int nchunk, int n, R *a) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  for (int k = 0; k < 3; ++k) {
    R v = mu ? mu[(size_t)k * n + i] : (R)0;
    for (int c = 0; c < nchunk; ++c) v += part[((size_t)c * 3 + k) * n + i];
    a[(size_t)k * n + i] = v;
  }
}

}  // namespace bgpu

using namespace bgpu;

struct bromoc_adj {
  bromoc_ctx *proto = nullptr;
  cudaStream_t stream = nullptr;
  int orphaned = 0;  // set when the prototype context is destroyed first
  int precision = BROMOC_FP32;
  std::string err;
  int cap = 0, n = 0, nt = 0, ntp = 0;
  int nchunk = 1, chunk = 64;
  int *typei = nullptr;
  float4 *x0h = nullptr, *x0l = nullptr;    // initial configuration
  float4 *xfh = nullptr, *xfl = nullptr;    // final configuration of the forward run
  std::vector<float4 *> ckh, ckl;           // checkpoints
  std::vector<float4 *> trh, trl;           // one recomputed segment, ckpt + 1 slots
  uint8_t *mask = nullptr;                  // [ckpt][cap]
  void *part = nullptr, *a = nullptr, *mu = nullptr, *v = nullptr;
  unsigned long long *hist = nullptr;
  double *sbin = nullptr, *g_ep = nullptr, *g_sc = nullptr;
  int nbins = 0;
  double r0 = 0.0, dr = 0.0, sigma = 0.0;
  // the last forward run
  int nsteps = 0, ckpt = 0;
  uint64_t seed = 0, step0 = 0;
  bool have_forward = false;
  std::vector<void *> allocs;
};

namespace {

int aset(bromoc_adj *a, int code, const char *fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  if (a) a->err = buf;
  return code;
}

#define ACU(call)                                                              \
  do {                                                                         \
    cudaError_t e_ = (call);                                                   \
    if (e_ != cudaSuccess)                                                     \
      return aset(ad, BROMOC_E_CUDA, "%s: %s", #call, cudaGetErrorString(e_)); \
  } while (0)

template <class T>
int aalloc(bromoc_adj *ad, T **p, size_t count) {
  *p = nullptr;
  cudaError_t e = cudaMalloc((void **)p, std::max<size_t>(count, 1) * sizeof(T));
  if (e != cudaSuccess)
    return aset(ad, BROMOC_E_NOMEM, "cudaMalloc(%zu bytes): %s", count * sizeof(T),
                cudaGetErrorString(e));
  ad->allocs.push_back((void *)*p);
  return BROMOC_OK;
}

// the prototype's current parameter block with the adjoint's particle types
int view(bromoc_adj *ad, KP &p) {
  const KP *pk = nullptr;
  cudaStream_t s = nullptr;
  int prec = 0;
  if (!bromoc_ctx_pair_view(ad->proto, &pk, &s, &prec))
    return aset(ad, BROMOC_E_STATE, "adjoint: the prototype has no system/types/pairs");
  p = *pk;
  p.typei = ad->typei;
  return BROMOC_OK;
}

template <typename R>
void run_pairs(bromoc_adj *ad, const KP &p, int mode, const float4 *h, const float4 *l,
               const void *v, bool obs, bool theta) {
  AdjArgs a{};
  a.h = h;
  a.l = l;
  a.v = v;
  a.out = ad->part;
  a.g_ep = ad->g_ep;
  a.g_sc = ad->g_sc;
  a.hist = ad->hist;
  a.sbin = ad->sbin;
  a.n = ad->n;
  a.nchunk = ad->nchunk;
  a.chunk = ad->chunk;
  a.nbins = ad->nbins;
  a.r0 = (float)ad->r0;
  a.dr = (float)ad->dr;
  a.sigma = (float)ad->sigma;
  const double rc = ad->r0 + ad->dr * (ad->nbins - 1) + 5.0 * ad->sigma;
  a.rcut2 = obs ? (float)(rc * rc) : 0.0f;
  a.theta = theta ? 1 : 0;
  const dim3 g((ad->n + kAdjThreads - 1) / kAdjThreads, ad->nchunk);
  if (mode == kModeForce)
    k_adj_pairs<R, kModeForce><<<g, kAdjThreads, 0, ad->stream>>>(p, a);
  else if (mode == kModeBack)
    k_adj_pairs<R, kModeBack><<<g, kAdjThreads, 0, ad->stream>>>(p, a);
  else
    k_adj_pairs<R, kModeHist><<<g, kAdjThreads, 0, ad->stream>>>(p, a);
}

template <typename R>
void step_forward(bromoc_adj *ad, const KP &p, const float4 *h, const float4 *l, float4 *hn,
                  float4 *ln, uint8_t *mask, uint64_t step) {
  run_pairs<R>(ad, p, kModeForce, h, l, nullptr, false, false);
  k_adj_move<R><<<(ad->n + 127) / 128, 128, 0, ad->stream>>>(
      p, h, l, (const R *)ad->part, ad->nchunk, ad->n, hn, ln, mask, p.f.box, ad->seed, step);
}

template <typename R>
int forward_impl(bromoc_adj *ad, const KP &p, double *hist_out) {
  const size_t n = ad->n;
  ACU(cudaMemsetAsync(ad->hist, 0, (size_t)ad->ntp * ad->nbins * sizeof(unsigned long long),
                      ad->stream));
  ACU(cudaMemcpyAsync(ad->ckh[0], ad->x0h, n * sizeof(float4), cudaMemcpyDeviceToDevice,
                      ad->stream));
  ACU(cudaMemcpyAsync(ad->ckl[0], ad->x0l, n * sizeof(float4), cudaMemcpyDeviceToDevice,
                      ad->stream));
  const float4 *h = ad->x0h, *l = ad->x0l;
  for (int t = 0; t < ad->nsteps; ++t) {
    float4 *hn = ad->trh[(t + 1) & 1], *ln = ad->trl[(t + 1) & 1];
    step_forward<R>(ad, p, h, l, hn, ln, nullptr, ad->step0 + t);
    run_pairs<R>(ad, p, kModeHist, hn, ln, nullptr, true, false);  // RDF of x_{t+1}
    if ((t + 1) % ad->ckpt == 0 && t + 1 < ad->nsteps) {
      const int c = (t + 1) / ad->ckpt;
      ACU(cudaMemcpyAsync(ad->ckh[c], hn, n * sizeof(float4), cudaMemcpyDeviceToDevice,
                          ad->stream));
      ACU(cudaMemcpyAsync(ad->ckl[c], ln, n * sizeof(float4), cudaMemcpyDeviceToDevice,
                          ad->stream));
    }
    h = hn;
    l = ln;
  }
  ACU(cudaMemcpyAsync(ad->xfh, h, n * sizeof(float4), cudaMemcpyDeviceToDevice, ad->stream));
  ACU(cudaMemcpyAsync(ad->xfl, l, n * sizeof(float4), cudaMemcpyDeviceToDevice, ad->stream));
  std::vector<unsigned long long> hh((size_t)ad->ntp * ad->nbins);
  ACU(cudaMemcpyAsync(hh.data(), ad->hist, hh.size() * sizeof(unsigned long long),
                      cudaMemcpyDeviceToHost, ad->stream));
  ACU(cudaStreamSynchronize(ad->stream));
  ACU(cudaGetLastError());
  for (size_t k = 0; k < hh.size(); ++k) hist_out[k] = (double)hh[k] / kHistScale;
  return BROMOC_OK;
}

template <typename R>
int backward_impl(bromoc_adj *ad, const KP &p) {
  const int n = ad->n, nb = (n + 127) / 128;
  const int T = ad->nsteps, K = ad->ckpt;
  // a = dL/dx_T (observable of the last configuration only)
  ACU(cudaMemsetAsync(ad->v, 0, 3 * (size_t)n * sizeof(R), ad->stream));
  run_pairs<R>(ad, p, kModeBack, ad->xfh, ad->xfl, ad->v, true, false);
  k_adj_combine<R><<<nb, 128, 0, ad->stream>>>(nullptr, (const R *)ad->part, ad->nchunk, n,
                                               (R *)ad->a);
  const int nseg = (T + K - 1) / K;
  for (int seg = nseg - 1; seg >= 0; --seg) {
    const int t0 = seg * K, t1 = std::min(T, t0 + K);
    ACU(cudaMemcpyAsync(ad->trh[0], ad->ckh[seg], n * sizeof(float4), cudaMemcpyDeviceToDevice,
                        ad->stream));
    ACU(cudaMemcpyAsync(ad->trl[0], ad->ckl[seg], n * sizeof(float4), cudaMemcpyDeviceToDevice,
                        ad->stream));
    for (int t = t0; t < t1; ++t) {  // recompute the segment, keeping x_t and masks
      const int k = t - t0;
      step_forward<R>(ad, p, ad->trh[k], ad->trl[k], ad->trh[k + 1], ad->trl[k + 1],
                      ad->mask + (size_t)k * ad->cap, ad->step0 + t);
    }
    for (int t = t1 - 1; t >= t0; --t) {
      const int k = t - t0;
      k_adj_prep<R><<<nb, 128, 0, ad->stream>>>(p, (const R *)ad->a,
                                                ad->mask + (size_t)k * ad->cap, n,
                                                (R *)ad->mu, (R *)ad->v);
      run_pairs<R>(ad, p, kModeBack, ad->trh[k], ad->trl[k], ad->v, t >= 1, true);
      k_adj_combine<R><<<nb, 128, 0, ad->stream>>>((const R *)ad->mu, (const R *)ad->part,
                                                   ad->nchunk, n, (R *)ad->a);
    }
  }
  ACU(cudaGetLastError());
  return BROMOC_OK;
}

}  // namespace

extern "C" {

int bromoc_adj_create(bromoc_ctx *proto, int32_t capacity, int32_t precision,
                      bromoc_adj **out) {
  if (!proto || !out || capacity < 2 ||
      (precision != BROMOC_FP32 && precision != BROMOC_FP64))
    return BROMOC_E_ARG;
  *out = nullptr;
  const KP *pk = nullptr;
  cudaStream_t s = nullptr;
  int prec = 0;
  if (!bromoc_ctx_pair_view(proto, &pk, &s, &prec))
    return bromoc_ctx_fail(proto, BROMOC_E_STATE, "adjoint: set_system/types/pairs first");
  // the FP32 constants (box, fact_f) and scratch of the prototype
  const KP *pk32 = nullptr;
  if (prec == BROMOC_FP32) {
    int rc = bromoc_ctx_prepare_f32(proto, &pk32, &s);
    if (rc) return rc;
  } else if (precision == BROMOC_FP32) {
    return bromoc_ctx_fail(proto, BROMOC_E_STATE,
                           "adjoint: FP32 arithmetic needs an FP32 prototype");
  }
  if (pk->periodic)
    return bromoc_ctx_fail(proto, BROMOC_E_STATE, "adjoint: the periodic mode is not supported");
  if (pk->nsites != 0 || pk->shape != BROMOC_BOX)
    return bromoc_ctx_fail(proto, BROMOC_E_STATE, "adjoint: ions only, in a box");
  if (pk->mm.on)
    return bromoc_ctx_fail(proto, BROMOC_E_STATE, "adjoint: the MMIJ reaction field is not supported");
  if (pk->nion_t > kAdjMaxIonTypes)
    return bromoc_ctx_fail(proto, BROMOC_E_STATE, "adjoint: at most 4 ion types");
  bromoc_adj *ad = new bromoc_adj;
  ad->proto = proto;
  ad->stream = s;
  bromoc_ctx_attach(proto, &ad->orphaned);
  ad->precision = precision;
  ad->cap = capacity;
  ad->nt = pk->nion_t;
  ad->ntp = ad->nt * (ad->nt + 1) / 2;
  const size_t cap = capacity, rs = precision == BROMOC_FP64 ? 8 : 4;
  int rc = aalloc(ad, &ad->typei, cap);
  if (!rc) rc = aalloc(ad, &ad->x0h, cap);
  if (!rc) rc = aalloc(ad, &ad->x0l, cap);
  if (!rc) rc = aalloc(ad, &ad->xfh, cap);
  if (!rc) rc = aalloc(ad, &ad->xfl, cap);
  char *buf = nullptr;
  if (!rc) rc = aalloc(ad, &buf, rs * 3 * cap * 35);  // part (32 chunks) + a, mu, v
  if (!rc) {
    ad->part = buf;
    ad->a = buf + rs * 3 * cap * 32;
    ad->mu = buf + rs * 3 * cap * 33;
    ad->v = buf + rs * 3 * cap * 34;
  }
  if (!rc) rc = aalloc(ad, &ad->g_ep, 3 * (size_t)std::max(pk->cnt, 1));
  if (!rc) rc = aalloc(ad, &ad->g_sc, 3 * (size_t)pk->ntc);
  if (rc) {
    const std::string msg = ad->err;
    bromoc_adj_destroy(ad);
    return bromoc_ctx_fail(proto, rc, msg.c_str());
  }
  *out = ad;
  return BROMOC_OK;
}

int bromoc_adj_destroy(bromoc_adj *ad) {
  if (!ad) return BROMOC_E_ARG;
  if (!ad->orphaned) {
    if (ad->stream) cudaStreamSynchronize(ad->stream);
    bromoc_ctx_detach(ad->proto, &ad->orphaned);
  }
  for (void *p : ad->allocs) cudaFree(p);
  delete ad;
  cudaGetLastError();  // leave no non-sticky error behind for the next call
  return BROMOC_OK;
}

const char *bromoc_adj_last_error(const bromoc_adj *ad) {
  return ad ? ad->err.c_str() : "null adjoint";
}

}  // extern "C"

extern "C" {

int bromoc_adj_set_particles(bromoc_adj *ad, int32_t n, const double *x, const double *y,
                             const double *z, const int32_t *typei) {
  if (ad && ad->orphaned) return aset(ad, BROMOC_E_STATE, "the prototype context was destroyed");
  if (!ad || !x || !y || !z || !typei) return aset(ad, BROMOC_E_ARG, "set_particles: null");
  if (n < 2 || n > ad->cap)
    return aset(ad, BROMOC_E_CAPACITY, "set_particles: n = %d outside [2, %d]", n, ad->cap);
  KP p;
  int rc = view(ad, p);
  if (rc) return rc;
  std::vector<int> nw(p.ntype + 1);
  ACU(cudaMemcpy(nw.data(), p.nwtype, (p.ntype + 1) * sizeof(int), cudaMemcpyDeviceToHost));
  std::vector<float4> h(n), l(n);
  for (int i = 0; i < n; ++i) {
    const int t = typei[i] < 0 ? -typei[i] : typei[i];
    if (t <= p.nold || t > p.ntype)
      return aset(ad, BROMOC_E_ARG, "set_particles: typei(%d) = %d is not an ion type", i + 1,
                  typei[i]);
    const double v[3] = {x[i], y[i], z[i]};
    float hi[3], lo[3];
    for (int k = 0; k < 3; ++k) {
      hi[k] = (float)v[k];
      lo[k] = (float)(v[k] - (double)hi[k]);
    }
    const int code = (nw[t] - 1) | (1 << 16);
    float fc;
    std::memcpy(&fc, &code, sizeof fc);
    h[i] = make_float4(hi[0], hi[1], hi[2], fc);
    l[i] = make_float4(lo[0], lo[1], lo[2], 0.0f);
  }
  ACU(cudaStreamSynchronize(ad->stream));
  ACU(cudaMemcpy(ad->x0h, h.data(), n * sizeof(float4), cudaMemcpyHostToDevice));
  ACU(cudaMemcpy(ad->x0l, l.data(), n * sizeof(float4), cudaMemcpyHostToDevice));
  ACU(cudaMemcpy(ad->typei, typei, n * sizeof(int), cudaMemcpyHostToDevice));
  ad->n = n;
  // source chunks: ~8 blocks per SM, at most 32
  const int tiles = (n + kAdjThreads - 1) / kAdjThreads;
  int want = std::max(1, std::min(32, (8 * 152 + tiles - 1) / tiles));
  want = std::min(want, tiles);
  ad->chunk = (tiles + want - 1) / want * kAdjThreads;
  ad->nchunk = (n + ad->chunk - 1) / ad->chunk;
  ad->have_forward = false;
  return BROMOC_OK;
}

int bromoc_adj_forward(bromoc_adj *ad, int32_t nsteps, int32_t ckpt, uint64_t seed,
                       uint64_t step0, int32_t nbins, double r0, double dr, double sigma,
                       double *hist) {
  if (ad && ad->orphaned) return aset(ad, BROMOC_E_STATE, "the prototype context was destroyed");
  if (!ad || !hist || nsteps < 1 || ckpt < 1 || nbins < 1 || !(dr > 0.0) || !(sigma > 0.0) ||
      r0 < 0.0)
    return aset(ad, BROMOC_E_ARG, "forward: bad arguments");
  if (ad->n < 2) return aset(ad, BROMOC_E_STATE, "forward: set_particles first");
  KP p;
  int rc = view(ad, p);
  if (rc) return rc;
  {  // every ion-ion law must be tabulated
    std::vector<PairParamF> pf(p.ntc);
    ACU(cudaMemcpy(pf.data(), p.ppf, p.ntc * sizeof(PairParamF), cudaMemcpyDeviceToHost));
    std::vector<int> pidx((size_t)p.nttyp * p.nttyp);
    ACU(cudaMemcpy(pidx.data(), p.pidx, pidx.size() * sizeof(int), cudaMemcpyDeviceToHost));
    for (int a = p.ndna; a < p.nttyp; ++a)
      for (int b = p.ndna; b < p.nttyp; ++b) {
        const int is = pidx[(size_t)a * p.nttyp + b];
        if (is < 0 || !(pf[is].flags & kEfp))
          return aset(ad, BROMOC_E_STATE, "forward: every ion-ion law must be EFPOT");
      }
  }
  // buffers of this run (grow-only)
  const int nck = (nsteps + ckpt - 1) / ckpt;
  const int nslot = std::max(2, ckpt + 1);
  const size_t cap = ad->cap;
  while ((int)ad->ckh.size() < nck) {
    float4 *a = nullptr, *b = nullptr;
    if ((rc = aalloc(ad, &a, cap)) || (rc = aalloc(ad, &b, cap))) return rc;
    ad->ckh.push_back(a);
    ad->ckl.push_back(b);
  }
  while ((int)ad->trh.size() < nslot) {
    float4 *a = nullptr, *b = nullptr;
    if ((rc = aalloc(ad, &a, cap)) || (rc = aalloc(ad, &b, cap))) return rc;
    ad->trh.push_back(a);
    ad->trl.push_back(b);
  }
  if (ckpt > ad->ckpt || !ad->mask) {
    if ((rc = aalloc(ad, &ad->mask, (size_t)ckpt * cap))) return rc;
  }
  if (nbins != ad->nbins || !ad->hist) {
    if ((rc = aalloc(ad, &ad->hist, (size_t)ad->ntp * nbins))) return rc;
    if ((rc = aalloc(ad, &ad->sbin, (size_t)ad->ntp * nbins))) return rc;
  }
  ad->nbins = nbins;
  ad->r0 = r0;
  ad->dr = dr;
  ad->sigma = sigma;
  ad->nsteps = nsteps;
  ad->ckpt = ckpt;
  ad->seed = seed;
  ad->step0 = step0;
  rc = ad->precision == BROMOC_FP64 ? forward_impl<double>(ad, p, hist)
                                    : forward_impl<float>(ad, p, hist);
  ad->have_forward = rc == BROMOC_OK;
  return rc;
}

int bromoc_adj_backward(bromoc_adj *ad, const double *dl_dhist, double *g_ep, double *g_sc) {
  if (ad && ad->orphaned) return aset(ad, BROMOC_E_STATE, "the prototype context was destroyed");
  if (!ad || !dl_dhist || !g_ep || !g_sc) return aset(ad, BROMOC_E_ARG, "backward: null");
  if (!ad->have_forward) return aset(ad, BROMOC_E_STATE, "backward: run forward first");
  KP p;
  int rc = view(ad, p);
  if (rc) return rc;
  ACU(cudaMemcpyAsync(ad->sbin, dl_dhist, (size_t)ad->ntp * ad->nbins * sizeof(double),
                      cudaMemcpyHostToDevice, ad->stream));
  const size_t nep = 3 * (size_t)std::max(p.cnt, 1), nsc = 3 * (size_t)p.ntc;
  ACU(cudaMemsetAsync(ad->g_ep, 0, nep * sizeof(double), ad->stream));
  ACU(cudaMemsetAsync(ad->g_sc, 0, nsc * sizeof(double), ad->stream));
  rc = ad->precision == BROMOC_FP64 ? backward_impl<double>(ad, p) : backward_impl<float>(ad, p);
  if (rc) return rc;
  ACU(cudaMemcpyAsync(g_ep, ad->g_ep, nep * sizeof(double), cudaMemcpyDeviceToHost, ad->stream));
  ACU(cudaMemcpyAsync(g_sc, ad->g_sc, nsc * sizeof(double), cudaMemcpyDeviceToHost, ad->stream));
  ACU(cudaStreamSynchronize(ad->stream));
  return BROMOC_OK;
}

// which = 0: the initial configuration, 1: the last forward run's final one
int bromoc_adj_get_particles(bromoc_adj *ad, int32_t which, double *x, double *y, double *z) {
  if (ad && ad->orphaned) return aset(ad, BROMOC_E_STATE, "the prototype context was destroyed");
  if (!ad || !x || !y || !z) return aset(ad, BROMOC_E_ARG, "get_particles: null");
  const int n = ad->n;
  std::vector<float4> h(n), l(n);
  ACU(cudaStreamSynchronize(ad->stream));
  ACU(cudaMemcpy(h.data(), which ? ad->xfh : ad->x0h, n * sizeof(float4),
                 cudaMemcpyDeviceToHost));
  ACU(cudaMemcpy(l.data(), which ? ad->xfl : ad->x0l, n * sizeof(float4),
                 cudaMemcpyDeviceToHost));
  for (int i = 0; i < n; ++i) {
    x[i] = (double)h[i].x + (double)l[i].x;
    y[i] = (double)h[i].y + (double)l[i].y;
    z[i] = (double)h[i].z + (double)l[i].z;
  }
  return BROMOC_OK;
}

}  // extern "C"
