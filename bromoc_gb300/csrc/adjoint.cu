// Adjoint of a Brownian-dynamics segment with respect to the tabulated
// effective-potential tables.  No reference counterpart: the reference fits
// effective potentials with the IMC covariance method (imc-macro.f90)
// instead of differentiating dynamics.
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

constexpr int kAdjTileWarps = 4;    // tile pairs (warps) per block of the pair sweep
constexpr int kAdjMaxIonTypes = 4;  // per-lane tail accumulators
constexpr int kAdjTypePairs = kAdjMaxIonTypes * kAdjMaxIonTypes;
constexpr double kHistScale = 68719476736.0;  // 2^36 fixed point

enum AdjMode { kModeForce = 0, kModeBack = 1, kModeHist = 2 };

struct AdjArgs {
  const float4 *h, *l;       // positions (hi + type code, lo) of the configuration
  const void *v;             // backward: c bdmask mu, R[3][n]
  void *out;                 // R[tile pair][side][3][32]: partial forces / J v + dL/dx
  void *tail;                // backward: R[kAdjTypePairs][tile pair] tail sums
  double *g_ep, *g_sc;       // backward: dL/d(p1,p2,p3) [3 cnt], dL/d(sc) [3 ntc]
  unsigned long long *hist;  // [ntypes2][nbins] fixed-point smoothed histogram
  const double *sbin;        // backward: dL/dH [ntypes2][nbins]
  int n, nbins;
  int deposit;               // force: also the histogram deposit of the configuration
  float r0, dr, sigma;       // bin centres r0 + b dr, kernel width
  double ia;                 // 1 / (sqrt(2 pi) sigma), sigma as the float above
  float rcut2;               // observable range (last centre + 5 sigma)^2, 0: none
  int theta;                 // backward: accumulate dL/dtheta
};

// local index of the unordered ion-type pair (a <= b), a, b in [0, nt)
__device__ __forceinline__ int tpair(int a, int b, int nt) {
  const int lo = min(a, b), hi = max(a, b);
  return lo * nt - lo * (lo - 1) / 2 + (hi - lo);
}

// r, 1/r and 1/r^2 from r^2 as the adjoint's laws take them: FP64 through
// the square root, FP32 through the reciprocal square root.
template <typename R>
__device__ __forceinline__ void efp_r(R x2, R &r, R &ir, R &ir2) {
  if constexpr (sizeof(R) == 8) {
    r = sqrt(x2);
    ir = 1.0 / r;
  } else {
    ir = rsqrtf(x2);
    r = x2 * ir;
  }
  ir2 = ir * ir;
}

// The analytic tail of a tabulated law (r^2 above the table): g, g' from
// sc2 / r^6 and, with a charge term, fct / r (fct zero without one).
template <typename R>
__device__ __forceinline__ void efp_tail(R sc2, R fct, R ir, R ir2, R &g, R &gp) {
  const R i8 = ir2 * ir2 * ir2 * ir2;
  const R f = fct * ir2 * ir;
  g = (R)6 * sc2 * i8 + f;
  gp = ((R)-48 * sc2 * i8 - (R)3 * f) * ir;
}

// g = -(dU/dr)/r, gp = dg/dr of the tabulated law of pair type is at r^2;
// region 0 table piece `piece`, 1 core, 2 tail.
template <typename R>
__device__ __forceinline__ void efp_adj(const KP &p, int is, R x2, R &g, R &gp, R &r,
                                        int &region, int &piece) {
  R ir, ir2;
  efp_r<R>(x2, r, ir, ir2);
  if constexpr (sizeof(R) == 8) {
    const PairParam &q = p.pp[is];
    if (x2 < q.dm2lo) {
      const R i6 = ir2 * ir2 * ir2;
      g = 12.0 * q.sc0 * i6 * i6 * ir2;
      gp = -14.0 * g * ir;
      region = 1;
    } else if (x2 > q.dm2hi) {
      efp_tail<R>(q.sc2, (q.flags & kChr) ? q.fct : 0.0, ir, ir2, g, gp);
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
    if (x2 < q.dm2lo) {
      const R i6 = ir2 * ir2 * ir2;
      g = 12.0f * q.sc0 * i6 * i6 * ir2;
      gp = -14.0f * g * ir;
      region = 1;
    } else if (x2 > q.dm2hi) {
      efp_tail<R>(q.sc2, (q.flags & kChr) ? q.fct : 0.0f, ir, ir2, g, gp);
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

// Pair sweep of the adjoint engine on Newton-3 tile pairs: each unordered
// pair once.  One warp per tile pair (I, J), I <= J (row-major, n3_pair);
// lane l holds row ion I*32 + l, the column tile's records, v (backward) and
// sums sit in the warp's shared memory and are visited in the rotating order
// m = (l + k) mod 32, so the lanes of one step touch distinct entries
// (k = 0..31 off the diagonal; on it k = 1..16, the last step by lanes
// 0..15).  Every per-pair term is odd in the separation d (and in dv): the
// row ion gets it, the column entry its negative.  Per mode:
//   force: g d; with deposit, also the smoothed-histogram deposit
//   back:  g dv + (g'/r) (d.dv) d + dL/dr d/r   (J v + dL/dx), and with
//          theta dL/dtheta: table pieces and core constants by FP64 atomics,
//          tail constants per (row type, column type) summed over the warp
//          into tail[type pair][tile pair] (reduced in fixed order by
//          k_adj_tails)
//   hist:  the deposit alone
// Most pairs of a segment lie beyond the table, on the analytic tail, and
// outside the histogram's range: the loop evaluates those itself and queues
// the rest (table and core pairs, pairs the histogram sees) per warp; the
// queue is evaluated 32 pairs at a time, one a lane, and the terms added in
// queue order (deterministic).
// Output: out[tile pair][side][3][32] (side 0 the row ions, 1 the column
// entries), gathered per particle in fixed order (adj_gather).
constexpr int kAdjQ = 64;  // queue: room for two steps
template <typename R>
struct AdjWarp {
  float4 h[32], l[32];
  R v[3][32];
  R s[3][32];
  int q[kAdjQ];  // row lane | column entry << 5
};
// the analytic tail of one (row type, column type) law: x2 > dm2hi
template <typename R>
struct AdjTail {
  R dm2hi, sc2, fct;
};

template <typename R>
__device__ __forceinline__ void adj_deposit(const KP &p, const AdjArgs &a, int ta, int scode,
                                            R r) {
  const int tp = tpair(ta, scode - p.ndna, p.nion_t);
  unsigned long long *hb = a.hist + (size_t)tp * a.nbins;
  const R sg = (R)a.sigma, ia = (R)a.ia;
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

// dL/dr of the observable at r for the type pair of (ta, scode)
template <typename R>
__device__ __forceinline__ R adj_dldr(const KP &p, const AdjArgs &a, int ta, int scode, R r) {
  const int tp = tpair(ta, scode - p.ndna, p.nion_t);
  const double *sb = a.sbin + (size_t)tp * a.nbins;
  const R sg = (R)a.sigma, ia = (R)a.ia;
  const int b0 = max(0, (int)ceil((r - 5 * sg - (R)a.r0) / (R)a.dr));
  const int b1 = min(a.nbins - 1, (int)floor((r + 5 * sg - (R)a.r0) / (R)a.dr));
  R dldr = 0;
  for (int b = b0; b <= b1; ++b) {
    const R u = ((R)a.r0 + b * (R)a.dr - r) / sg;
    dldr += (R)sb[b] * ia * exp(-(R)0.5 * u * u) * u / sg;
  }
  return dldr;
}

template <typename R, int MODE>
__global__ void __launch_bounds__(32 * kAdjTileWarps) k_adj_tiles(KP p, AdjArgs a) {
  __shared__ AdjWarp<R> ws[kAdjTileWarps];
  __shared__ AdjTail<R> tails[kAdjTypePairs];
  const int nt = p.nion_t;
  if (MODE != kModeHist)
    for (int c = threadIdx.x; c < nt * nt; c += blockDim.x) {
      const int is = p.pidx[(c / nt + p.ndna) * p.nttyp + p.ndna + c % nt];
      AdjTail<R> t;
      if constexpr (sizeof(R) == 8) {
        const PairParam &q = p.pp[is];
        t = AdjTail<R>{q.dm2hi, q.sc2, (q.flags & kChr) ? q.fct : 0.0};
      } else {
        const PairParamF &q = p.ppf[is];
        t = AdjTail<R>{q.dm2hi, q.sc2, (q.flags & kChr) ? q.fct : 0.0f};
      }
      tails[(c / nt) * kAdjMaxIonTypes + c % nt] = t;
    }
  __syncthreads();
  constexpr unsigned kAll = 0xffffffffu;
  const int lane = threadIdx.x & 31, wi = threadIdx.x >> 5;
  const int n = a.n, T = (n + 31) >> 5;
  const int q = blockIdx.x * kAdjTileWarps + wi;
  if (q >= n3_pairs(T)) return;  // warp-uniform; no block barrier follows
  AdjWarp<R> &w = ws[wi];
  int I, J;
  n3_pair(T, q, I, J);
  const bool diag = I == J;
  const R *vin = (const R *)a.v;
  const int j = J * 32 + lane, ncol = min(32, n - J * 32);
  if (j < n) {
    w.h[lane] = a.h[j];
    w.l[lane] = a.l[j];
    if (MODE == kModeBack) {
      w.v[0][lane] = vin[j];
      w.v[1][lane] = vin[n + j];
      w.v[2][lane] = vin[2 * n + j];
    }
  }
  w.s[0][lane] = w.s[1][lane] = w.s[2][lane] = (R)0;
  const int t = I * 32 + lane;
  const bool tv = t < n;
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
  const bool dep = MODE == kModeHist || (MODE == kModeForce && a.deposit);
  const R rcut2 = MODE == kModeForce && !a.deposit ? (R)0 : (R)a.rcut2;
  const unsigned below = (1u << lane) - 1u;
  R ox = 0, oy = 0, oz = 0;
  R ttail[kAdjMaxIonTypes] = {0, 0, 0, 0};
  int qn = 0;  // queued pairs (warp-uniform)
  // separation of row ion (h0, l0) and column entry m, as the FP32 path forms it
  auto sep = [&](const float4 &h0, const float4 &l0, int m, R &dx, R &dy, R &dz) {
    const float4 h = w.h[m], l = w.l[m];
    dx = (to_r<R>(h0.x, l0.x) - to_r<R>(h.x, l.x)) + (sizeof(R) == 8 ? R(0) : R(l0.x - l.x));
    dy = (to_r<R>(h0.y, l0.y) - to_r<R>(h.y, l.y)) + (sizeof(R) == 8 ? R(0) : R(l0.y - l.y));
    dz = (to_r<R>(h0.z, l0.z) - to_r<R>(h.z, l.z)) + (sizeof(R) == 8 ? R(0) : R(l0.z - l.z));
  };
  auto add_tail = [&](int tb, R v) {
#pragma unroll
    for (int m = 0; m < kAdjMaxIonTypes; ++m)
      if (m == tb) ttail[m] += v;
  };
  auto flush = [&]() {  // warp-uniform
    for (int b = 0; b < qn; b += 32) {
      const int idx = b + lane;
      const bool act = idx < qn;
      const int ent = act ? w.q[idx] : 0;
      const int rl = ent & 31, m = ent >> 5;
      // the row ion: lane rl's records
      const float4 h0 = make_float4(__shfl_sync(kAll, th.x, rl), __shfl_sync(kAll, th.y, rl),
                                    __shfl_sync(kAll, th.z, rl), 0.f);
      const float4 l0 = make_float4(__shfl_sync(kAll, tl.x, rl), __shfl_sync(kAll, tl.y, rl),
                                    __shfl_sync(kAll, tl.z, rl), 0.f);
      const int rcode = __shfl_sync(kAll, tcode, rl), ra = rcode - p.ndna;
      const R rvx = __shfl_sync(kAll, tvx, rl), rvy = __shfl_sync(kAll, tvy, rl),
              rvz = __shfl_sync(kAll, tvz, rl);
      R px = 0, py = 0, pz = 0, pt = 0;
      int tb = 0;
      if (act) {
        R dx, dy, dz;
        sep(h0, l0, m, dx, dy, dz);
        const R x2 = dx * dx + dy * dy + dz * dz;
        const int scode = __float_as_int(w.h[m].w) & 0xffff;
        tb = scode - p.ndna;
        if (MODE == kModeHist) {
          adj_deposit<R>(p, a, ra, scode, sqrt(x2));
        } else {
          const int is = p.pidx[rcode * p.nttyp + scode];
          R g, gp, r;
          int region, piece = 0;
          efp_adj<R>(p, is, x2, g, gp, r, region, piece);
          if (MODE == kModeForce) {
            if (dep && x2 < rcut2) adj_deposit<R>(p, a, ra, scode, r);
            px = g * dx;
            py = g * dy;
            pz = g * dz;
          } else {
            const R vx = rvx - w.v[0][m], vy = rvy - w.v[1][m], vz = rvz - w.v[2][m];
            const R qv = dx * vx + dy * vy + dz * vz;
            R r_, ir, ir2;
            efp_r<R>(x2, r_, ir, ir2);
            const R c = gp * ir * qv;
            px = g * vx + c * dx;
            py = g * vy + c * dy;
            pz = g * vz + c * dz;
            if (a.theta) {
              if (region == 0) {
                atomicAdd(a.g_ep + 3 * piece + 1, (double)(-qv * ir));
                atomicAdd(a.g_ep + 3 * piece + 2, (double)(-2 * qv));
              } else if (region == 1) {
                const R i6 = ir2 * ir2 * ir2;
                atomicAdd(a.g_sc + 3 * is, (double)(12 * i6 * i6 * ir2 * qv));
              } else {
                pt = 6 * ir2 * ir2 * ir2 * ir2 * qv;
              }
            }
            if (x2 < rcut2) {
              const R dldr = adj_dldr<R>(p, a, ra, scode, r);
              px += dldr * dx * ir;
              py += dldr * dy * ir;
              pz += dldr * dz * ir;
            }
          }
        }
      }
      if (MODE != kModeHist) {
        const int nb = min(32, qn - b);
        for (int u = 0; u < nb; ++u) {  // queue order
          const int rt = __shfl_sync(kAll, rl, u), mt = __shfl_sync(kAll, m, u),
                    tbt = __shfl_sync(kAll, tb, u);
          const R vx = __shfl_sync(kAll, px, u), vy = __shfl_sync(kAll, py, u),
                  vz = __shfl_sync(kAll, pz, u), vt = __shfl_sync(kAll, pt, u);
          if (lane == rt) {
            ox += vx;
            oy += vy;
            oz += vz;
            w.s[0][mt] -= vx;
            w.s[1][mt] -= vy;
            w.s[2][mt] -= vz;
            if (MODE == kModeBack) add_tail(tbt, vt);
          }
          __syncwarp();
        }
      }
    }
    qn = 0;
  };
  __syncwarp();
  const int k0 = diag ? 1 : 0, k1 = diag ? 16 : 31;
  for (int k = k0; k <= k1; ++k) {
    const int mm = (lane + k) & 31;
    bool slow = false;
    if (tv && mm < ncol && !(diag && k == 16 && lane >= 16)) {
      R dx, dy, dz;
      sep(th, tl, mm, dx, dy, dz);
      const R x2 = dx * dx + dy * dy + dz * dz;
      if (MODE == kModeHist) {
        slow = x2 < rcut2;
      } else {
        const int tb = (__float_as_int(w.h[mm].w) & 0xffff) - p.ndna;
        const AdjTail<R> L = tails[ta * kAdjMaxIonTypes + tb];
        slow = !(x2 > L.dm2hi) || x2 < rcut2;
        if (!slow) {  // the analytic tail, outside the histogram's range
          R r, ir, ir2, g, gp;
          efp_r<R>(x2, r, ir, ir2);
          efp_tail<R>(L.sc2, L.fct, ir, ir2, g, gp);
          R px, py, pz;
          if (MODE == kModeForce) {
            px = g * dx;
            py = g * dy;
            pz = g * dz;
          } else {
            const R vx = tvx - w.v[0][mm], vy = tvy - w.v[1][mm], vz = tvz - w.v[2][mm];
            const R qv = dx * vx + dy * vy + dz * vz;
            const R c = gp * ir * qv;
            px = g * vx + c * dx;
            py = g * vy + c * dy;
            pz = g * vz + c * dz;
            if (a.theta) add_tail(tb, 6 * ir2 * ir2 * ir2 * ir2 * qv);
          }
          ox += px;
          oy += py;
          oz += pz;
          w.s[0][mm] -= px;
          w.s[1][mm] -= py;
          w.s[2][mm] -= pz;
        }
      }
    }
    const unsigned bs = __ballot_sync(kAll, slow);
    if (slow) w.q[qn + __popc(bs & below)] = lane | (mm << 5);
    qn += __popc(bs);
    __syncwarp();
    if (qn > kAdjQ - 32) flush();
  }
  if (qn) flush();
  if (MODE == kModeHist) return;
  R *o = (R *)a.out + (size_t)q * 192;
  o[lane] = tv ? ox : (R)0;
  o[32 + lane] = tv ? oy : (R)0;
  o[64 + lane] = tv ? oz : (R)0;
  o[96 + lane] = w.s[0][lane];
  o[128 + lane] = w.s[1][lane];
  o[160 + lane] = w.s[2][lane];
  if (MODE == kModeBack && a.theta) {
    // the tail sums per (row type, column type), over the warp in a fixed
    // shuffle tree
    R *tq = (R *)a.tail + q;
    const size_t np = n3_pairs(T);
#pragma unroll
    for (int m = 0; m < kAdjMaxIonTypes; ++m) {
      if (m >= nt) break;
      for (int ra = 0; ra < nt; ++ra) {
        R v = ra == ta && tv ? ttail[m] : (R)0;
#pragma unroll
        for (int o2 = 16; o2 > 0; o2 >>= 1) v += __shfl_xor_sync(kAll, v, o2);
        if (lane == 0) tq[(ra * kAdjMaxIonTypes + m) * np] = v;
      }
    }
  }
}

// dL/dtheta of the tail constants: per (row type, column type) the sum over
// the tile pairs in a fixed order -- kTailBlocks blocks each sum a stretch of
// tile pairs (a strided pass, then a fixed shuffle and warp order) into
// part[block][type pair], then a warp per type pair adds the blocks' sums
// (a fixed shuffle tree) and one thread adds each type pair's total to g_sc,
// one type pair after another.
// FP64 sums spread over the SMs (the FP64 rate of one SM is low).
constexpr int kTailBlocks = 64, kTailThreads = 256;
template <typename R>
__global__ void __launch_bounds__(kTailThreads)
    k_adj_tails(KP p, const R *tail, int npair, double *part) {
  __shared__ double wsum[kAdjTypePairs][kTailThreads / 32];
  const int nt = p.nion_t, w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int per = (npair + kTailBlocks - 1) / kTailBlocks;
  const int k0 = blockIdx.x * per, k1 = min(npair, k0 + per);
  for (int c = 0; c < nt * nt; ++c) {
    const int off = (c / nt) * kAdjMaxIonTypes + c % nt;
    double v = 0.0;
    for (int k = k0 + threadIdx.x; k < k1; k += kTailThreads)
      v += (double)tail[(size_t)off * npair + k];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) wsum[c][w] = v;
  }
  __syncthreads();
  if (threadIdx.x < nt * nt) {
    double v = 0.0;
    for (int k = 0; k < kTailThreads / 32; ++k) v += wsum[threadIdx.x][k];
    part[(size_t)blockIdx.x * kAdjTypePairs + threadIdx.x] = v;
  }
}

__global__ void k_adj_tails_fin(KP p, const double *part, double *g_sc) {
  static_assert(kTailBlocks == 64, "two block sums a lane");
  __shared__ double tot[kAdjTypePairs];
  const int nt = p.nion_t, w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int c = w; c < nt * nt; c += blockDim.x >> 5) {  // a warp per type pair
    double v = part[(size_t)lane * kAdjTypePairs + c] +
               part[(size_t)(lane + 32) * kAdjTypePairs + c];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) tot[c] = v;
  }
  __syncthreads();
  if (threadIdx.x == 0)
    for (int c = 0; c < nt * nt; ++c) {
      const int is = p.pidx[(c / nt + p.ndna) * p.nttyp + p.ndna + c % nt];
      g_sc[3 * is + 2] += tot[c];
    }
}

// The sums of tile t's 32 particles over their tile-pair partials, in a
// fixed order: block of kGatherWarps warps, warp w takes the tile pairs (u,
// t) and (t, u) of u = w, w + kGatherWarps, ... in order, then warp 0 adds
// the warps' sums in order w = 0, 1, ... (lane l: particle 32 t + l).
constexpr int kGatherWarps = 8;
template <typename R>
__device__ __forceinline__ void adj_gather_tile(const R *tp, int n, int t, R (&F)[3]) {
  __shared__ R sh[kGatherWarps][3][32];
  const int T = (n + 31) >> 5, lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  R v[3] = {0, 0, 0};
#pragma unroll 4
  for (int u = w; u < T; u += kGatherWarps) {
    const R *e = tp + (size_t)(u <= t ? n3_index(T, u, t) : n3_index(T, t, u)) * 192 + lane;
    for (int k = 0; k < 3; ++k) {
      if (u < t)
        v[k] += e[96 + 32 * k];
      else if (u > t)
        v[k] += e[32 * k];
      else
        v[k] += e[32 * k] + e[96 + 32 * k];
    }
  }
  for (int k = 0; k < 3; ++k) sh[w][k][lane] = v[k];
  __syncthreads();
  for (int k = 0; k < 3; ++k) {
    R s = 0;
    for (int x = 0; x < kGatherWarps; ++x) s += sh[x][k][lane];
    F[k] = s;
  }
}

// Forward step, a block per tile: forces from the tile-pair partials (fixed
// order), the BD move of dynamics0 with frozen noise, the box clamp, and the
// clamp masks of the step (bit k: bdmax clamp of component k; bit 3 + k:
// wall clamp).
template <typename R>
__global__ void __launch_bounds__(32 * kGatherWarps)
    k_adj_move(KP p, const float4 *h, const float4 *l, const R *part, int n, float4 *hn,
               float4 *ln, uint8_t *mask, BoxF box, uint64_t seed, uint64_t step) {
  R F[3];
  adj_gather_tile(part, n, blockIdx.x, F);
  const int i = blockIdx.x * 32 + threadIdx.x;
  if (threadIdx.x >= 32 || i >= n) return;
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

// Backward, after the pair sweep, a block per tile: a = mu + the tile-pair
// partials.
template <typename R>
__global__ void __launch_bounds__(32 * kGatherWarps)
    k_adj_combine(const R *mu, const R *part, int n, R *a) {
  R F[3];
  adj_gather_tile(part, n, blockIdx.x, F);
  const int i = blockIdx.x * 32 + threadIdx.x;
  if (threadIdx.x >= 32 || i >= n) return;
  for (int k = 0; k < 3; ++k) a[(size_t)k * n + i] = (mu ? mu[(size_t)k * n + i] : (R)0) + F[k];
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
  size_t part_bytes = 0, tail_bytes = 0;  // tile-pair partials (grow-only)
  void *tail = nullptr;
  int *typei = nullptr;
  float4 *x0h = nullptr, *x0l = nullptr;    // initial configuration
  float4 *xfh = nullptr, *xfl = nullptr;    // final configuration of the forward run
  std::vector<float4 *> ckh, ckl;           // checkpoints
  std::vector<float4 *> trh, trl;           // one recomputed segment, ckpt + 1 slots
  uint8_t *mask = nullptr;                  // [ckpt][cap]
  void *part = nullptr, *a = nullptr, *mu = nullptr, *v = nullptr;
  unsigned long long *hist = nullptr;
  double *sbin = nullptr, *g_ep = nullptr, *g_sc = nullptr;
  double *tail_part = nullptr;  // [kTailBlocks][kAdjTypePairs]
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

// (re)allocates *p for at least `bytes` (grow-only); `have` tracks its size
int agrow(bromoc_adj *ad, void **p, size_t &have, size_t bytes) {
  if (*p && bytes <= have) return BROMOC_OK;
  if (*p) {
    cudaFree(*p);
    ad->allocs.erase(std::find(ad->allocs.begin(), ad->allocs.end(), *p));
    *p = nullptr;
    have = 0;
  }
  cudaError_t e = cudaMalloc(p, std::max<size_t>(bytes, 1));
  if (e != cudaSuccess)
    return aset(ad, BROMOC_E_NOMEM, "cudaMalloc(%zu bytes): %s", bytes, cudaGetErrorString(e));
  ad->allocs.push_back(*p);
  have = bytes;
  return BROMOC_OK;
}

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
               const void *v, bool obs, bool theta, bool deposit = false) {
  AdjArgs a{};
  a.h = h;
  a.l = l;
  a.v = v;
  a.out = ad->part;
  a.tail = ad->tail;
  a.g_ep = ad->g_ep;
  a.g_sc = ad->g_sc;
  a.hist = ad->hist;
  a.sbin = ad->sbin;
  a.n = ad->n;
  a.nbins = ad->nbins;
  a.deposit = deposit ? 1 : 0;
  a.r0 = (float)ad->r0;
  a.dr = (float)ad->dr;
  a.sigma = (float)ad->sigma;
  a.ia = 0.3989422804014327 / (double)a.sigma;
  const double rc = ad->r0 + ad->dr * (ad->nbins - 1) + 5.0 * ad->sigma;
  a.rcut2 = obs || deposit ? (float)(rc * rc) : 0.0f;
  a.theta = theta ? 1 : 0;
  const int npair = n3_pairs((ad->n + 31) / 32);
  const int g = (npair + kAdjTileWarps - 1) / kAdjTileWarps, b = 32 * kAdjTileWarps;
  if (mode == kModeForce) {
    k_adj_tiles<R, kModeForce><<<g, b, 0, ad->stream>>>(p, a);
  } else if (mode == kModeBack) {
    k_adj_tiles<R, kModeBack><<<g, b, 0, ad->stream>>>(p, a);
    if (theta) {
      k_adj_tails<R><<<kTailBlocks, kTailThreads, 0, ad->stream>>>(p, (const R *)ad->tail,
                                                                   npair, ad->tail_part);
      k_adj_tails_fin<<<1, 32 * kAdjTypePairs, 0, ad->stream>>>(p, ad->tail_part, ad->g_sc);
    }
  } else {
    k_adj_tiles<R, kModeHist><<<g, b, 0, ad->stream>>>(p, a);
  }
}

// one forward step from (h, l); deposit: the histogram of (h, l) in the same
// pair sweep
template <typename R>
void step_forward(bromoc_adj *ad, const KP &p, const float4 *h, const float4 *l, float4 *hn,
                  float4 *ln, uint8_t *mask, uint64_t step, bool deposit = false) {
  run_pairs<R>(ad, p, kModeForce, h, l, nullptr, false, false, deposit);
  k_adj_move<R><<<(ad->n + 31) / 32, 32 * kGatherWarps, 0, ad->stream>>>(
      p, h, l, (const R *)ad->part, ad->n, hn, ln, mask, p.f.box, ad->seed, step);
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
  // the histogram of x_1 .. x_T: x_t's deposit rides on step t's force
  // sweep, x_T's is a sweep of its own
  const float4 *h = ad->x0h, *l = ad->x0l;
  for (int t = 0; t < ad->nsteps; ++t) {
    float4 *hn = ad->trh[(t + 1) & 1], *ln = ad->trl[(t + 1) & 1];
    step_forward<R>(ad, p, h, l, hn, ln, nullptr, ad->step0 + t, t >= 1);
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
  run_pairs<R>(ad, p, kModeHist, h, l, nullptr, true, false);
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
  const int ntile = (n + 31) / 32, gb = 32 * kGatherWarps;
  k_adj_combine<R><<<ntile, gb, 0, ad->stream>>>(nullptr, (const R *)ad->part, n, (R *)ad->a);
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
      k_adj_combine<R><<<ntile, gb, 0, ad->stream>>>((const R *)ad->mu, (const R *)ad->part, n,
                                                     (R *)ad->a);
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
  if (!rc) rc = aalloc(ad, &buf, rs * 3 * cap * 3);  // a, mu, v
  if (!rc) {
    ad->a = buf;
    ad->mu = buf + rs * 3 * cap;
    ad->v = buf + rs * 3 * cap * 2;
  }
  if (!rc) rc = aalloc(ad, &ad->g_ep, 3 * (size_t)std::max(pk->cnt, 1));
  if (!rc) rc = aalloc(ad, &ad->g_sc, 3 * (size_t)pk->ntc);
  if (!rc) rc = aalloc(ad, &ad->tail_part, (size_t)kTailBlocks * kAdjTypePairs);
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
  // tile-pair partials: [tile pair][side][3][32] and the tail sums
  const size_t npair = n3_pairs((n + 31) / 32), rs = ad->precision == BROMOC_FP64 ? 8 : 4;
  if ((rc = agrow(ad, &ad->part, ad->part_bytes, npair * 192 * rs)) ||
      (rc = agrow(ad, &ad->tail, ad->tail_bytes, npair * kAdjTypePairs * rs)))
    return rc;
  ad->n = n;
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
