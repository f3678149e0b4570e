// ENERGY on the device (energy.mono.f90:19-692 without the DNA bonded
// terms).  One launch per term family; partial forces and block-partial
// energies go to scratch and are reduced in a fixed order, so a run is
// bit-reproducible.
#include "launch.h"
#include "physics.cuh"

namespace bgpu {

constexpr int kPairThreads = 64;  // targets per block == source tile size

// ---------------------------------------------------------------------------
// Ion-ion pairs, FP64.  Block (tx, cy): 128 mobile targets x source chunk cy.
// Every target sums over all other ions of the chunk; the energy of a pair of
// two mobile ions is counted half by each, that of a mobile-fixed pair once.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kPairThreads)
    k_ionion64(KP p, int qforces, int slot0) {
  __shared__ double sx[kPairThreads], sy[kPairThreads], sz[kPairThreads];
  __shared__ int sc[kPairThreads];
  __shared__ double red[(kPairThreads / 32) * 4];
  const int ntot = p.st->ntot;
  const int m0 = p.nsites + p.nfix;
  const int t = m0 + blockIdx.x * kPairThreads + threadIdx.x;
  const bool tv = t < ntot;
  const int s0 = p.nsites + blockIdx.y * p.chunk_ii;
  const int s1 = min(ntot, s0 + p.chunk_ii);
  double xt = 0, yt = 0, zt = 0;
  int row = 0;
  if (tv) {
    xt = p.x[t];
    yt = p.y[t];
    zt = p.z[t];
    row = (p.nwtype[abs(p.typei[t])] - 1) * p.nttyp;
  }
  double fxa = 0.0, fya = 0.0, fza = 0.0, e[4] = {0, 0, 0, 0};
  int err = 0;
  for (int base = s0; base < s1; base += kPairThreads) {
    const int s = base + threadIdx.x;
    __syncthreads();
    if (s < s1) {
      sx[threadIdx.x] = p.x[s];
      sy[threadIdx.x] = p.y[s];
      sz[threadIdx.x] = p.z[s];
      sc[threadIdx.x] = (p.nwtype[abs(p.typei[s])] - 1) | ((s >= m0) << 16);
    }
    __syncthreads();
    const int n = min(kPairThreads, s1 - base);
    if (tv) {
      for (int k = 0; k < n; ++k) {
        if (base + k == t) continue;
        const int code = sc[k];
        const PairParam &q = p.pp[p.pidx[row + (code & 0xffff)]];
        const double dx = xt - sx[k], dy = yt - sy[k], dz = zt - sz[k];
        const double d2 = dx * dx + dy * dy + dz * dz;
        const double w = (code >> 16) ? 0.5 : 1.0;
        double dist;
        const double de = law64(p, q, d2, w, e, dist, err);
        if (qforces) {
          fxa += de * dx;
          fya += de * dy;
          fza += de * dz;
        }
      }
    }
  }
  if (tv) {
    double *f = p.fii + (size_t)blockIdx.y * 3 * p.cap;
    f[t] = fxa;
    f[p.cap + t] = fya;
    f[2 * p.cap + t] = fza;
  }
  if (err) atomicOr(&p.st->err, err);
  __shared__ double tot[4];
  block_sum<4>(e, red, tot);
  if (threadIdx.x == 0) {
    double *dst = p.epart + (size_t)(slot0 + blockIdx.y * gridDim.x + blockIdx.x) * kNTerms;
    for (int k = 0; k < kNTerms; ++k) dst[k] = 0.0;
    dst[1] = tot[0];
    dst[2] = tot[1];
    dst[3] = tot[2];
    dst[4] = tot[3];
  }
}

// hi/lo split of a double coordinate: x == hi + lo to ~2^-48 relative, so
// (hi_i - hi_j) + (lo_i - lo_j) keeps ~1e-7 relative accuracy of dx even
// when |x| >> |dx|.
__device__ __forceinline__ void split2(double v, float &hi, float &lo) {
  hi = (float)v;
  lo = (float)(v - (double)hi);
}

// ---------------------------------------------------------------------------
// Ion-ion pairs, FP32 arithmetic with per-tile FP32 and cross-tile FP64
// accumulation.  Same decomposition as k_ionion64.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kPairThreads)
    k_ionion32(KP p, int qforces, int slot0) {
  __shared__ float4 sh[kPairThreads];
  __shared__ float4 sl[kPairThreads];
  __shared__ double red[(kPairThreads / 32) * 4];
  const int ntot = p.st->ntot;
  const int m0 = p.nsites + p.nfix;
  const int t = m0 + blockIdx.x * kPairThreads + threadIdx.x;
  const bool tv = t < ntot;
  const int s0 = p.nsites + blockIdx.y * p.chunk_ii;
  const int s1 = min(ntot, s0 + p.chunk_ii);
  float xh = 0, yh = 0, zh = 0, xl = 0, yl = 0, zl = 0;
  int row = 0;
  if (tv) {
    split2(p.x[t], xh, xl);
    split2(p.y[t], yh, yl);
    split2(p.z[t], zh, zl);
    row = (p.nwtype[abs(p.typei[t])] - 1) * p.nttyp;
  }
  double fxa = 0.0, fya = 0.0, fza = 0.0, ed[4] = {0, 0, 0, 0};
  int err = 0;
  for (int base = s0; base < s1; base += kPairThreads) {
    const int s = base + threadIdx.x;
    __syncthreads();
    if (s < s1) {
      float4 h, l;
      split2(p.x[s], h.x, l.x);
      split2(p.y[s], h.y, l.y);
      split2(p.z[s], h.z, l.z);
      h.w = __int_as_float((p.nwtype[abs(p.typei[s])] - 1) | ((s >= m0) << 16));
      l.w = 0.0f;
      sh[threadIdx.x] = h;
      sl[threadIdx.x] = l;
    }
    __syncthreads();
    const int n = min(kPairThreads, s1 - base);
    if (tv) {
      float fx = 0.f, fy = 0.f, fz = 0.f, e[4] = {0.f, 0.f, 0.f, 0.f};
      for (int k = 0; k < n; ++k) {
        if (base + k == t) continue;
        const float4 h = sh[k], l = sl[k];
        const int code = __float_as_int(h.w);
        const int is = __ldg(p.pidx + row + (code & 0xffff));
        const float dx = (xh - h.x) + (xl - l.x);
        const float dy = (yh - h.y) + (yl - l.y);
        const float dz = (zh - h.z) + (zl - l.z);
        const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
        const float w = (code >> 16) ? 0.5f : 1.0f;
        const float de = law32k(p, is, r2, w, e);
        fx = fmaf(de, dx, fx);
        fy = fmaf(de, dy, fy);
        fz = fmaf(de, dz, fz);
      }
      if (qforces) {
        fxa += fx;
        fya += fy;
        fza += fz;
      }
#pragma unroll
      for (int m = 0; m < 4; ++m) ed[m] += e[m];
    }
  }
  if (tv) {
    double *f = p.fii + (size_t)blockIdx.y * 3 * p.cap;
    f[t] = fxa;
    f[p.cap + t] = fya;
    f[2 * p.cap + t] = fza;
  }
  __shared__ double tot[4];
  block_sum<4>(ed, red, tot);
  if (threadIdx.x == 0) {
    double *dst = p.epart + (size_t)(slot0 + blockIdx.y * gridDim.x + blockIdx.x) * kNTerms;
    for (int k = 0; k < kNTerms; ++k) dst[k] = 0.0;
    dst[1] = tot[0];
    dst[2] = tot[1];
    dst[3] = tot[2];
    dst[4] = tot[3];
  }
}

// ---------------------------------------------------------------------------
// Ion-site pairs, ion-centred (energy.mono.f90:585-687): each ion walks the
// sites in order (which also reproduces the PROXDIFF nearest-site record,
// seeded by site 1 exactly as the reference).  Energies of all pairs, forces
// on mobile ions.  Sites are staged in shared memory (nsites <= 1024).
// ---------------------------------------------------------------------------
template <bool FP32>
__global__ void __launch_bounds__(kPairThreads)
    k_ionsite(KP p, int qforces, int slot0) {
  extern __shared__ double sm[];
  double *sxs = sm, *sys = sm + p.nsites, *szs = sm + 2 * p.nsites;
  int *sts = (int *)(sm + 3 * p.nsites);
  __shared__ double red[(kPairThreads / 32) * 4];
  for (int k = threadIdx.x; k < p.nsites; k += blockDim.x) {
    sxs[k] = p.x[k];
    sys[k] = p.y[k];
    szs[k] = p.z[k];
    sts[k] = p.typtyp[k] - 1;
  }
  __syncthreads();
  const int ntot = p.st->ntot;
  const int i = p.nsites + blockIdx.x * blockDim.x + threadIdx.x;
  double e[4] = {0, 0, 0, 0};
  int err = 0;
  if (i < ntot) {
    const bool mobile = i >= p.nsites + p.nfix;
    const double xi = p.x[i], yi = p.y[i], zi = p.z[i];
    const int row = (p.nwtype[abs(p.typei[i])] - 1) * p.nttyp;
    double f[3] = {0, 0, 0}, dd[5] = {0, 0, 0, 0, 0};
    for (int j = 0; j < p.nsites; ++j) {
      const int is = p.pidx[row + sts[j]];
      const double dx = xi - sxs[j], dy = yi - sys[j], dz = zi - szs[j];
      const double d2 = dx * dx + dy * dy + dz * dz;
      double de, dist = 0.0;
      if (FP32) {
        float ef[4] = {0.f, 0.f, 0.f, 0.f};
        const float r2 = (float)d2;
        de = (double)law32(p, p.ppf[is], r2, 1.0f, ef, err);
        for (int m = 0; m < 4; ++m) e[m] += (double)ef[m];
        if (p.qproxdiff && (p.pp[is].flags & kEfp) && d2 >= p.pp[is].dm2lo &&
            d2 <= p.pp[is].dm2hi)
          dist = sqrt(d2);
      } else {
        de = law64(p, p.pp[is], d2, 1.0, e, dist, err);
      }
      if (p.qproxdiff && (p.pp[is].flags & kEfp) && dist > 0.0) {
        const double dm = dist - p.pp[is].dmi;
        if (j == 0 || dm < dd[0]) {
          dd[0] = dm;
          dd[1] = dist;
          dd[2] = dx;
          dd[3] = dy;
          dd[4] = dz;
        }
      }
      if (qforces && mobile) {
        f[0] += de * dx;
        f[1] += de * dy;
        f[2] += de * dz;
      }
    }
    p.fis[i] = f[0];
    p.fis[p.cap + i] = f[1];
    p.fis[2 * p.cap + i] = f[2];
    if (p.qproxdiff)
      for (int m = 0; m < 5; ++m) p.dids[5 * i + m] = dd[m];
  }
  if (err) atomicOr(&p.st->err, err);
  __shared__ double tot[4];
  // site terms: eqqmx(5) evdwmx(6) esrpmfmx(7) eefpotmx(8)
  block_sum<4>(e, red, tot);
  if (threadIdx.x == 0) {
    double *dst = p.epart + (size_t)(slot0 + blockIdx.x) * kNTerms;
    for (int k = 0; k < kNTerms; ++k) dst[k] = 0.0;
    dst[5] = tot[0];
    dst[6] = tot[1];
    dst[7] = tot[2];
    dst[8] = tot[3];
  }
}

// Forces on free sites: block per site, threads over ions, fixed-tree sum.
template <bool FP32>
__global__ void __launch_bounds__(kPairThreads) k_siteforce(KP p) {
  __shared__ double red[(kPairThreads / 32) * 3];
  const int j = blockIdx.x;
  const int ntot = p.st->ntot;
  double f[3] = {0, 0, 0};
  int err = 0;
  if (p.stfree[j]) {
    const double xj = p.x[j], yj = p.y[j], zj = p.z[j];
    const int col = p.typtyp[j] - 1;
    for (int i = p.nsites + threadIdx.x; i < ntot; i += blockDim.x) {
      const int is = p.pidx[(p.nwtype[abs(p.typei[i])] - 1) * p.nttyp + col];
      const double dx = p.x[i] - xj, dy = p.y[i] - yj, dz = p.z[i] - zj;
      const double d2 = dx * dx + dy * dy + dz * dz;
      double de, dist;
      if (FP32) {
        float ef[4];
        de = (double)law32(p, p.ppf[is], (float)d2, 0.0f, ef, err);
      } else {
        double ed[4];
        de = law64(p, p.pp[is], d2, 0.0, ed, dist, err);
      }
      f[0] -= de * dx;
      f[1] -= de * dy;
      f[2] -= de * dz;
    }
  }
  __shared__ double tot[3];
  block_sum<3>(f, red, tot);
  if (threadIdx.x == 0) {
    p.fis[j] = tot[0];
    p.fis[p.cap + j] = tot[1];
    p.fis[2 * p.cap + j] = tot[2];
  }
}

// ---------------------------------------------------------------------------
// RFPAR cross term (rfpar.f90:177-223), target-centred over in-grid ions.
// Pair (i > j) counts when i is mobile and srfe(j) != 0; its energy is added
// by the target that plays i, each side adds its own force:
//   F_t = A sd1_t + B sd2_t + P,  A = sum -a1 srfe_s,  B = sum aux3 reff_s,
//   P = sum a2 reff_ts (r_t - r_s).
// ---------------------------------------------------------------------------
template <bool FP32>
__global__ void __launch_bounds__(kPairThreads)
    k_rfcross(KP p, int qforces, int slot0) {
  __shared__ double sx[kPairThreads], sy[kPairThreads], sz[kPairThreads];
  __shared__ double ss[kPairThreads], sr[kPairThreads], sq[kPairThreads];
  __shared__ int sflag[kPairThreads];
  __shared__ double red[(kPairThreads / 32) * 1];
  const int ntot = p.st->ntot;
  const int m0 = p.nsites + p.nfix;
  const int t = p.nsites + blockIdx.x * kPairThreads + threadIdx.x;
  const bool tv = t < ntot && p.rf_in[t];
  const int s0 = p.nsites + blockIdx.y * p.chunk_rf;
  const int s1 = min(ntot, s0 + p.chunk_rf);
  double xt = 0, yt = 0, zt = 0, srt = 0, rft = 0, qt = 0;
  if (tv) {
    xt = p.x[t];
    yt = p.y[t];
    zt = p.z[t];
    srt = p.rf_srfe[t];
    rft = p.rf_reff[t];
    qt = p.cg[abs(p.typei[t])];
  }
  const bool tmob = t >= m0;
  double A = 0, B = 0, P[3] = {0, 0, 0}, e = 0;
  for (int base = s0; base < s1; base += kPairThreads) {
    const int s = base + threadIdx.x;
    __syncthreads();
    if (s < s1) {
      sx[threadIdx.x] = p.x[s];
      sy[threadIdx.x] = p.y[s];
      sz[threadIdx.x] = p.z[s];
      ss[threadIdx.x] = p.rf_srfe[s];
      sr[threadIdx.x] = p.rf_reff[s];
      sq[threadIdx.x] = p.cg[abs(p.typei[s])];
      sflag[threadIdx.x] = p.rf_in[s] | ((s >= m0) << 1);
    }
    __syncthreads();
    const int n = min(kPairThreads, s1 - base);
    if (tv) {
      for (int k = 0; k < n; ++k) {
        const int s = base + k;
        if (s == t) continue;
        const int fl = sflag[k];
        if (!(fl & 1)) continue;
        // roles: i = max(t, s) must be mobile, srfe(min) must be nonzero
        const bool t_is_i = t > s;
        const bool i_mobile = t_is_i ? tmob : ((fl >> 1) & 1);
        const double srj = t_is_i ? ss[k] : srt;
        if (!i_mobile || srj == 0.0) continue;
        const double dx = xt - sx[k], dy = yt - sy[k], dz = zt - sz[k];
        if (FP32) {
          const float d2 = (float)(dx * dx + dy * dy + dz * dz);
          const float rij = (float)(sr[k] * rft);
          const float srij = (float)(ss[k] * srt);
          const float rfdn = rsqrtf(fmaf(rij, rij, d2));
          const float aux0 = (float)(p.celec * qt * sq[k]);
          const float a1 = aux0 * rij * rfdn;
          if (t_is_i) e += (double)(a1 * srij);
          if (qforces) {
            const float a2 = aux0 * srij * rfdn * rfdn * rfdn;
            const float aux3 = -a2 * (d2 + rij * 0.5f);
            A += (double)(-a1 * (float)ss[k]);
            B += (double)(aux3 * (float)sr[k]);
            const float pr = a2 * rij;
            P[0] += (double)pr * dx;
            P[1] += (double)pr * dy;
            P[2] += (double)pr * dz;
          }
        } else {
          const double d2 = dx * dx + dy * dy + dz * dz;
          const double rij = sr[k] * rft;
          const double srij = ss[k] * srt;
          const double rfdn = 1.0 / sqrt(rij * rij + d2);
          const double aux0 = p.celec * qt * sq[k];
          const double a1 = aux0 * (rij * rfdn);
          if (t_is_i) e += a1 * srij;
          if (qforces) {
            const double a2 = aux0 * srij * rfdn * rfdn * rfdn;
            const double aux3 = -a2 * (d2 + rij * 0.5);
            A += -a1 * ss[k];
            B += aux3 * sr[k];
            const double pr = a2 * rij;
            P[0] += pr * dx;
            P[1] += pr * dy;
            P[2] += pr * dz;
          }
        }
      }
    }
  }
  if (t < ntot) {
    double *f = p.frf + (size_t)blockIdx.y * 3 * p.cap;
    double fo[3] = {0, 0, 0};
    if (tv && qforces)
      for (int k = 0; k < 3; ++k)
        fo[k] = A * p.rf_d1[3 * t + k] + B * p.rf_d2[3 * t + k] + P[k];
    f[t] = fo[0];
    f[p.cap + t] = fo[1];
    f[2 * p.cap + t] = fo[2];
  }
  __shared__ double tot[1];
  block_sum<1>(&e, red, tot);
  if (threadIdx.x == 0) {
    double *dst = p.epart + (size_t)(slot0 + blockIdx.y * gridDim.x + blockIdx.x) * kNTerms;
    for (int k = 0; k < kNTerms; ++k) dst[k] = 0.0;
    dst[13] = tot[0];
  }
}

// ---------------------------------------------------------------------------
// RFPAR cross term in single precision: hi/lo coordinates, FP32 pair math,
// per-tile FP32 and cross-tile FP64 accumulation (no FP64 in the inner loop).
// Source tile: (x_hi, y_hi, z_hi, srfe) (x_lo, y_lo, z_lo, reff) (q, flags).
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kPairThreads)
    k_rfcross32(KP p, int qforces, int slot0) {
  __shared__ float4 sh[kPairThreads], sl[kPairThreads];
  __shared__ float2 sqf[kPairThreads];
  __shared__ double red[(kPairThreads / 32) * 1];
  const int ntot = p.st->ntot;
  const int m0 = p.nsites + p.nfix;
  const int t = p.nsites + blockIdx.x * kPairThreads + threadIdx.x;
  const bool tv = t < ntot && p.rf_in[t];
  const int s0 = p.nsites + blockIdx.y * p.chunk_rf;
  const int s1 = min(ntot, s0 + p.chunk_rf);
  float xh = 0, yh = 0, zh = 0, xl = 0, yl = 0, zl = 0, srt = 0, rft = 0, ct = 0;
  if (tv) {
    split2(p.x[t], xh, xl);
    split2(p.y[t], yh, yl);
    split2(p.z[t], zh, zl);
    srt = (float)p.rf_srfe[t];
    rft = (float)p.rf_reff[t];
    ct = (float)(p.celec * p.cg[abs(p.typei[t])]);
  }
  const bool tmob = t >= m0;
  double Ad = 0, Bd = 0, Pd[3] = {0, 0, 0}, ed = 0;
  for (int base = s0; base < s1; base += kPairThreads) {
    const int s = base + threadIdx.x;
    __syncthreads();
    if (s < s1) {
      float4 h, l;
      split2(p.x[s], h.x, l.x);
      split2(p.y[s], h.y, l.y);
      split2(p.z[s], h.z, l.z);
      h.w = (float)p.rf_srfe[s];
      l.w = (float)p.rf_reff[s];
      sh[threadIdx.x] = h;
      sl[threadIdx.x] = l;
      sqf[threadIdx.x] = make_float2((float)p.cg[abs(p.typei[s])],
                                     __int_as_float(p.rf_in[s] | ((s >= m0) << 1)));
    }
    __syncthreads();
    const int n = min(kPairThreads, s1 - base);
    if (tv) {
      float A = 0.f, B = 0.f, P0 = 0.f, P1 = 0.f, P2 = 0.f, e = 0.f;
      for (int k = 0; k < n; ++k) {
        const int s = base + k;
        const float2 qf = sqf[k];
        const int fl = __float_as_int(qf.y);
        if (s == t || !(fl & 1)) continue;
        const float4 h = sh[k], l = sl[k];
        const bool t_is_i = t > s;
        const bool i_mobile = t_is_i ? tmob : ((fl >> 1) & 1);
        const float srj = t_is_i ? h.w : srt;
        if (!i_mobile || srj == 0.0f) continue;
        const float dx = (xh - h.x) + (xl - l.x);
        const float dy = (yh - h.y) + (yl - l.y);
        const float dz = (zh - h.z) + (zl - l.z);
        const float d2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
        const float rij = l.w * rft, srij = h.w * srt;
        const float rfdn = rsqrtf(fmaf(rij, rij, d2));
        const float aux0 = ct * qf.x;
        const float a1 = aux0 * rij * rfdn;
        if (t_is_i) e = fmaf(a1, srij, e);
        const float a2 = aux0 * srij * rfdn * rfdn * rfdn;
        const float aux3 = -a2 * fmaf(rij, 0.5f, d2);
        A = fmaf(-a1, h.w, A);
        B = fmaf(aux3, l.w, B);
        const float pr = a2 * rij;
        P0 = fmaf(pr, dx, P0);
        P1 = fmaf(pr, dy, P1);
        P2 = fmaf(pr, dz, P2);
      }
      Ad += A;
      Bd += B;
      Pd[0] += P0;
      Pd[1] += P1;
      Pd[2] += P2;
      ed += e;
    }
  }
  if (t < ntot) {
    double *f = p.frf + (size_t)blockIdx.y * 3 * p.cap;
    double fo[3] = {0, 0, 0};
    if (tv && qforces)
      for (int k = 0; k < 3; ++k)
        fo[k] = Ad * p.rf_d1[3 * t + k] + Bd * p.rf_d2[3 * t + k] + Pd[k];
    f[t] = fo[0];
    f[p.cap + t] = fo[1];
    f[2 * p.cap + t] = fo[2];
  }
  __shared__ double tot[1];
  block_sum<1>(&ed, red, tot);
  if (threadIdx.x == 0) {
    double *dst = p.epart + (size_t)(slot0 + blockIdx.y * gridDim.x + blockIdx.x) * kNTerms;
    for (int k = 0; k < kNTerms; ++k) dst[k] = 0.0;
    dst[13] = tot[0];
  }
}

// ---------------------------------------------------------------------------
// Final energy reduction over all block slots in a fixed order, then the
// reference's totals: ener = ememb + egsbpa + evdwgd + erfpar + pair terms
// (energy.mono.f90:83-115, 689); egsbpb = erfpar when RFPAR is on.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_ereduce(KP p, int nslot, int rfpar_on) {
  __shared__ double red[(256 / 32) * kNTerms];
  double v[kNTerms];
#pragma unroll
  for (int k = 0; k < kNTerms; ++k) v[k] = 0.0;
  for (int s = threadIdx.x; s < nslot; s += blockDim.x) {
    const double *src = p.epart + (size_t)s * kNTerms;
#pragma unroll
    for (int k = 1; k < kNTerms; ++k) v[k] += src[k];
  }
  __shared__ double tot[kNTerms];
  block_sum<kNTerms>(v, red, tot);
  if (threadIdx.x == 0) {
    double o[kNTerms];
    for (int k = 0; k < kNTerms; ++k) o[k] = tot[k];
    o[11] = rfpar_on ? o[13] : 0.0;  // egsbpb = erfpar
    o[0] = o[9] + o[10] + o[12] + o[13] + o[1] + o[2] + o[3] + o[7] + o[5] +
           o[6] + o[4] + o[8];
    for (int k = 0; k < kNTerms; ++k) p.eterms[k] = o[k];
  }
}

// ---------------------------------------------------------------------------
// Host launcher: the energy pipeline of one step.
// ---------------------------------------------------------------------------
int launch_energy(const KP &p, const EnergyPlan &plan, uint32_t mask,
                  int qforces, cudaStream_t stream) {
  int slot = 0, nk = 0;
  const int nub = plan.ntot_ub;
  const int nfb = fields_blocks(nub);
  if (nfb > 0) {
    if (plan.t_fields) cudaEventRecord(plan.t_fields->a, stream);
    launch_fields(p, nub, mask, qforces, plan.fp32, slot, stream);
    if (plan.t_fields) cudaEventRecord(plan.t_fields->b, stream);
    slot += nfb;
    ++nk;
  }
  const bool nonbond = (mask & 1u) != 0;
  const int nmob_ub = nub - p.nsites - p.nfix;
  if (nonbond && nmob_ub > 0 && plan.nchunk_ii > 0) {
    dim3 g((nmob_ub + kPairThreads - 1) / kPairThreads, plan.nchunk_ii);
    if (plan.t_pairs) cudaEventRecord(plan.t_pairs->a, stream);
    if (plan.fp32)
      k_ionion32<<<g, kPairThreads, 0, stream>>>(p, qforces, slot);
    else
      k_ionion64<<<g, kPairThreads, 0, stream>>>(p, qforces, slot);
    if (plan.t_pairs) cudaEventRecord(plan.t_pairs->b, stream);
    slot += g.x * g.y;
    ++nk;
  }
  if (nonbond && p.nsites > 0 && nub > p.nsites) {
    const int nion_ub = nub - p.nsites;
    const int nb = (nion_ub + kPairThreads - 1) / kPairThreads;
    const size_t smem = (size_t)p.nsites * (3 * sizeof(double) + sizeof(int));
    if (plan.fp32) {
      k_ionsite<true><<<nb, kPairThreads, smem, stream>>>(p, qforces, slot);
      if (qforces) k_siteforce<true><<<p.nsites, kPairThreads, 0, stream>>>(p);
    } else {
      k_ionsite<false><<<nb, kPairThreads, smem, stream>>>(p, qforces, slot);
      if (qforces) k_siteforce<false><<<p.nsites, kPairThreads, 0, stream>>>(p);
    }
    slot += nb;
    nk += qforces ? 2 : 1;
  }
  if ((mask & 16u) && p.qrfpar && nub > p.nsites && plan.nchunk_rf > 0) {
    dim3 g((nub - p.nsites + kPairThreads - 1) / kPairThreads, plan.nchunk_rf);
    if (plan.t_rf) cudaEventRecord(plan.t_rf->a, stream);
    if (plan.fp32)
      k_rfcross32<<<g, kPairThreads, 0, stream>>>(p, qforces, slot);
    else
      k_rfcross<false><<<g, kPairThreads, 0, stream>>>(p, qforces, slot);
    if (plan.t_rf) cudaEventRecord(plan.t_rf->b, stream);
    slot += g.x * g.y;
    ++nk;
  }
  if (plan.reduce_energy) {
    k_ereduce<<<1, 256, 0, stream>>>(p, slot, (mask & 16u) && p.qrfpar);
    ++nk;
  }
  return nk;  // kernels launched
}

int energy_slots(const KP &p, const EnergyPlan &plan, uint32_t mask) {
  const int nub = plan.ntot_ub;
  int slot = fields_blocks(nub);
  const int nmob_ub = nub - p.nsites - p.nfix;
  if ((mask & 1u) && nmob_ub > 0 && plan.nchunk_ii > 0)
    slot += ((nmob_ub + kPairThreads - 1) / kPairThreads) * plan.nchunk_ii;
  if ((mask & 1u) && p.nsites > 0 && nub > p.nsites)
    slot += (nub - p.nsites + kPairThreads - 1) / kPairThreads;
  if ((mask & 16u) && p.qrfpar && nub > p.nsites && plan.nchunk_rf > 0)
    slot += ((nub - p.nsites + kPairThreads - 1) / kPairThreads) * plan.nchunk_rf;
  return slot;
}

}  // namespace bgpu
