// ENERGY on the device (energy.mono.f90:19-692 without the DNA bonded
// terms).  One launch per term family; partial forces and block-partial
// energies go to scratch and are reduced in a fixed order, so a run is
// bit-reproducible.
#include "ff.cuh"
#include "launch.h"
#include "physics.cuh"
#include "pairs_n3.cuh"

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
        double dx = xt - sx[k], dy = yt - sy[k], dz = zt - sz[k];
        if (p.periodic) {  // extension mode: nearest image, plain cutoff
          dx -= p.lx * rint(dx / p.lx);
          dy -= p.ly * rint(dy / p.ly);
          dz -= p.lz * rint(dz / p.lz);
        }
        const double d2 = dx * dx + dy * dy + dz * dz;
        if (p.periodic && d2 >= p.rc2) continue;
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

// ---------------------------------------------------------------------------
// FP32 pair kernel: ion-ion laws and the RFPAR cross term in one pass over
// (target, source) pairs.  Block (tx, cy): 64 targets x source chunk cy;
// sources staged in shared memory from the float-float records (pk1 hi +
// code, pk2 lo + srfe, pk3 reff/charge/flags).  No double-precision
// instruction: dx = (hi_t - hi_s) + (lo_t - lo_s); forces and energies
// accumulate in FP32 within the chunk and leave as FP32 partials (fii_f).
//
//   ion-ion (II): mobile targets against every other ion; weight 1/2 for a
//     mobile source (the pair is summed by both), 1 for a fixed one.  With
//     a dense type table (!EFP) the law is branch-free Coulomb + LJ (absent
//     terms have zero coefficients) plus the SRPMF branch inside rth.
//   RFPAR (RF): pair i = max(t, s), j = min: counts when i is mobile and in
//     the map and srfe(j) != 0 (rfpar.f90:177-223); the energy is added by
//     the target playing i; F_t = A sd1_t + B sd2_t + sum pr (r_t - r_s),
//     the last sum folded into the per-pair radial factor.
// ---------------------------------------------------------------------------
template <bool II, bool RF, bool EFP>
__global__ void __launch_bounds__(kPairThreads)
    k_pairs32(KP p, int qforces, int slot0, int t0) {
  __shared__ float4 sh[kPairThreads], sl[kPairThreads], sq[RF ? kPairThreads : 1];
  __shared__ float4 tab[EFP ? 1 : kIpqMax];
  __shared__ float red[(kPairThreads / 32) * 5];
  __shared__ float tot[5];
  const int nt = p.nion_t;
  if (II && !EFP)
    for (int k = threadIdx.x; k < nt * ipq_stride(nt); k += blockDim.x) tab[k] = __ldg(p.ipq + k);
  const int ntot = p.st->ntot;
  const int m0 = p.nsites + p.nfix;
  const int t = t0 + blockIdx.x * kPairThreads + threadIdx.x;
  float4 th = make_float4(0.f, 0.f, 0.f, 0.f), tl = th, tq = th;
  int row = 0, tb = 0;
  if (t < ntot) {
    th = p.pk1[t];
    tl = p.pk2[t];
    if (RF) tq = p.pk3[t];
    tb = __float_as_int(tq.z);
    const int code = __float_as_int(th.w) & 0xffff;
    row = EFP ? code * p.nttyp : (code - p.ndna) * ipq_stride(nt);
  }
  const bool tmob = II && t < ntot && t >= m0;
  const bool trf = RF && t < ntot && (tb & 1);
  const float srt = tl.w, rft = tq.x, ct = p.f.celec * tq.y;
  const int s0 = p.nsites + blockIdx.y * p.chunk_ii;
  const int s1 = min(ntot, s0 + p.chunk_ii);
  float fx = 0.f, fy = 0.f, fz = 0.f, A = 0.f, B = 0.f;
  float e[5] = {0.f, 0.f, 0.f, 0.f, 0.f};  // ecoul, elj, esrpmf, eefpot, erfpar
  for (int base = s0; base < s1; base += kPairThreads) {
    const int s = base + threadIdx.x;
    __syncthreads();
    if (s < s1) {
      sh[threadIdx.x] = p.pk1[s];
      sl[threadIdx.x] = p.pk2[s];
      if (RF) sq[threadIdx.x] = p.pk3[s];
    }
    __syncthreads();
    const int n = min(kPairThreads, s1 - base);
    if (tmob || trf) {
#pragma unroll 2
      for (int k = 0; k < n; ++k) {
        const int s = base + k;
        if (s == t) continue;
        const float4 h = sh[k], l = sl[k];
        const float dx = (th.x - h.x) + (tl.x - l.x);
        const float dy = (th.y - h.y) + (tl.y - l.y);
        const float dz = (th.z - h.z) + (tl.z - l.z);
        const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
        float de = 0.0f;
        if (II && tmob) {
          const int code = __float_as_int(h.w);
          const float w = (code >> 16) ? 0.5f : 1.0f;
          if (EFP) {
            de = law32k(p, __ldg(p.pidx + row + (code & 0xffff)), r2, w, e,
                        [&] { return r2_ff64(th, tl, h, l); });
          } else {
            const float4 q = tab[row + (code & 0xffff) - p.ndna];
            const float ir = rsqrtf(r2), ir2 = ir * ir;
            const float cofo = q.x * ir;
            e[0] = fmaf(w, cofo, e[0]);
            float d6 = q.z * ir2;
            d6 = d6 * d6 * d6;
            const float d12 = d6 * d6;
            e[1] = fmaf(w, q.y * (d12 - d6), e[1]);
            de = ir2 * fmaf(q.y, fmaf(2.0f, d12, -d6), cofo);
            if (r2 <= q.w)
              de += srpmf32(p, srp_index(p, __float_as_int(th.w), code), r2, ir, w, e,
                            srp_branch(p, r2, [&] { return r2_ff64(th, tl, h, l); }));
          }
        }
        if (RF && trf) {
          const float4 q = sq[k];
          const int sb = __float_as_int(q.z);
          const bool t_is_i = t > s;
          if (t_is_i ? ((tb & 4) && (sb & 8)) : ((sb & 4) && (tb & 8))) {
            const float rij = q.x * rft, srij = l.w * srt;
            const float rfdn = rsqrtf(fmaf(rij, rij, r2));
            const float aux0 = ct * q.y;
            const float a1 = aux0 * rij * rfdn;
            if (t_is_i) e[4] = fmaf(a1, srij, e[4]);
            const float a2 = aux0 * srij * rfdn * rfdn * rfdn;
            A = fmaf(-a1, l.w, A);
            B = fmaf(-a2 * fmaf(rij, 0.5f, r2), q.x, B);
            de = fmaf(a2, rij, de);
          }
        }
        fx = fmaf(de, dx, fx);
        fy = fmaf(de, dy, fy);
        fz = fmaf(de, dz, fz);
      }
    }
  }
  if (t < ntot) {
    float fo[3] = {0.f, 0.f, 0.f};
    if (qforces) {
      fo[0] = fx;
      fo[1] = fy;
      fo[2] = fz;
      if (trf) {
        const float4 d1 = p.rfd[2 * (size_t)t], d2 = p.rfd[2 * (size_t)t + 1];
        fo[0] = fmaf(A, d1.x, fmaf(B, d2.x, fo[0]));
        fo[1] = fmaf(A, d1.y, fmaf(B, d2.y, fo[1]));
        fo[2] = fmaf(A, d1.z, fmaf(B, d2.z, fo[2]));
      }
    }
    float *f = p.fii_f + (size_t)blockIdx.y * 3 * p.cap;
    f[t] = fo[0];
    f[p.cap + t] = fo[1];
    f[2 * p.cap + t] = fo[2];
  }
  block_sum_f<5>(e, red, tot);
  if (threadIdx.x == 0) {
    double *dst = p.epart + (size_t)(slot0 + blockIdx.y * gridDim.x + blockIdx.x) * kNTerms;
    for (int k = 0; k < kNTerms; ++k) dst[k] = 0.0;
    dst[1] = tot[0];
    dst[2] = EFP ? (double)tot[1] : (double)tot[1] / 6.0;  // dense table: 6 x elj
    dst[3] = tot[2];
    dst[4] = tot[3];
    dst[13] = tot[4];
  }
}

constexpr int kN3Warps = 4;

template <bool II, bool RF, bool EFP, bool PBC = false>
__global__ void __launch_bounds__(32 * kN3Warps)
    k_pairs32n(KP p, int qforces, int slot0, int rows) {
  __shared__ N3Warp<RF> nw[kN3Warps];
  __shared__ float4 tab[EFP ? 1 : kIpqMax];
  __shared__ float red[kN3Warps * 5];
  __shared__ float tot[5];
  const int nt = p.nion_t;
  if (II && !EFP)
    for (int k = threadIdx.x; k < nt * ipq_stride(nt); k += blockDim.x) tab[k] = __ldg(p.ipq + k);
  __syncthreads();
  const int w = threadIdx.x >> 5;
  const int T = p.ntile;
  const int it = blockIdx.x * kN3Warps + w;
  float e[5] = {0.f, 0.f, 0.f, 0.f, 0.f};  // ecoul, elj, esrpmf, eefpot, erfpar
  if (it < n3_work(T, rows))  // warp-uniform
    n3_tile<II, RF, EFP, PBC>(p, pair_sys(p, p.st->ntot, T, rows), it, qforces, nw[w], tab, e);
  block_sum_f<5>(e, red, tot);
  if (threadIdx.x == 0) {
    double *dst = p.epart + (size_t)(slot0 + blockIdx.x) * kNTerms;
    for (int k = 0; k < kNTerms; ++k) dst[k] = 0.0;
    dst[1] = tot[0];
    dst[2] = EFP ? (double)tot[1] : (double)tot[1] / 6.0;  // dense table: 6 x elj
    dst[3] = tot[2];
    dst[4] = tot[3];
    dst[13] = tot[4];
  }
}

int n3_rows(int T) {
  static int nsm[64] = {};
  int dev = 0;
  cudaGetDevice(&dev);
  if (!nsm[dev] &&
      cudaDeviceGetAttribute(&nsm[dev], cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    nsm[dev] = 1;
  return n3_pairs(T) > 16 * nsm[dev] ? 2 : 1;
}

int n3_blocks(int ntile) {
  return (n3_work(ntile, n3_rows(ntile)) + kN3Warps - 1) / kN3Warps;
}

// ---------------------------------------------------------------------------
// Ion-site pairs, ion-centred (energy.mono.f90:585-687): each ion walks the
// sites in order (which also reproduces the PROXDIFF nearest-site record,
// seeded by site 1 exactly as the reference).  Energies of all pairs, forces
// on mobile ions.  Sites are staged in shared memory (nsites <= 1024).
// ---------------------------------------------------------------------------
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
      double dist = 0.0;
      const double de = law64(p, p.pp[is], d2, 1.0, e, dist, err);
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
      double ed[4], dist;
      const double de = law64(p, p.pp[is], d2, 0.0, ed, dist, err);
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
// Ion-site pairs in FP32 from the float-float records: the ion-centred walk
// over the sites (energies, forces on ions, PROXDIFF record) and the
// site-centred force sum, as the FP64 kernels above.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kPairThreads)
    k_ionsite32(KP p, int qforces, int slot0) {
  extern __shared__ float4 smf[];
  float4 *sh = smf, *sl = smf + p.nsites;
  __shared__ float red[(kPairThreads / 32) * 4];
  __shared__ float tot[4];
  for (int k = threadIdx.x; k < p.nsites; k += blockDim.x) {
    sh[k] = p.pk1[k];
    sl[k] = p.pk2[k];
  }
  __syncthreads();
  const int ntot = p.st->ntot;
  const int i = p.nsites + blockIdx.x * blockDim.x + threadIdx.x;
  float e[4] = {0.f, 0.f, 0.f, 0.f};
  int err = 0;
  if (i < ntot) {
    const bool mobile = i >= p.nsites + p.nfix;
    const float4 th = p.pk1[i], tl = p.pk2[i];
    const int row = (__float_as_int(th.w) & 0xffff) * p.nttyp;
    float f[3] = {0.f, 0.f, 0.f}, dd[5] = {0.f, 0.f, 0.f, 0.f, 0.f};
    for (int j = 0; j < p.nsites; ++j) {
      const float4 h = sh[j], l = sl[j];
      const int is = p.pidx[row + (__float_as_int(h.w) & 0xffff)];
      const PairParamF &q = p.ppf[is];
      const float dx = ff_diff(th.x, tl.x, h.x, l.x), dy = ff_diff(th.y, tl.y, h.y, l.y),
                  dz = ff_diff(th.z, tl.z, h.z, l.z);
      const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
      const float de = law32(p, q, r2, 1.0f, e, err, [&] { return r2_ff64(th, tl, h, l); });
      if (p.qproxdiff && (q.flags & kEfp) && r2 >= q.dm2lo && r2 <= q.dm2hi) {
        const float dist = sqrtf(r2);
        const float dm = dist - q.dmi;
        if (dist > 0.0f && (j == 0 || dm < dd[0])) {
          dd[0] = dm;
          dd[1] = dist;
          dd[2] = dx;
          dd[3] = dy;
          dd[4] = dz;
        }
      }
      if (qforces && mobile) {
        f[0] = fmaf(de, dx, f[0]);
        f[1] = fmaf(de, dy, f[1]);
        f[2] = fmaf(de, dz, f[2]);
      }
    }
    p.fis_f[i] = f[0];
    p.fis_f[p.cap + i] = f[1];
    p.fis_f[2 * p.cap + i] = f[2];
    if (p.qproxdiff)
      for (int m = 0; m < 5; ++m) p.dids[5 * (size_t)i + m] = (double)dd[m];
  }
  if (err) atomicOr(&p.st->err, err);
  block_sum_f<4>(e, red, tot);
  if (threadIdx.x == 0) {
    double *dst = p.epart + (size_t)(slot0 + blockIdx.x) * kNTerms;
    for (int k = 0; k < kNTerms; ++k) dst[k] = 0.0;
    dst[5] = tot[0];
    dst[6] = tot[1];
    dst[7] = tot[2];
    dst[8] = tot[3];
  }
}

// Ion-site pairs as tiles: one warp per (ion tile of 32, site tile of
// kIsSiteTile), lane l holds ion 32 t + l and meets the tile's sites one
// after another (the same site on every lane: one broadcast read), keeping
// its term on each site in registers; each site's sum over the tile's ions
// is a fixed shuffle tree (no atomics).  Small site tiles give the warps of
// a few thousand ions against ~100 sites enough work items to fill the
// SMs.  The same per-pair law, energies and forces as k_ionsite32 /
// k_siteforce32 (the pair's r^2 and de are the same numbers on both sides);
// the PROXDIFF record keeps, per site tile, the smallest dist - mindist over
// sites j >= 1 (ties: the smaller j), and the first site's own record, which
// k_ionsite_sum combines in the reference's site order (energy.mono.f90:
// 603-621: site 1 seeds it, a later site replaces it only when smaller).
constexpr int kIsWarps = 4;

__global__ void __launch_bounds__(32 * kIsWarps)
    k_ionsite_tiles(KP p, int qforces, int slot0, int S, int nwork) {
  constexpr int W = kIsSiteTile;
  __shared__ float4 sh[kIsWarps][W], sl[kIsWarps][W];
  __shared__ float red[kIsWarps * 4];
  __shared__ float tot[4];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int wi = blockIdx.x * kIsWarps + w;
  const int ntot = p.st->ntot, ns = p.nsites;
  float e[4] = {0.f, 0.f, 0.f, 0.f};
  int err = 0;
  if (wi < nwork) {  // warp-uniform
    const int t = wi / S, s = wi - t * S;
    const int j0 = W * s, nj = min(W, ns - j0);
    if (lane < W) {
      const bool jv = lane < nj;
      sh[w][lane] = jv ? p.pk1[j0 + lane] : make_float4(0.f, 0.f, 0.f, 0.f);
      sl[w][lane] = jv ? p.pk2[j0 + lane] : make_float4(0.f, 0.f, 0.f, 0.f);
    }
    const int i = ns + 32 * t + lane;
    const bool iv = i < ntot;
    const bool mobile = i >= ns + p.nfix;
    float4 th = make_float4(0.f, 0.f, 0.f, 0.f), tl = th;
    if (iv) {
      th = p.pk1[i];
      tl = p.pk2[i];
    }
    const int row = (__float_as_int(th.w) & 0xffff) * p.nttyp;
    float f[3] = {0.f, 0.f, 0.f};
    float gs[3] = {0.f, 0.f, 0.f};  // lane k: site k's sum over the tile's ions
    float bv = 3.4e38f, bd = 0.f, bx = 0.f, by = 0.f, bz = 0.f;  // best j >= 1
    int bj = 1 << 30;
    float seed[5] = {0.f, 0.f, 0.f, 0.f, 0.f};
    __syncwarp();
#pragma unroll 1
    for (int k = 0; k < nj; ++k) {  // warp-uniform
      float g[3] = {0.f, 0.f, 0.f};  // this lane's term on site k
      if (iv) {
        const float4 h = sh[w][k], l = sl[w][k];  // the same site on every lane
        const int is = p.pidx[row + (__float_as_int(h.w) & 0xffff)];
        const PairParamF &q = p.ppf[is];
        const float dx = ff_diff(th.x, tl.x, h.x, l.x), dy = ff_diff(th.y, tl.y, h.y, l.y),
                    dz = ff_diff(th.z, tl.z, h.z, l.z);
        const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
        const float de = law32(p, q, r2, 1.0f, e, err, [&] { return r2_ff64(th, tl, h, l); });
        const int j = j0 + k;
        if (p.qproxdiff && (q.flags & kEfp) && r2 >= q.dm2lo && r2 <= q.dm2hi) {
          const float dist = sqrtf(r2);
          const float dm = dist - q.dmi;
          if (dist > 0.0f) {
            if (j == 0) {
              seed[0] = dm;
              seed[1] = dist;
              seed[2] = dx;
              seed[3] = dy;
              seed[4] = dz;
            } else if (dm < bv || (dm == bv && j < bj)) {
              bv = dm;
              bj = j;
              bd = dist;
              bx = dx;
              by = dy;
              bz = dz;
            }
          }
        }
        if (qforces && mobile) {
          f[0] = fmaf(de, dx, f[0]);
          f[1] = fmaf(de, dy, f[1]);
          f[2] = fmaf(de, dz, f[2]);
        }
        if (qforces && p.stfree[j]) {
          g[0] = -de * dx;
          g[1] = -de * dy;
          g[2] = -de * dz;
        }
      }
#pragma unroll
      for (int c = 0; c < 3; ++c) {  // a fixed shuffle tree over the ions
        float v = g[c];
#pragma unroll
        for (int x = 16; x > 0; x >>= 1) v += __shfl_xor_sync(0xffffffffu, v, x);
        if (lane == k) gs[c] = v;
      }
    }
    if (iv) {
      const size_t cap = p.cap;
      float *o = p.isp_ion + (size_t)s * 3 * cap;
      o[i] = f[0];
      o[cap + i] = f[1];
      o[2 * cap + i] = f[2];
      if (p.qproxdiff) {
        float *d = p.isp_dids + (size_t)s * 6 * cap;
        d[i] = bv;
        d[cap + i] = __int_as_float(bj);
        d[2 * cap + i] = bd;
        d[3 * cap + i] = bx;
        d[4 * cap + i] = by;
        d[5 * cap + i] = bz;
        if (s == 0)
          for (int c = 0; c < 5; ++c) p.isp_seed[c * cap + i] = seed[c];
      }
    }
    if (lane < nj) {
      float *o = p.isp_site + (size_t)t * 3 * ns;
#pragma unroll
      for (int c = 0; c < 3; ++c) o[c * ns + j0 + lane] = gs[c];
    }
  }
  if (err) atomicOr(&p.st->err, err);
  block_sum_f<4>(e, red, tot);
  if (threadIdx.x == 0) {
    double *dst = p.epart + (size_t)(slot0 + blockIdx.x) * kNTerms;
    for (int k = 0; k < kNTerms; ++k) dst[k] = 0.0;
    dst[5] = tot[0];
    dst[6] = tot[1];
    dst[7] = tot[2];
    dst[8] = tot[3];
  }
}

// Ion forces: the site tiles' partials in tile order; PROXDIFF: the first
// site's record, replaced by the smallest later one (smaller j on ties) only
// when it is below.
__global__ void __launch_bounds__(256) k_ionsite_sum(KP p, int qforces, int S, int T) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  const int ntot = p.st->ntot, ns = p.nsites;
  const size_t cap = p.cap;
  const int nion = ntot - ns;
  if (k < nion) {
    const int i = ns + k;
    float f[3] = {0.f, 0.f, 0.f};
    for (int s = 0; s < S; ++s) {
      const float *o = p.isp_ion + (size_t)s * 3 * cap;
#pragma unroll
      for (int c = 0; c < 3; ++c) f[c] += o[c * cap + i];
    }
#pragma unroll
    for (int c = 0; c < 3; ++c) p.fis_f[c * cap + i] = qforces ? f[c] : 0.f;
    if (p.qproxdiff) {
      float d[5];
      for (int c = 0; c < 5; ++c) d[c] = p.isp_seed[c * cap + i];
      float bv = 3.4e38f;
      int bj = 1 << 30, bs = -1;
      for (int s = 0; s < S; ++s) {
        const float *o = p.isp_dids + (size_t)s * 6 * cap;
        const float v = o[i];
        const int j = __float_as_int(o[cap + i]);
        if (v < bv || (v == bv && j < bj)) {
          bv = v;
          bj = j;
          bs = s;
        }
      }
      if (bs >= 0 && bv < d[0]) {
        const float *o = p.isp_dids + (size_t)bs * 6 * cap;
        d[0] = bv;
        d[1] = o[2 * cap + i];
        d[2] = o[3 * cap + i];
        d[3] = o[4 * cap + i];
        d[4] = o[5 * cap + i];
      }
      for (int c = 0; c < 5; ++c) p.dids[5 * (size_t)i + c] = (double)d[c];
    }
  }
}

// Site forces: one warp per site, lanes over the ion tiles (lane l takes
// tiles l, l + 32, ...), then a fixed shuffle tree.
__global__ void __launch_bounds__(256) k_ionsite_sites(KP p, int qforces, int T) {
  const int j = blockIdx.x * 8 + (threadIdx.x >> 5), lane = threadIdx.x & 31;
  const int ns = p.nsites;
  if (j >= ns) return;  // warp-uniform
  float f[3] = {0.f, 0.f, 0.f};
  if (qforces && p.stfree[j])
    for (int t = lane; t < T; t += 32) {
      const float *o = p.isp_site + (size_t)t * 3 * ns;
#pragma unroll
      for (int c = 0; c < 3; ++c) f[c] += o[c * ns + j];
    }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1)
#pragma unroll
    for (int c = 0; c < 3; ++c) f[c] += __shfl_xor_sync(0xffffffffu, f[c], o);
  if (lane == 0)
#pragma unroll
    for (int c = 0; c < 3; ++c) p.fis_f[c * (size_t)p.cap + j] = f[c];
}

int ionsite_tile_blocks(const KP &p, int nub) {
  const int S = (p.nsites + kIsSiteTile - 1) / kIsSiteTile;
  const int T = (std::max(0, nub - p.nsites) + 31) / 32;
  return (S * T + kIsWarps - 1) / kIsWarps;
}

// The FP32 ion-site pairs run as tiles when the context holds their partial
// buffers for this many ions.
bool ionsite_tiled(const KP &p, bool fp32, int nub) {
  return fp32 && p.isp_ion && (std::max(0, nub - p.nsites) + 31) / 32 <= p.isp_tcap;
}

__global__ void __launch_bounds__(kPairThreads) k_siteforce32(KP p) {
  __shared__ float red[(kPairThreads / 32) * 3];
  __shared__ float tot[3];
  const int j = blockIdx.x;
  const int ntot = p.st->ntot;
  float f[3] = {0.f, 0.f, 0.f};
  int err = 0;
  if (p.stfree[j]) {
    const float4 sh = p.pk1[j], sl = p.pk2[j];
    const int col = __float_as_int(sh.w) & 0xffff;
    for (int i = p.nsites + threadIdx.x; i < ntot; i += blockDim.x) {
      const float4 h = p.pk1[i], l = p.pk2[i];
      const int is = p.pidx[(__float_as_int(h.w) & 0xffff) * p.nttyp + col];
      const float dx = ff_diff(h.x, l.x, sh.x, sl.x), dy = ff_diff(h.y, l.y, sh.y, sl.y),
                  dz = ff_diff(h.z, l.z, sh.z, sl.z);
      const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
      float ef[4];
      const float de =
          law32(p, p.ppf[is], r2, 0.0f, ef, err, [&] { return r2_ff64(h, l, sh, sl); });
      f[0] = fmaf(-de, dx, f[0]);
      f[1] = fmaf(-de, dy, f[1]);
      f[2] = fmaf(-de, dz, f[2]);
    }
  }
  block_sum_f<3>(f, red, tot);
  if (threadIdx.x == 0) {
    p.fis_f[j] = tot[0];
    p.fis_f[p.cap + j] = tot[1];
    p.fis_f[2 * p.cap + j] = tot[2];
  }
}

// ---------------------------------------------------------------------------
// RFPAR cross term (rfpar.f90:177-223), target-centred over in-grid ions.
// Pair (i > j) counts when i is mobile and srfe(j) != 0; its energy is added
// by the target that plays i, each side adds its own force:
//   F_t = A sd1_t + B sd2_t + P,  A = sum -a1 srfe_s,  B = sum aux3 reff_s,
//   P = sum a2 reff_ts (r_t - r_s).
// ---------------------------------------------------------------------------
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
        double dx = xt - sx[k], dy = yt - sy[k], dz = zt - sz[k];
        if (p.periodic) {  // extension mode: nearest image, plain cutoff
          dx -= p.lx * rint(dx / p.lx);
          dy -= p.ly * rint(dy / p.ly);
          dz -= p.lz * rint(dz / p.lz);
        }
        const double d2 = dx * dx + dy * dy + dz * dz;
        if (p.periodic && d2 >= p.rc2) continue;
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
    // energy.mono.f90:65-115, 689: ememb, the MMIJ egsbpb (slot 11 of the
    // partials), egsbpa, evdwgd, erfpar, then ..., esrpmfmx, ebond .. esolv,
    // eqqmx, evdwmx, eefpot, eefpotmx, econ; RFPAR then reports
    // egsbpb = erfpar
    o[0] = o[9] + o[11] + o[10] + o[12] + o[13] + o[1] + o[2] + o[3] + o[7] + o[14] + o[15] +
           o[16] + o[17] + o[18] + o[19] + o[20] + o[21] + o[5] + o[6] + o[4] + o[8] + o[22];
    if (rfpar_on) o[11] = o[13];
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
  if (plan.mmij) {  // energy.mono.f90:71-79; forces added to the field forces
    nk += launch_mmij(p, plan.fp32, nub, qforces, slot, stream);
    ++slot;
  }
  const bool nonbond = (mask & 1u) != 0;
  const int nmob_ub = nub - p.nsites - p.nfix;
  const PairCfg32 pc = pair_cfg32(p, nub, mask);
  if (plan.fp32 && plan.cells) {
    if (plan.t_pairs) cudaEventRecord(plan.t_pairs->a, stream);
    nk += launch_cells(p, nub, qforces, slot, stream);
    if (plan.t_pairs) cudaEventRecord(plan.t_pairs->b, stream);
    slot += cell_pair_blocks(p, nub);
  } else if (plan.fp32 && plan.ntile > 0 && (pc.ii || pc.rf)) {
    const int nb = n3_blocks(plan.ntile), rows = n3_rows(plan.ntile);
    if (plan.t_pairs) cudaEventRecord(plan.t_pairs->a, stream);
    const bool efp = !p.ipq_ok;
    if (p.periodic)  // extension mode: ion-ion only (no RFPAR)
      (efp ? k_pairs32n<true, false, true, true> : k_pairs32n<true, false, false, true>)
          <<<nb, 32 * kN3Warps, 0, stream>>>(p, qforces, slot, rows);
    else if (pc.ii && pc.rf)
      (efp ? k_pairs32n<true, true, true> : k_pairs32n<true, true, false>)
          <<<nb, 32 * kN3Warps, 0, stream>>>(p, qforces, slot, rows);
    else if (pc.ii)
      (efp ? k_pairs32n<true, false, true> : k_pairs32n<true, false, false>)
          <<<nb, 32 * kN3Warps, 0, stream>>>(p, qforces, slot, rows);
    else
      k_pairs32n<false, true, true><<<nb, 32 * kN3Warps, 0, stream>>>(p, qforces, slot, rows);
    if (plan.t_pairs) cudaEventRecord(plan.t_pairs->b, stream);
    slot += nb;
    ++nk;
  } else if (plan.fp32 && pc.ntg > 0 && plan.nchunk_ii > 0) {
    dim3 g((pc.ntg + kPairThreads - 1) / kPairThreads, plan.nchunk_ii);
    if (plan.t_pairs) cudaEventRecord(plan.t_pairs->a, stream);
    const bool efp = !p.ipq_ok;
    if (pc.ii && pc.rf)
      (efp ? k_pairs32<true, true, true> : k_pairs32<true, true, false>)
          <<<g, kPairThreads, 0, stream>>>(p, qforces, slot, pc.t0);
    else if (pc.ii)
      (efp ? k_pairs32<true, false, true> : k_pairs32<true, false, false>)
          <<<g, kPairThreads, 0, stream>>>(p, qforces, slot, pc.t0);
    else
      k_pairs32<false, true, true><<<g, kPairThreads, 0, stream>>>(p, qforces, slot, pc.t0);
    if (plan.t_pairs) cudaEventRecord(plan.t_pairs->b, stream);
    slot += g.x * g.y;
    ++nk;
  }
  if (!plan.fp32 && nonbond && nmob_ub > 0 && plan.nchunk_ii > 0) {
    dim3 g((nmob_ub + kPairThreads - 1) / kPairThreads, plan.nchunk_ii);
    if (plan.t_pairs) cudaEventRecord(plan.t_pairs->a, stream);
    k_ionion64<<<g, kPairThreads, 0, stream>>>(p, qforces, slot);
    if (plan.t_pairs) cudaEventRecord(plan.t_pairs->b, stream);
    slot += g.x * g.y;
    ++nk;
  }
  if (nonbond && p.nsites > 0 && nub > p.nsites) {
    const int nion_ub = nub - p.nsites;
    const int nb = (nion_ub + kPairThreads - 1) / kPairThreads;
    if (ionsite_tiled(p, plan.fp32, nub)) {  // FP32: tiles of 32 ions x kIsSiteTile sites
      const int S = (p.nsites + kIsSiteTile - 1) / kIsSiteTile, T = (nion_ub + 31) / 32;
      const int tb = ionsite_tile_blocks(p, nub);
      k_ionsite_tiles<<<tb, 32 * kIsWarps, 0, stream>>>(p, qforces, slot, S, S * T);
      k_ionsite_sum<<<(nion_ub + 255) / 256, 256, 0, stream>>>(p, qforces, S, T);
      k_ionsite_sites<<<(p.nsites + 7) / 8, 256, 0, stream>>>(p, qforces, T);
      slot += tb;
      nk += 3;
    } else {
      if (plan.fp32) {
        const size_t smem = (size_t)p.nsites * 2 * sizeof(float4);
        k_ionsite32<<<nb, kPairThreads, smem, stream>>>(p, qforces, slot);
        if (qforces) k_siteforce32<<<p.nsites, kPairThreads, 0, stream>>>(p);
      } else {
        const size_t smem = (size_t)p.nsites * (3 * sizeof(double) + sizeof(int));
        k_ionsite<<<nb, kPairThreads, smem, stream>>>(p, qforces, slot);
        if (qforces) k_siteforce<<<p.nsites, kPairThreads, 0, stream>>>(p);
      }
      slot += nb;
      nk += qforces ? 2 : 1;
    }
  }
  if (plan.nuc) {  // DNA bonded and Go-like terms, after the ion-site forces
    const bool is_ran = nonbond && p.nsites > 0 && nub > p.nsites;
    if (qforces && !is_ran && nub > p.nsites)  // fis holds the site terms alone
      for (int k = 0; k < 3; ++k) {
        if (plan.fp32)
          cudaMemsetAsync(p.fis_f + (size_t)k * p.cap + p.nsites, 0,
                          (size_t)(nub - p.nsites) * sizeof(float), stream);
        else
          cudaMemsetAsync(p.fis + (size_t)k * p.cap + p.nsites, 0,
                          (size_t)(nub - p.nsites) * sizeof(double), stream);
      }
    nk += launch_nucl(p, plan.fp32, mask, qforces, is_ran ? 1 : 0, slot, stream);
    slot += nucl_slots(p);
  }
  if (!plan.fp32 && (mask & 16u) && p.qrfpar && nub > p.nsites && plan.nchunk_rf > 0) {
    dim3 g((nub - p.nsites + kPairThreads - 1) / kPairThreads, plan.nchunk_rf);
    if (plan.t_rf) cudaEventRecord(plan.t_rf->a, stream);
    k_rfcross<<<g, kPairThreads, 0, stream>>>(p, qforces, slot);
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
  if (plan.mmij) ++slot;
  const int nmob_ub = nub - p.nsites - p.nfix;
  if (plan.fp32) {
    const PairCfg32 pc = pair_cfg32(p, nub, mask);
    if (plan.cells)
      slot += cell_pair_blocks(p, nub);
    else if (plan.ntile > 0 && (pc.ii || pc.rf))
      slot += n3_blocks(plan.ntile);
    else if (pc.ntg > 0 && plan.nchunk_ii > 0)
      slot += ((pc.ntg + kPairThreads - 1) / kPairThreads) * plan.nchunk_ii;
  } else if ((mask & 1u) && nmob_ub > 0 && plan.nchunk_ii > 0) {
    slot += ((nmob_ub + kPairThreads - 1) / kPairThreads) * plan.nchunk_ii;
  }
  if ((mask & 1u) && p.nsites > 0 && nub > p.nsites)
    slot += ionsite_tiled(p, plan.fp32, nub) ? ionsite_tile_blocks(p, nub)
                                              : (nub - p.nsites + kPairThreads - 1) / kPairThreads;
  if (plan.nuc) slot += nucl_slots(p);
  if (!plan.fp32 && (mask & 16u) && p.qrfpar && nub > p.nsites && plan.nchunk_rf > 0)
    slot += ((nub - p.nsites + kPairThreads - 1) / kPairThreads) * plan.nchunk_rf;
  return slot;
}

}  // namespace bgpu
