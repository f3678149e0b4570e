// DNA bonded and Go-like terms between interaction sites
// (energy.mono.f90:196-582; INTERACT of a site, interact.f90:211-334).
//
// The terms form one list in kind order (NucDev).  A step runs:
//   k_nucl_terms   one thread per term: its energy, and its force on each of
//                  its (up to four) sites, each into its own slot, in FP64
//                  from the FP64 coordinates or the float-float records;
//   k_nucl_reduce  one block: per-kind energy sums in a fixed tree, the
//                  CONTRANS centre sums and spring forces, one energy slot;
//   k_nucl_gather  one warp per site: the site's term slots in ascending term
//                  order (lanes stride, a fixed shuffle tree), APFOR, CONTRANS,
//                  added to (or written into) the site's ion-site force.
// No atomics: every sum has one order, so a run repeats bit for bit.
// The site counts this serves are a few hundred; the work is latency, not
// bandwidth (a few thousand terms of ~100 FP64 operations).
#include "launch.h"
#include "physics.cuh"

namespace bgpu {

constexpr int kNucThreads = 128;
constexpr int kNucReduceThreads = 256;
constexpr int kNucGatherWarps = 4;

template <bool F32>
__device__ __forceinline__ void site_pos(const KP &p, int i, double r[3]) {
  if (F32) {
    const float4 h = p.pk1[i], l = p.pk2[i];
    r[0] = (double)h.x + (double)l.x;
    r[1] = (double)h.y + (double)l.y;
    r[2] = (double)h.z + (double)l.z;
  } else {
    r[0] = p.x[i];
    r[1] = p.y[i];
    r[2] = p.z[i];
  }
}

// grandmod.f90:74-98
__device__ __forceinline__ bool outbox(const KP &p, const double r[3]) {
  if (p.shape == 1)
    return (r[0] - p.cx) * (r[0] - p.cx) + (r[1] - p.cy) * (r[1] - p.cy) +
               (r[2] - p.cz) * (r[2] - p.cz) > p.rsphe2;
  if (p.shape == 2) {
    const double u = (r[0] - p.cx) * p.iecx, v = (r[1] - p.cy) * p.iecy;
    return u * u + v * v > 1.0 || r[2] < p.lz2m || r[2] > p.lz2p;
  }
  return r[0] < p.lx2m || r[0] > p.lx2p || r[1] < p.ly2m || r[1] > p.ly2p || r[2] < p.lz2m ||
         r[2] > p.lz2p;
}

__device__ __forceinline__ int nuc_kind(const NucDev &n, int t) {
  int k = 0;
#pragma unroll
  for (int m = 1; m < kNucKinds; ++m) k += t >= n.off[m];
  return k;
}

__device__ __forceinline__ double dot3(const double a[3], const double b[3]) {
  return a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
}

// One term: energy e and the forces f[m] on its sites (zero where the kind
// has fewer sites).  Pair kinds: v1 = r2 - r1, F1 = -de v1, F2 = +de v1.
template <bool F32>
__device__ void nucl_term(const KP &p, uint32_t mask, int t, int kind, double &e,
                          double f[4][3]) {
  const NucDev &n = p.nuc;
  const int4 s = n.site[t];
  const double eps = n.epsnuc;
  e = 0.0;
#pragma unroll
  for (int m = 0; m < 4; ++m) f[m][0] = f[m][1] = f[m][2] = 0.0;
  if (kind <= 2 && !(mask & 32u)) return;                 // Qnobond
  if (kind >= 3 && kind <= 7 && !(mask & 1u)) return;     // Qnonbond
  if (kind == 7 && !n.qsolv) return;
  if (kind == 8) {  // APFOR (energy.mono.f90:506-515)
    const int k = t - n.off[8];
    f[0][0] = n.af[3 * k];
    f[0][1] = n.af[3 * k + 1];
    f[0][2] = n.af[3 * k + 2];
    return;
  }
  double r1[3], r2[3];
  site_pos<F32>(p, s.x, r1);
  site_pos<F32>(p, s.y, r2);
  const double par = n.par[t];
  if (kind == 0) {  // bond stretch :205-230
    const double v1[3] = {r2[0] - r1[0], r2[1] - r1[1], r2[2] - r1[2]};
    const double dist = sqrt(dot3(v1, v1));
    const double vard = dist - par, vard2 = vard * vard;
    e = eps * vard2 * (1.0 + 100.0 * vard2);
    const double de = eps * vard * (2.0 + 400.0 * vard2) / dist;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      f[0][c] = de * v1[c];
      f[1][c] = -de * v1[c];
    }
    return;
  }
  if (kind == 1) {  // bond angle :234-276, vertex r2
    double r3[3];
    site_pos<F32>(p, s.z, r3);
    const double v1[3] = {r1[0] - r2[0], r1[1] - r2[1], r1[2] - r2[2]};
    const double v2[3] = {r3[0] - r2[0], r3[1] - r2[1], r3[2] - r2[2]};
    const double m1 = dot3(v1, v1), m2 = dot3(v2, v2), m3 = dot3(v1, v2);
    const double modval = 1.0 / sqrt(m1 * m2);
    const double ang = acos(m3 * modval);
    const double varang = ang - par;
    e = 700.0 * eps * (varang * varang);
    const double de = 1400.0 * eps * varang * modval / sin(ang);
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      f[0][c] = de * v2[c];
      f[1][c] = -(de * v1[c] + de * v2[c]);
      f[2][c] = de * v1[c];
    }
    return;
  }
  if (kind == 2) {  // torsion :279-336
    double r3[3], r4[3];
    site_pos<F32>(p, s.z, r3);
    site_pos<F32>(p, s.w, r4);
    const double v1[3] = {r1[0] - r2[0], r1[1] - r2[1], r1[2] - r2[2]};
    const double v2[3] = {r3[0] - r2[0], r3[1] - r2[1], r3[2] - r2[2]};
    const double v3[3] = {r3[0] - r4[0], r3[1] - r4[1], r3[2] - r4[2]};
    const double n1[3] = {v1[1] * v2[2] - v1[2] * v2[1], v1[2] * v2[0] - v1[0] * v2[2],
                          v1[0] * v2[1] - v1[1] * v2[0]};
    const double n2[3] = {v2[1] * v3[2] - v2[2] * v3[1], v2[2] * v3[0] - v2[0] * v3[2],
                          v2[0] * v3[1] - v2[1] * v3[0]};
    const double v22 = dot3(v2, v2), v2v = sqrt(v22);
    const double dihe = atan2(v2v * dot3(v1, n2), dot3(n1, n2));
    const double vardihe = dihe - par;
    e = 28.0 * eps * (1.0 - cos(vardihe));
    const double n1v = dot3(n1, n1), n2v = dot3(n2, n2);
    const double de = 28.0 * eps * sin(vardihe) * v2v;
    const double iv22 = 1.0 / v22;
    const double v12 = dot3(v1, v2) * iv22, v23 = dot3(v2, v3) * iv22;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const double f1 = -de / n1v * n1[c], f4 = de / n2v * n2[c];
      f[0][c] = f1;
      f[1][c] = -f1 + v12 * f1 - v23 * f4;
      f[2][c] = -f4 - v12 * f1 + v23 * f4;
      f[3][c] = f4;
    }
    return;
  }
  // pair kinds
  const double v1[3] = {r2[0] - r1[0], r2[1] - r1[1], r2[2] - r1[2]};
  const double dist2 = dot3(v1, v1);
  double de = 0.0;
  if (kind == 3) {  // stacking :341-366
    const double idist2 = 1.0 / dist2;
    const double c = par * par * idist2, cte1 = c * c * c;
    e = 4.0 * eps * cte1 * (cte1 - 1.0);
    de = 24.0 * eps * cte1 * (2.0 * cte1 - 1.0) * idist2;
  } else if (kind == 4) {  // base pairs :368-397
    const double epsln = s.z ? 2.532 * eps * n.scalepairing : 2.0 * eps * n.scalepairing;
    const double idist2 = 1.0 / dist2;
    const double cte1 = par * par * idist2;
    const double c5 = cte1 * cte1 * cte1 * cte1 * cte1;
    e = epsln * c5 * (20.0 * cte1 - 24.0);
    de = 240.0 * epsln * c5 * (cte1 - 1.0) * idist2;
  } else if (kind == 5) {  // excluded volume :399-426
    const double sgex2 = par * par;
    if (dist2 < sgex2) {
      const double idist2 = 1.0 / dist2;
      const double c = sgex2 * idist2, cte1 = c * c * c;
      e = 4.0 * eps * cte1 * (cte1 - 1.0) + eps;
      de = 24.0 * eps * cte1 * (2.0 * cte1 - 1.0) * idist2;
    }
  } else if (kind == 6) {  // P-P electrostatics :428-479
    const double dist = sqrt(dist2), idist = 1.0 / dist;
    bool deby = n.qdeby == 1;
    if (n.qdeby == 2) deby = outbox(p, r1) && outbox(p, r2);
    if (deby) {
      const double idistkd = exp(-dist * n.ikappa);
      e = n.fctn * idist * idistkd;
      de = n.fctn * (dist + n.kappa) * (idist * idist * idist) * n.ikappa * idistkd;
    } else {
      e = n.fctn * idist;
      de = n.fctn * (idist * idist * idist);
    }
  } else {  // solvent-induced :481-503
    const double dist = sqrt(dist2);
    const double cte1 = exp((13.38 - dist) * 0.1875);
    e = n.epsolv * ((1.0 - cte1) * (1.0 - cte1)) - n.epsolv;
    de = 0.375 * n.epsolv * cte1 * (cte1 - 1.0) / dist;
  }
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    f[0][c] = -de * v1[c];
    f[1][c] = de * v1[c];
  }
}

// One thread per term; the block's energies per kind (a fixed tree) into
// energy slot slot0 + block.
template <bool F32>
__global__ void __launch_bounds__(kNucThreads)
    k_nucl_terms(KP p, uint32_t mask, int qforces, int slot0) {
  const NucDev &n = p.nuc;
  __shared__ double red[(kNucThreads / 32) * 8];
  __shared__ double tot[8];
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  double v[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  if (t < n.nterm) {
    double e, f[4][3];
    const int kind = nuc_kind(n, t);
    nucl_term<F32>(p, mask, t, kind, e, f);
#pragma unroll
    for (int k = 0; k < 8; ++k) v[k] = kind == k ? e : 0.0;
    if (qforces) {
      double *o = n.tf + (size_t)t * 12;
#pragma unroll
      for (int m = 0; m < 4; ++m)
#pragma unroll
        for (int c = 0; c < 3; ++c) o[3 * m + c] = f[m][c];
    }
  }
  block_sum<8>(v, red, tot);
  if (threadIdx.x == 0) {
    double *dst = p.epart + (size_t)(slot0 + blockIdx.x) * kNTerms;
    for (int k = 0; k < kNTerms; ++k) dst[k] = 0.0;
    for (int k = 0; k < 8; ++k) dst[14 + k] = tot[k];
  }
}

// CONTRANS (energy.mono.f90:516-581): centre sums of the site coordinates
// (per strand when unsplit), the centre springs' force per strand and axis
// into n.cf[0..5], econ into one energy slot.
template <bool F32>
__global__ void __launch_bounds__(kNucReduceThreads) k_nucl_reduce(KP p, int slot) {
  const NucDev &n = p.nuc;
  __shared__ double red[(kNucReduceThreads / 32) * 6];
  __shared__ double tot6[6];
  double v[6] = {0, 0, 0, 0, 0, 0};
  const int ns = p.nsites, n1 = n.qunsplit ? n.nsites1st : ns;
  for (int j = threadIdx.x; j < ns; j += blockDim.x) {
    double r[3];
    site_pos<F32>(p, j, r);
    const int b = j < n1 ? 0 : 3;
#pragma unroll
    for (int c = 0; c < 3; ++c) v[b + c] += r[c];
  }
  block_sum<6>(v, red, tot6);  // first strand (or all sites) xyz, second strand xyz
  if (threadIdx.x != 0) return;
  const double insites = 1.0 / ns;
  const int ctn = n.ctn;
  double cf[6] = {0, 0, 0, 0, 0, 0}, econ = 0.0;
  for (int i = 0; i < ctn; ++i) {
    const int j = n.csn[i];
    for (int a = 0; a < 3; ++a) {
      const double kv = n.ck[3 * i + a];
      if (kv == 0.0) continue;
      const double *c = n.cc + 3 * 0 + a;  // anchors: cc[3*entry + axis]
      if (j == 0) {
        if (n.qunsplit) {
          double con = tot6[a] * insites * 2.0 - c[3 * i];
          cf[a] -= kv * con * insites * 2.0;
          econ = econ + 0.5 * kv * (con * con);
          con = tot6[3 + a] * insites * 2.0 - c[3 * ctn];
          cf[3 + a] -= kv * con * insites * 2.0;
          econ = econ + 0.5 * kv * (con * con);
        } else {
          const double con = tot6[a] * insites - c[3 * i];
          cf[a] -= kv * con * insites;
          econ = econ + 0.5 * kv * (con * con);
        }
      } else {
        double r[3];
        site_pos<F32>(p, j - 1, r);
        const double d = r[a] - c[3 * i];
        econ = econ + 0.5 * kv * (d * d);
      }
    }
  }
  for (int k = 0; k < 6; ++k) n.cf[k] = cf[k];
  double *dst = p.epart + (size_t)slot * kNTerms;
  for (int k = 0; k < kNTerms; ++k) dst[k] = 0.0;
  dst[22] = econ;
}

// One warp per site; lanes take every 32nd entry of the site's list and a
// fixed shuffle tree joins them.
template <bool F32>
__global__ void __launch_bounds__(32 * kNucGatherWarps) k_nucl_gather(KP p, int accum) {
  const NucDev &n = p.nuc;
  const int j = blockIdx.x * kNucGatherWarps + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (j >= p.nsites) return;  // warp-uniform
  double f[3] = {0.0, 0.0, 0.0};
  if (p.stfree[j])
    for (int e = n.csr_start[j] + lane; e < n.csr_start[j + 1]; e += 32) {
      const double *src = n.tf + (size_t)n.csr_ent[e] * 3;
#pragma unroll
      for (int c = 0; c < 3; ++c) f[c] += src[c];
    }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1)
#pragma unroll
    for (int c = 0; c < 3; ++c) f[c] += __shfl_xor_sync(0xffffffffu, f[c], o);
  if (lane != 0) return;
  // CONTRANS on every site, free or not (energy.mono.f90:516-581)
  if (n.ctn > 0) {
    const int b = (n.qunsplit && j >= n.nsites1st) ? 3 : 0;
    double r[3];
    site_pos<F32>(p, j, r);
#pragma unroll
    for (int c = 0; c < 3; ++c) f[c] += n.cf[b + c];
    for (int i = 0; i < n.ctn; ++i) {
      if (n.csn[i] != j + 1) continue;
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const double kv = n.ck[3 * i + c];
        if (kv != 0.0) f[c] -= kv * (r[c] - n.cc[3 * i + c]);
      }
    }
  }
  const int cap = p.cap;
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    if (F32) {
      float *o = p.fis_f + c * cap + j;
      *o = accum ? (float)((double)*o + f[c]) : (float)f[c];
    } else {
      double *o = p.fis + c * cap + j;
      *o = accum ? *o + f[c] : f[c];
    }
  }
}

// INTERACT of site j (interact.f90:211-334): the terms that involve j at the
// stored positions, added to *dener.  The angle and torsion are formed as
// angbond.f90 and angdih.f90 do; base pairs without the pairing scale.
__global__ void __launch_bounds__(kNucReduceThreads)
    k_nucl_interact(KP p, uint32_t mask, int j, double *dener) {
  const NucDev &n = p.nuc;
  __shared__ double red[kNucReduceThreads / 32];
  __shared__ double tot[1];
  const double eps = n.epsnuc;
  double acc[1] = {0.0};
  for (int t = threadIdx.x; t < n.off[8]; t += blockDim.x) {
    const int kind = nuc_kind(n, t);
    const int4 s = n.site[t];
    const bool mine = s.x == j || s.y == j || (kind <= 2 && (s.z == j || (kind == 2 && s.w == j)));
    if (!mine) continue;
    if (kind <= 2 && !(mask & 32u)) continue;
    if (kind >= 3 && !(mask & 1u)) continue;
    if (kind == 7 && !n.qsolv) continue;
    double r1[3], r2[3];
    site_pos<false>(p, s.x, r1);
    site_pos<false>(p, s.y, r2);
    const double par = n.par[t];
    double e = 0.0;
    if (kind == 0) {
      const double d[3] = {r1[0] - r2[0], r1[1] - r2[1], r1[2] - r2[2]};
      const double vard = sqrt(dot3(d, d)) - par;
      e = eps * (vard * vard) * (1.0 + 100.0 * (vard * vard));
    } else if (kind == 1) {
      double r3[3];
      site_pos<false>(p, s.z, r3);
      const double a[3] = {r1[0] - r2[0], r1[1] - r2[1], r1[2] - r2[2]};
      const double b[3] = {r3[0] - r2[0], r3[1] - r2[1], r3[2] - r2[2]};
      const double ang = acos(dot3(a, b) / (sqrt(dot3(a, a)) * sqrt(dot3(b, b))));
      const double varang = ang - par;
      e = 700.0 * eps * (varang * varang);
    } else if (kind == 2) {
      double r3[3], r4[3];
      site_pos<false>(p, s.z, r3);
      site_pos<false>(p, s.w, r4);
      const double a[3] = {r2[0] - r1[0], r2[1] - r1[1], r2[2] - r1[2]};
      const double b[3] = {r3[0] - r2[0], r3[1] - r2[1], r3[2] - r2[2]};
      const double c[3] = {r4[0] - r3[0], r4[1] - r3[1], r4[2] - r3[2]};
      const double n1[3] = {a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2],
                            a[0] * b[1] - a[1] * b[0]};
      const double n2[3] = {b[1] * c[2] - b[2] * c[1], b[2] * c[0] - b[0] * c[2],
                            b[0] * c[1] - b[1] * c[0]};
      const double dihe = atan2(sqrt(dot3(b, b)) * dot3(a, n2), dot3(n1, n2));
      e = 28.0 * eps * (1.0 - cos(dihe - par));
    } else {
      const double d[3] = {r2[0] - r1[0], r2[1] - r1[1], r2[2] - r1[2]};
      const double dist2 = dot3(d, d);
      if (kind == 3) {
        const double c = par * par / dist2, cte1 = c * c * c;
        e = 4.0 * eps * cte1 * (cte1 - 1.0);
      } else if (kind == 4) {
        const double epsln = s.z ? 2.532 * eps : 2.0 * eps;
        const double cte1 = par * par / dist2;
        e = epsln * (cte1 * cte1 * cte1 * cte1 * cte1) * (20.0 * cte1 - 24.0);
      } else if (kind == 5) {
        const double sgex2 = par * par;
        if (dist2 < sgex2) {
          const double c = sgex2 / dist2, cte1 = c * c * c;
          e = 4.0 * eps * cte1 * (cte1 - 1.0) + eps;
        }
      } else if (kind == 6) {
        const double dist = sqrt(dist2), idist = 1.0 / dist;
        bool deby = n.qdeby == 1;
        if (n.qdeby == 2) deby = outbox(p, r1) && outbox(p, r2);
        e = deby ? n.fctn * idist * exp(-dist * n.ikappa) : n.fctn * idist;
      } else {
        const double cte1 = exp((13.38 - sqrt(dist2)) * 0.1875);
        e = n.epsolv * ((1.0 - cte1) * (1.0 - cte1)) - n.epsolv;
      }
    }
    acc[0] += e;
  }
  block_sum<1>(acc, red, tot);
  if (threadIdx.x == 0) *dener += tot[0];
}

// NOTRAN (simul1.f90:380-385): x(1:nsites) = x(1:nsites) - sum(x)*insites
// + notrx per flagged axis, after the move; the sum as a fixed tree in FP64.
template <bool F32>
__global__ void __launch_bounds__(kNucReduceThreads) k_notrans(KP p) {
  const NucDev &n = p.nuc;
  __shared__ double red[(kNucReduceThreads / 32) * 3];
  __shared__ double tot[3];
  const int ns = p.nsites;
  double v[3] = {0.0, 0.0, 0.0};
  for (int j = threadIdx.x; j < ns; j += blockDim.x) {
    double r[3];
    site_pos<F32>(p, j, r);
#pragma unroll
    for (int c = 0; c < 3; ++c) v[c] += r[c];
  }
  block_sum<3>(v, red, tot);
  const double insites = 1.0 / ns;
  for (int j = threadIdx.x; j < ns; j += blockDim.x) {
    double r[3];
    site_pos<F32>(p, j, r);
#pragma unroll
    for (int c = 0; c < 3; ++c)
      if (n.qnotr[c]) r[c] = r[c] - tot[c] * insites + n.notr[c];
    if (F32) {
      float4 h = p.pk1[j], l = p.pk2[j];
      float *hc[3] = {&h.x, &h.y, &h.z}, *lc[3] = {&l.x, &l.y, &l.z};
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        if (!n.qnotr[c]) continue;
        *hc[c] = __double2float_rn(r[c]);
        *lc[c] = __double2float_rn(r[c] - (double)*hc[c]);
      }
      p.pk1[j] = h;
      p.pk2[j] = l;
    } else {
      if (n.qnotr[0]) p.x[j] = r[0];
      if (n.qnotr[1]) p.y[j] = r[1];
      if (n.qnotr[2]) p.z[j] = r[2];
    }
  }
}

int launch_notrans(const KP &p, bool fp32, cudaStream_t stream) {
  const NucDev &n = p.nuc;
  if (p.nsites <= 0 || !(n.qnotr[0] || n.qnotr[1] || n.qnotr[2])) return 0;
  (fp32 ? k_notrans<true> : k_notrans<false>)<<<1, kNucReduceThreads, 0, stream>>>(p);
  return 1;
}

// Energy slots of the DNA terms: one per term block, one for CONTRANS.
int nucl_slots(const KP &p) {
  const NucDev &n = p.nuc;
  return (n.nterm + kNucThreads - 1) / kNucThreads + (n.ctn > 0 ? 1 : 0);
}

int launch_nucl(const KP &p, bool fp32, uint32_t mask, int qforces, int accum, int slot,
                cudaStream_t stream) {
  const NucDev &n = p.nuc;
  if (n.nterm <= 0 && n.ctn <= 0) return 0;
  int nk = 0;
  const int nb = (n.nterm + kNucThreads - 1) / kNucThreads;
  if (nb > 0) {
    (fp32 ? k_nucl_terms<true> : k_nucl_terms<false>)<<<nb, kNucThreads, 0, stream>>>(
        p, mask, qforces, slot);
    ++nk;
  }
  if (n.ctn > 0) {
    (fp32 ? k_nucl_reduce<true> : k_nucl_reduce<false>)<<<1, kNucReduceThreads, 0, stream>>>(
        p, slot + nb);
    ++nk;
  }
  if (qforces) {
    const int nb = (p.nsites + kNucGatherWarps - 1) / kNucGatherWarps;
    (fp32 ? k_nucl_gather<true> : k_nucl_gather<false>)<<<nb, 32 * kNucGatherWarps, 0,
                                                         stream>>>(p, accum);
    ++nk;
  }
  return nk;
}

void launch_nucl_interact(const KP &p, uint32_t mask, int j, double *dener,
                          cudaStream_t stream) {
  if (p.nuc.off[8] <= 0) return;
  k_nucl_interact<<<1, kNucReduceThreads, 0, stream>>>(p, mask, j, dener);
}

}  // namespace bgpu
