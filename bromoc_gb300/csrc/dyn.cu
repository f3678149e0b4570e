// Force assembly and the Ermak-McCammon BD update (dynamics0-3.mono.f90,
// dynamics0nuc.f90, fixcoor.f90, countions.f90), fused in one kernel: one
// warp per particle sums its partial forces in a fixed order, writes
// fx,fy,fz and, for a BD step, moves the particle with in-register Philox
// noise.
#include "ff.cuh"
#include "launch.h"
#include "physics.cuh"

namespace bgpu {

constexpr int kAsmWarps = 8;  // particles per assembly block

__device__ __forceinline__ void clamp_bd(double bdmax, double &d) {
  if (fabs(d) > bdmax) d = fsign(bdmax, d);
}

// fixcoor.f90:19-68
__device__ __forceinline__ void fixcoor(const KP &p, double &x, double &y,
                                        double &z) {
  if (p.shape == 1) {  // sphere: reflect through the wall
    const double r2 = (x - p.cx) * (x - p.cx) + (y - p.cy) * (y - p.cy) +
                      (z - p.cz) * (z - p.cz);
    if (r2 > p.rsphe2) {
      const double lzrad = 2.0 * p.rsphe / sqrt(r2) - 1.0;
      x = lzrad * (x - p.cx) + p.cx;
      y = lzrad * (y - p.cy) + p.cy;
      z = lzrad * (z - p.cz) + p.cz;
    }
  } else if (p.shape == 2) {  // elliptic cylinder
    const double ex = (x - p.cx) * p.iecx, ey = (y - p.cy) * p.iecy;
    const double r2 = ex * ex + ey * ey;
    if (r2 > 1.0) {
      const double r = 0.999999999999999 / sqrt(r2);
      x = r * (x - p.cx) + p.cx;
      y = r * (y - p.cy) + p.cy;
    }
    if (z < p.lz2m)
      z = p.lz2m;
    else if (z > p.lz2p)
      z = p.lz2p;
  } else {  // box: clamp
    if (x < p.lx2m)
      x = p.lx2m;
    else if (x > p.lx2p)
      x = p.lx2p;
    if (y < p.ly2m)
      y = p.ly2m;
    else if (y > p.ly2p)
      y = p.ly2p;
    if (z < p.lz2m)
      z = p.lz2m;
    else if (z > p.lz2p)
      z = p.lz2p;
  }
}

// Diffusion model of ion i at height zold: the drift and noise factors and
// the gradient drift dD (dynamics0-3.mono.f90).
__device__ __forceinline__ void diff_model(const KP &p, int variant, int i, int itype,
                                           double zold, double &fact1, double &fact2,
                                           double dD[3]) {
  dD[0] = dD[1] = dD[2] = 0.0;
  if (variant == 1) {  // dynamics1.mono.f90:39-72
    const double pp3 = p.p3[itype];
    const double pore1 = -p.plength2 + p.pcenter, pore2 = p.plength2 + p.pcenter;
    double sw, dsw;
    if (zold > pore1 - pp3 && zold < pore2 + pp3) {
      sw = 0.0;
      dsw = 0.0;
      if (!(zold >= pore1 && zold <= pore2)) {
        const double ipp3 = 1.0 / pp3;
        if (zold > pore2) {
          const double d = (zold - pore2) * ipp3;
          sw = 2.0 * d * d * d - 3.0 * d * d;
          dsw = 6.0 * (d * d - d) * ipp3;
        } else if (zold < pore1) {
          const double d = (zold - pore1) * ipp3;
          sw = -2.0 * d * d * d - 3.0 * d * d;
          dsw = -6.0 * (d * d + d) * ipp3;
        }
        sw = -sw;
        dsw = -dsw;
      }
    } else {
      sw = 1.0;
      dsw = 0.0;
    }
    const double D = p.diffusion[itype];
    const double idif = D * (p.ampl3[itype] + (1.0 - p.ampl3[itype]) * sw);
    const double didif = D * (1.0 - p.ampl3[itype]) * dsw;
    fact1 = idif * p.kbtdt;
    fact2 = sqrt(2.0 * p.dt * idif);
    dD[2] = didif * p.dt;
  } else if (variant == 2) {  // dynamics2.mono.f90:41-74
    const int n = p.nspline;
    double sw = 0.0, dsw = 0.0;
    bool inside = false;
    if (p.xs[1] < p.xs[n]) {
      if (zold < p.xs[1])
        sw = p.ys[1];
      else if (zold > p.xs[n])
        sw = p.ys[n];
      else
        inside = true;
    } else if (p.xs[1] > p.xs[n]) {
      if (zold > p.xs[1])
        sw = p.ys[1];
      else if (zold < p.xs[n])
        sw = p.ys[n];
      else
        inside = true;
    }
    if (inside) {  // sevalmod.f90 bisection
      int lo = 1, hi = n + 1;
      do {
        const int k = (lo + hi) / 2;
        if (zold < p.xs[k]) hi = k;
        if (zold >= p.xs[k]) lo = k;
      } while (hi > lo + 1);
      const double dx = zold - p.xs[lo];
      sw = p.ys[lo] + dx * (p.sb[lo] + dx * (p.scc[lo] + dx * p.sd[lo]));
      dsw = p.sb[lo] + dx * (p.scc[lo] + dx * p.sd[lo]);
    }
    const double D = p.diffusion[itype];
    const double idif = D * sw;
    fact1 = idif * p.kbtdt;
    fact2 = sqrt(2.0 * p.dt * idif);
    dD[2] = D * dsw * p.dt;
  } else if (variant == 3) {  // dynamics3.mono.f90:40-59
    const double *dd = p.dids + 5 * (size_t)i;
    if (dd[0] > 0.0 && dd[0] <= p.diffcutoff) {
      const double D = p.diffusion[itype];
      const double ebet = exp(-dd[0] * p.ibeta);
      const double idif = D - (D - p.diff0) * ebet;
      const double didif = (D - p.diff0) * p.ibeta * ebet;
      const double idist = 1.0 / dd[1];
      fact1 = idif * p.kbtdt;
      fact2 = sqrt(2.0 * p.dt * idif);
      dD[0] = didif * p.dt * dd[2] * idist;
      dD[1] = didif * p.dt * dd[3] * idist;
      dD[2] = didif * p.dt * dd[4] * idist;
    } else {
      fact1 = p.fact1a[itype];
      fact2 = p.fact2a[itype];
    }
  } else {  // dynamics0.mono.f90:31-46
    fact1 = p.fact1a[itype];
    fact2 = p.fact2a[itype];
  }
}

// countions.f90:25-31
__device__ __forceinline__ void count_crossings(const KP &p, int itype, double zold,
                                                double z) {
  const int it = itype - p.nold - 1;
  for (int j = 0; j < p.cntpts; ++j) {
    const double zc = p.zcont[j];
    if (zold < zc && z >= zc)
      atomicAdd(&p.nforward[it * p.cntpts + j], 1);
    else if (zold >= zc && z < zc)
      atomicAdd(&p.nbackward[it * p.cntpts + j], 1);
  }
}

// BD move of particle i under the assembled force f (dynamics*.f90), FP64.
__device__ __forceinline__ void bd_move(const KP &p, const AssembleFlags &fl,
                                        int variant, uint64_t seed,
                                        uint64_t step, int i, const double f[3]) {
  const int m0 = p.nsites + p.nfix;
  const uint32_t slot = (uint32_t)i;
  double g[3];
  if (i < m0 && (i >= p.nsites || !p.stfree[i])) return;  // fixed ions, frozen sites
  if (fl.fp32_noise) {
    float gf[3];
    bd_noise3_f(seed, step, slot, gf);
    g[0] = gf[0];
    g[1] = gf[1];
    g[2] = gf[2];
  } else {
    bd_noise3(seed, step, slot, g);
  }
  if (i < p.nsites) {  // dynamics0nuc.f90:31-44
    double dx = f[0] * p.fact0n1, dy = f[1] * p.fact0n1, dz = f[2] * p.fact0n1;
    clamp_bd(p.bdmax, dx);
    clamp_bd(p.bdmax, dy);
    clamp_bd(p.bdmax, dz);
    double x = p.x[i] + dx + p.fact0n2 * g[0];
    double y = p.y[i] + dy + p.fact0n2 * g[1];
    double z = p.z[i] + dz + p.fact0n2 * g[2];
    if (!p.qdnafree) fixcoor(p, x, y, z);
    p.x[i] = x;
    p.y[i] = y;
    p.z[i] = z;
    return;
  }
  const int itype = abs(p.typei[i]);
  const double zold = p.z[i];
  double fact1, fact2, dD[3];
  diff_model(p, variant, i, itype, zold, fact1, fact2, dD);
  double dx = f[0] * fact1, dy = f[1] * fact1, dz = f[2] * fact1;
  clamp_bd(p.bdmax, dx);
  clamp_bd(p.bdmax, dy);
  clamp_bd(p.bdmax, dz);
  double x = p.x[i] + dx + fact2 * g[0] + dD[0];
  double y = p.y[i] + dy + fact2 * g[1] + dD[1];
  double z = zold + dz + fact2 * g[2] + dD[2];
  if (p.qcountion) count_crossings(p, itype, zold, z);
  fixcoor(p, x, y, z);
  p.x[i] = x;
  p.y[i] = y;
  p.z[i] = z;
}

// One warp per particle: lane c adds chunk partials c, c+32, ...; a fixed
// shuffle tree sums the lanes, so the order is the same every run.
__global__ void __launch_bounds__(32 * kAsmWarps)
    k_assemble(KP p, AssembleFlags fl, int do_bd, int variant, uint64_t seed,
               uint64_t step) {
  const int i = blockIdx.x * kAsmWarps + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  const int ntot = p.st->ntot;
  if (i >= ntot) return;  // warp-uniform
  const int cap = p.cap;
  const int m0 = p.nsites + p.nfix;
  double v[3] = {0.0, 0.0, 0.0};
  if (fl.ii && i >= fl.ii_from)
    for (int c = lane; c < fl.nchunk_ii; c += 32)
#pragma unroll
      for (int k = 0; k < 3; ++k) v[k] += p.fii[((size_t)c * 3 + k) * cap + i];
  if (fl.rf && i >= p.nsites)
    for (int c = lane; c < fl.nchunk_rf; c += 32)
#pragma unroll
      for (int k = 0; k < 3; ++k) v[k] += p.frf[((size_t)c * 3 + k) * cap + i];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1)
#pragma unroll
    for (int k = 0; k < 3; ++k) v[k] += __shfl_xor_sync(0xffffffffu, v[k], o);
  if (lane != 0) return;
  double f[3];
  if (fl.use_total) {
    f[0] = p.fx[i];
    f[1] = p.fy[i];
    f[2] = p.fz[i];
  } else {
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      double w = p.ffield[k * cap + i] + v[k];
      if (fl.is) w += p.fis[k * cap + i];
      f[k] = w;
    }
    p.fx[i] = f[0];
    p.fy[i] = f[1];
    p.fz[i] = f[2];
  }
  if (do_bd) bd_move(p, fl, variant, seed, step, i, f);
}

// ---------------------------------------------------------------------------
// FP32 mode.  Compensated float sums of the partial forces (two_sum), and
// the BD move on the float-float position records.  Variants 1-3 evaluate
// their diffusion profile in FP64 (options off the hot path); variant 0 and
// everything else stay on the FP32 pipe.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void bd_move_f32(const KP &p, int variant, uint64_t seed,
                                            uint64_t step, int i, const float F[3]) {
  const int m0 = p.nsites + p.nfix;
  if (i < m0 && (i >= p.nsites || !p.stfree[i])) return;  // fixed ions, frozen sites
  float4 h4 = p.pk1[i], l4 = p.pk2[i];
  float h[3] = {h4.x, h4.y, h4.z}, l[3] = {l4.x, l4.y, l4.z};
  float g[3];
  bd_noise3_f(seed, step, (uint32_t)i, g);
  if (i < p.nsites) {  // dynamics0nuc.f90:31-44
    for (int k = 0; k < 3; ++k) {
      float d = F[k] * p.f.fact0n1;
      clamp_f(p.f.bdmax, d);
      ff_add(h[k], l[k], fmaf(p.f.fact0n2, g[k], d));
    }
    if (!p.qdnafree) fixcoor_ff(p.f.box, h, l);
  } else {
    const int itype = abs(p.typei[i]);
    float fact1, fact2, dD[3] = {0.0f, 0.0f, 0.0f};
    if (variant == 0) {
      const float2 fa = p.fact_f[itype];
      fact1 = fa.x;
      fact2 = fa.y;
    } else {
      double f1, f2, dd[3];
      diff_model(p, variant, i, itype, (double)h[2] + (double)l[2], f1, f2, dd);
      fact1 = (float)f1;
      fact2 = (float)f2;
      dD[0] = (float)dd[0];
      dD[1] = (float)dd[1];
      dD[2] = (float)dd[2];
    }
    const float zh0 = h[2], zl0 = l[2];
    for (int k = 0; k < 3; ++k) {
      float d = F[k] * fact1;
      clamp_f(p.f.bdmax, d);
      ff_add(h[k], l[k], fmaf(fact2, g[k], d) + dD[k]);
    }
    if (p.qcountion) {  // countions.f90:25-31, crossing tests in float-float
      const int it = itype - p.nold - 1;
      for (int j = 0; j < p.cntpts; ++j) {
        const float2 zc = p.zcont_ff[j];
        const bool was_below = ff_diff(zh0, zl0, zc.x, zc.y) < 0.0f;
        const bool is_below = ff_diff(h[2], l[2], zc.x, zc.y) < 0.0f;
        if (was_below && !is_below)
          atomicAdd(&p.nforward[it * p.cntpts + j], 1);
        else if (!was_below && is_below)
          atomicAdd(&p.nbackward[it * p.cntpts + j], 1);
      }
    }
    fixcoor_ff(p.f.box, h, l);
  }
  h4.x = h[0];
  h4.y = h[1];
  h4.z = h[2];
  l4.x = l[0];
  l4.y = l[1];
  l4.z = l[2];
  p.pk1[i] = h4;
  p.pk2[i] = l4;
}

__global__ void __launch_bounds__(32 * kAsmWarps)
    k_assemble_f32(KP p, AssembleFlags fl, int do_bd, int variant, uint64_t seed,
                   uint64_t step) {
  const int i = blockIdx.x * kAsmWarps + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  const int ntot = p.st->ntot;
  if (i >= ntot) return;  // warp-uniform
  const int cap = p.cap;
  const int m0 = p.nsites + p.nfix;
  float s[3] = {0.f, 0.f, 0.f}, c[3] = {0.f, 0.f, 0.f};  // compensated sums
  if (!fl.use_total) {
    if (fl.ii && i >= fl.ii_from)
      for (int ch = lane; ch < fl.nchunk_ii; ch += 32)
#pragma unroll
        for (int k = 0; k < 3; ++k) acc2(s[k], c[k], p.fii_f[((size_t)ch * 3 + k) * cap + i]);
    if (fl.rf && i >= p.nsites)
      for (int ch = lane; ch < fl.nchunk_rf; ch += 32)
#pragma unroll
        for (int k = 0; k < 3; ++k) acc2(s[k], c[k], p.frf_f[((size_t)ch * 3 + k) * cap + i]);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        const float s2 = __shfl_xor_sync(0xffffffffu, s[k], o);
        const float c2 = __shfl_xor_sync(0xffffffffu, c[k], o);
        acc2p(s[k], c[k], s2, c2);
      }
  }
  if (lane != 0) return;
  float F[3];
  if (fl.use_total) {
    F[0] = (float)p.fx[i];
    F[1] = (float)p.fy[i];
    F[2] = (float)p.fz[i];
  } else {
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      acc2(s[k], c[k], p.ffield_f[k * cap + i]);
      if (fl.is) acc2(s[k], c[k], p.fis_f[k * cap + i]);
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) F[k] = s[k] + c[k];
    if (!do_bd) {  // forces for the host (energy calls)
      p.fx[i] = F[0];
      p.fy[i] = F[1];
      p.fz[i] = F[2];
    }
  }
  if (do_bd) bd_move_f32(p, variant, seed, step, i, F);
}

// FP32 assembly for the Newton-3 partials: one block per tile of 32
// particles (site tiles first, then the ion tiles of the pair kernel).  The
// eight warps take every eighth tile pair of the ion tile, four at a time
// with all loads issued first, each partial one coalesced 512-byte row;
// their compensated sums meet in shared memory in a fixed order; warp 0 then
// assembles and moves its 32 particles, one lane each.
constexpr int kTileWarps = 8;

__global__ void __launch_bounds__(32 * kTileWarps)
    k_assemble_tiles(KP p, AssembleFlags fl, int do_bd, int variant, uint64_t seed,
                     uint64_t step, int site_blocks) {
  __shared__ float part[kTileWarps][10][32];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const bool ionblk = (int)blockIdx.x >= site_blocks;
  const int Ti = blockIdx.x - site_blocks;
  const int i = ionblk ? p.nsites + 32 * Ti + lane : 32 * blockIdx.x + lane;
  const int ntot = p.st->ntot;
  float s[5] = {0.f, 0.f, 0.f, 0.f, 0.f}, c[5] = {0.f, 0.f, 0.f, 0.f, 0.f};
  if (ionblk) {
    const int T = fl.ntile;
    // batches of four tile pairs per warp: all loads issued before the sums
    for (int u0 = w; u0 < T; u0 += 4 * kTileWarps) {
      float4 va[4], vb[4];
      float ba[4], bb[4];
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int u = u0 + j * kTileWarps;
        va[j] = vb[j] = make_float4(0.f, 0.f, 0.f, 0.f);
        ba[j] = bb[j] = 0.f;
        if (u < T) {
          const int q = u < Ti ? n3_index(T, u, Ti) : n3_index(T, Ti, u);
          const size_t o = (size_t)q * 64 + (u < Ti ? 32 : 0) + lane;
          va[j] = p.tpf[o];
          if (fl.rf_ab) ba[j] = p.tpb[o];
          if (u == Ti) {  // diagonal tile pair: the column side too
            vb[j] = p.tpf[o + 32];
            if (fl.rf_ab) bb[j] = p.tpb[o + 32];
          }
        }
      }
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        acc2(s[0], c[0], va[j].x);
        acc2(s[1], c[1], va[j].y);
        acc2(s[2], c[2], va[j].z);
        acc2(s[3], c[3], va[j].w);
        acc2(s[4], c[4], ba[j]);
        if (u0 + j * kTileWarps == Ti) {
          acc2(s[0], c[0], vb[j].x);
          acc2(s[1], c[1], vb[j].y);
          acc2(s[2], c[2], vb[j].z);
          acc2(s[3], c[3], vb[j].w);
          acc2(s[4], c[4], bb[j]);
        }
      }
    }
  }
  if (w > 0)
#pragma unroll
    for (int k = 0; k < 5; ++k) {
      part[w][k][lane] = s[k];
      part[w][5 + k][lane] = c[k];
    }
  __syncthreads();
  if (w != 0) return;
  for (int ww = 1; ww < kTileWarps; ++ww)
#pragma unroll
    for (int k = 0; k < 5; ++k) acc2p(s[k], c[k], part[ww][k][lane], part[ww][5 + k][lane]);
  if (i >= ntot || (!ionblk && i >= p.nsites)) return;
  const int cap = p.cap;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    acc2(s[k], c[k], p.ffield_f[k * cap + i]);
    if (fl.is) acc2(s[k], c[k], p.fis_f[k * cap + i]);
  }
  if (fl.rf_ab && ionblk) {  // A sd1 + B sd2 of the cross term, rfpar.f90:177-223
    const float A = s[3] + c[3], B = s[4] + c[4];
    const float4 d1 = p.rfd[2 * (size_t)i], d2 = p.rfd[2 * (size_t)i + 1];
    acc2(s[0], c[0], fmaf(A, d1.x, B * d2.x));
    acc2(s[1], c[1], fmaf(A, d1.y, B * d2.y));
    acc2(s[2], c[2], fmaf(A, d1.z, B * d2.z));
  }
  float F[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) F[k] = s[k] + c[k];
  if (!do_bd) {  // forces for the host (energy calls)
    p.fx[i] = F[0];
    p.fy[i] = F[1];
    p.fz[i] = F[2];
    return;
  }
  bd_move_f32(p, variant, seed, step, i, F);
}

void launch_assemble(const KP &p, int ntot_ub, const AssembleFlags &fl,
                     int do_bd, int variant, uint64_t seed, uint64_t step,
                     cudaStream_t stream) {
  if (ntot_ub <= 0) return;
  if (fl.fp32_partials && fl.ntile > 0 && !fl.use_total) {
    const int sb = (p.nsites + 31) / 32;
    k_assemble_tiles<<<sb + fl.ntile, 32 * kTileWarps, 0, stream>>>(p, fl, do_bd, variant, seed,
                                                                    step, sb);
    return;
  }
  const int nb = (ntot_ub + kAsmWarps - 1) / kAsmWarps;
  if (fl.fp32_partials)
    k_assemble_f32<<<nb, 32 * kAsmWarps, 0, stream>>>(p, fl, do_bd, variant, seed, step);
  else
    k_assemble<<<nb, 32 * kAsmWarps, 0, stream>>>(p, fl, do_bd, variant, seed, step);
}

}  // namespace bgpu
