// Per-particle BD move of the FP32 path and the block-level force assembly
// of the Newton-3 partials, shared by the assembly kernel and the fused BD
// loop kernel.
#pragma once
#include "ff.cuh"
#include "launch.h"
#include "physics.cuh"

namespace bgpu {

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

// ---------------------------------------------------------------------------
// FP32 mode.  Compensated float sums of the partial forces (two_sum), and
// the BD move on the float-float position records.  Variants 1-3 evaluate
// their diffusion profile in FP64 (options off the hot path); variant 0 and
// everything else stay on the FP32 pipe.
// ---------------------------------------------------------------------------
// The arrays and sizes the FP32 assembly and move of one system work on: a
// context's own (ctx_asm_sys), or one replica's slots and partials in a
// batch.  ffield / fis are component-major with stride cap from the
// system's first particle; the noise of particle i is drawn from seed with
// i counted from the system's first particle.
struct AsmSys {
  float4 *pk1, *pk2;
  const float4 *pk3;
  const int *typei;
  const float *ffield, *fis;
  const float4 *rfd;
  const float4 *tpf;
  const float *tpb;
  int cap, nsites, nfix, ntot, T;
  uint64_t seed;
  const BoxF *box;
  double *fx, *fy, *fz;  // forces out when not moving (element i at i * fs)
  int fs;
};

__device__ __forceinline__ AsmSys ctx_asm_sys(const KP &p, int T, uint64_t seed) {
  return AsmSys{p.pk1, p.pk2, p.pk3, p.typei, p.ffield_f, p.fis_f, p.rfd, p.tpf, p.tpb, p.cap,
                p.nsites, p.nfix, p.st->ntot, T, seed, &p.f.box, p.fx, p.fy, p.fz, 1};
}

// What one particle's FP32 move needs besides its force: its position
// records, ion type, diffusion factors and noise.  None depends on the
// force, so the assembly gathers them before it sums the force.
struct MoveIn {
  float4 h4, l4;  // position hi / lo records
  float g[3];     // Gaussian noise of this step
  float2 fa;      // (fact1, fact2) of dynamics0
  float charge;   // from the pk3 record
  int itype;      // ion type, 0 for a site
  bool moves;     // false for fixed ions and frozen sites
};

// The loaded part (the types and factors do not change during BD and come
// through the read-only path); noise: whether to draw the noise here too.
__device__ __forceinline__ MoveIn move_in_f32(const KP &p, const AsmSys &ms, int variant,
                                              uint64_t step, int i, bool noise = true) {
  MoveIn m;
  const int m0 = ms.nsites + ms.nfix;
  m.moves = !(i < m0 && (i >= ms.nsites || !p.stfree[i]));
  m.h4 = ms.pk1[i];
  m.l4 = ms.pk2[i];
  m.itype = i < ms.nsites ? 0 : abs(__ldg(ms.typei + i));
  m.charge = __ldcg(&ms.pk3[i].y);
  m.fa = variant == 0 && i >= ms.nsites ? __ldg(p.fact_f + m.itype) : make_float2(0.f, 0.f);
  if (noise) bd_noise3_f(ms.seed, step, (uint32_t)i, m.g);
  return m;
}

// The move itself; m.h4 / m.l4 become the new records, also stored to
// pk1 / pk2.
__device__ __forceinline__ void bd_move_f32(const KP &p, const AsmSys &ms, int variant, int i,
                                            const float F[3], MoveIn &m) {
  if (!m.moves) return;
  float h[3] = {m.h4.x, m.h4.y, m.h4.z}, l[3] = {m.l4.x, m.l4.y, m.l4.z};
  const float *g = m.g;
  if (i < ms.nsites) {  // dynamics0nuc.f90:31-44
    for (int k = 0; k < 3; ++k) {
      float d = F[k] * p.f.fact0n1;
      clamp_f(p.f.bdmax, d);
      ff_add(h[k], l[k], fmaf(p.f.fact0n2, g[k], d));
    }
    if (!p.qdnafree) fixcoor_ff(*ms.box, h, l);
  } else {
    const int itype = m.itype;
    float fact1, fact2, dD[3] = {0.0f, 0.0f, 0.0f};
    if (variant == 0) {
      fact1 = m.fa.x;
      fact2 = m.fa.y;
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
    fixcoor_ff(*ms.box, h, l);
  }
  m.h4.x = h[0];
  m.h4.y = h[1];
  m.h4.z = h[2];
  m.l4.x = l[0];
  m.l4.y = l[1];
  m.l4.z = l[2];
  ms.pk1[i] = m.h4;
  ms.pk2[i] = m.l4;
}

__device__ __forceinline__ void bd_move_f32(const KP &p, int variant, uint64_t seed,
                                            uint64_t step, int i, const float F[3]) {
  const AsmSys ms = ctx_asm_sys(p, 0, seed);
  MoveIn m = move_in_f32(p, ms, variant, step, i);
  bd_move_f32(p, ms, variant, i, F, m);
}

// FP32 assembly for the Newton-3 partials: one block of NW warps per tile of
// 32 particles (site tiles first, then the ion tiles of the pair kernel).
// The warps take every NW-th tile pair of the ion tile, four at a time with
// all loads issued first, each partial one coalesced 512-byte row (the
// diagonal pair's column side last, by the warp that holds it); their
// compensated sums meet in shared memory in a fixed order; warp 0 then
// assembles and moves its 32 particles, one lane each.  Inputs that another
// block may have written in the same launch are read past L1.  blk: the tile
// (site tiles are 0 .. site_blocks-1); half: -1 for the whole tile, else only
// lanes 16 half .. 16 half + 15 assemble and move (two blocks share a tile).
// Warp 1 draws their noise while warp 0 gathers their other inputs.
// npos: when given, warp 0 leaves each of those particles' records there
// (npos[lane] = {hi, lo} after the move, {charge, ion type bits, 0, 0}).  Every thread of the block calls it.
template <int NW>
__device__ __forceinline__ void assemble_tile(const KP &p, const AsmSys &ms,
                                              const AssembleFlags &fl, int do_bd, int variant,
                                              uint64_t step, int blk, int site_blocks,
                                              float (*part)[10][32], int half = -1,
                                              float4 (*npos)[3] = nullptr) {
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const bool ionblk = blk >= site_blocks;
  const int Ti = blk - site_blocks;
  const int i = ionblk ? ms.nsites + 32 * Ti + lane : 32 * blk + lane;
  const int ntot = ms.ntot;
  float s[5] = {0.f, 0.f, 0.f, 0.f, 0.f}, c[5] = {0.f, 0.f, 0.f, 0.f, 0.f};
  // warp 0: the particle's own inputs, loaded while the partials are summed
  const bool own = w == 0 && (half < 0 || (lane >> 4) == half) && i < ntot &&
                   (ionblk || i < ms.nsites);
  MoveIn mv{};
  float fo[3] = {0.f, 0.f, 0.f}, fs[3] = {0.f, 0.f, 0.f};
  float4 d1 = make_float4(0.f, 0.f, 0.f, 0.f), d2 = d1;
  // warp 1 draws the noise of warp 0's particles meanwhile, into part[0]
  // (warp 0 keeps no partials there)
  if (w == 1 && do_bd && (half < 0 || (lane >> 4) == half) && i < ntot &&
      (ionblk || i < ms.nsites)) {
    float g[3];
    bd_noise3_f(ms.seed, step, (uint32_t)i, g);
    part[0][0][lane] = g[0];
    part[0][1][lane] = g[1];
    part[0][2][lane] = g[2];
  }
  if (own) {
    const int cap = ms.cap;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      fo[k] = __ldcg(ms.ffield + k * cap + i);
      if (fl.is) fs[k] = __ldcg(ms.fis + k * cap + i);
    }
    if (fl.rf_ab && ionblk) {
      d1 = __ldcg(ms.rfd + 2 * (size_t)i);
      d2 = __ldcg(ms.rfd + 2 * (size_t)i + 1);
    }
    if (do_bd) mv = move_in_f32(p, ms, variant, step, i, NW < 2);
  }
  if (ionblk) {
    const int T = ms.T;
    for (int u0 = w; u0 < T; u0 += 4 * NW) {
      float4 va[4];
      float ba[4];
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int u = u0 + j * NW;
        va[j] = make_float4(0.f, 0.f, 0.f, 0.f);
        ba[j] = 0.f;
        if (u < T) {
          const int q = u < Ti ? n3_index(T, u, Ti) : n3_index(T, Ti, u);
          const size_t o = (size_t)q * 64 + (u < Ti ? 32 : 0) + lane;
          va[j] = __ldcg(ms.tpf + o);
          if (fl.rf_ab) ba[j] = __ldcg(ms.tpb + o);
        }
      }
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        acc2(s[0], c[0], va[j].x);
        acc2(s[1], c[1], va[j].y);
        acc2(s[2], c[2], va[j].z);
        acc2(s[3], c[3], va[j].w);
        acc2(s[4], c[4], ba[j]);
      }
    }
    if (Ti < T && Ti % NW == w) {  // the diagonal tile pair's column side
      const size_t o = (size_t)n3_index(T, Ti, Ti) * 64 + 32 + lane;
      const float4 vb = __ldcg(ms.tpf + o);
      acc2(s[0], c[0], vb.x);
      acc2(s[1], c[1], vb.y);
      acc2(s[2], c[2], vb.z);
      acc2(s[3], c[3], vb.w);
      if (fl.rf_ab) acc2(s[4], c[4], __ldcg(ms.tpb + o));
    }
  }
  if (w > 0)
#pragma unroll
    for (int k = 0; k < 5; ++k) {
      part[w][k][lane] = s[k];
      part[w][5 + k][lane] = c[k];
    }
  __syncthreads();
  if (!own) return;
  for (int ww = 1; ww < NW; ++ww)
#pragma unroll
    for (int k = 0; k < 5; ++k) acc2p(s[k], c[k], part[ww][k][lane], part[ww][5 + k][lane]);
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    acc2(s[k], c[k], fo[k]);
    if (fl.is) acc2(s[k], c[k], fs[k]);
  }
  if (fl.rf_ab && ionblk) {  // A sd1 + B sd2 of the cross term, rfpar.f90:177-223
    const float A = s[3] + c[3], B = s[4] + c[4];
    acc2(s[0], c[0], fmaf(A, d1.x, B * d2.x));
    acc2(s[1], c[1], fmaf(A, d1.y, B * d2.y));
    acc2(s[2], c[2], fmaf(A, d1.z, B * d2.z));
  }
  float F[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) F[k] = s[k] + c[k];
  if (!do_bd) {  // forces for the host (energy calls)
    if (ms.fx) {
      ms.fx[(size_t)i * ms.fs] = F[0];
      ms.fy[(size_t)i * ms.fs] = F[1];
      ms.fz[(size_t)i * ms.fs] = F[2];
    }
    return;
  }
  if (NW >= 2) {
    mv.g[0] = part[0][0][lane];
    mv.g[1] = part[0][1][lane];
    mv.g[2] = part[0][2][lane];
  }
  bd_move_f32(p, ms, variant, i, F, mv);
  if (npos) {
    npos[lane][0] = mv.h4;
    npos[lane][1] = mv.l4;
    npos[lane][2] = make_float4(mv.charge, __int_as_float(mv.itype), 0.f, 0.f);
  }
}

}  // namespace bgpu
