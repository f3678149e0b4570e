// Force assembly and the Ermak-McCammon BD update (dynamics0-3.mono.f90,
// dynamics0nuc.f90, fixcoor.f90, countions.f90), fused in one kernel: one
// warp per particle sums its partial forces in a fixed order, writes
// fx,fy,fz and, for a BD step, moves the particle with in-register Philox
// noise.
#include "ff.cuh"
#include "launch.h"
#include "physics.cuh"
#include "move32.cuh"

namespace bgpu {

constexpr int kAsmWarps = 8;  // particles per assembly block

__device__ __forceinline__ void clamp_bd(double bdmax, double &d) {
  if (fabs(d) > bdmax) d = fsign(bdmax, d);
}

__device__ __forceinline__ void wrap1(double lo, double L, double &v) {
  if (v < lo)
    v += L;
  else if (v >= lo + L)
    v -= L;
}

// fixcoor.f90:19-68; in the extension mode (periodic box) one wrap into the
// box per axis instead of the clamp (BD moves are far shorter than a box).
__device__ __forceinline__ void fixcoor(const KP &p, double &x, double &y,
                                        double &z) {
  if (p.periodic) {
    wrap1(p.lx2m, p.lx, x);
    wrap1(p.ly2m, p.ly, y);
    wrap1(p.lz2m, p.lz, z);
    return;
  }
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


__global__ void __launch_bounds__(32 * kAsmWarps)
    k_assemble_f32(const __grid_constant__ KP p, AssembleFlags fl, int do_bd, int variant,
                   uint64_t seed, uint64_t step) {
  const int i = blockIdx.x * kAsmWarps + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  const int ntot = p.st->ntot;
  if (i >= ntot) return;  // warp-uniform
  const int cap = p.cap;
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

constexpr int kTileWarps = 16;  // as the fused loop's phase A: the same sums

__global__ void __launch_bounds__(32 * kTileWarps)
    k_assemble_tiles(const __grid_constant__ KP p, AssembleFlags fl, int do_bd, int variant,
                     uint64_t seed, uint64_t step, int site_blocks) {
  __shared__ float part[kTileWarps][10][32];
  assemble_tile<kTileWarps>(p, ctx_asm_sys(p, fl.ntile, seed), fl, do_bd, variant, step,
                            blockIdx.x, site_blocks, part);
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
