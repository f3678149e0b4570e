// Force assembly and the Ermak-McCammon BD update (dynamics0-3.mono.f90,
// dynamics0nuc.f90, fixcoor.f90, countions.f90), fused in one kernel: one
// thread per particle sums its partial forces in a fixed order, writes
// fx,fy,fz and, for a BD step, moves the particle with in-register Philox
// noise.
#include "launch.h"
#include "physics.cuh"

namespace bgpu {

constexpr int kBdThreads = 64;

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

__global__ void __launch_bounds__(kBdThreads)
    k_assemble(KP p, AssembleFlags fl, int do_bd, int variant, uint64_t seed,
               uint64_t step) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int ntot = p.st->ntot;
  if (i >= ntot) return;
  const int cap = p.cap;
  const int m0 = p.nsites + p.nfix;
  double f[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    double v = p.ffield[k * cap + i];
    if (fl.ii && i >= m0)
      for (int c = 0; c < fl.nchunk_ii; ++c) v += p.fii[((size_t)c * 3 + k) * cap + i];
    if (fl.is) v += p.fis[k * cap + i];
    if (fl.rf && i >= p.nsites)
      for (int c = 0; c < fl.nchunk_rf; ++c) v += p.frf[((size_t)c * 3 + k) * cap + i];
    f[k] = v;
  }
  p.fx[i] = f[0];
  p.fy[i] = f[1];
  p.fz[i] = f[2];
  if (!do_bd) return;
  const uint32_t slot = (uint32_t)i;
  if (i < p.nsites) {  // dynamics0nuc.f90:31-44
    if (!p.stfree[i]) return;
    double dx = f[0] * p.fact0n1, dy = f[1] * p.fact0n1, dz = f[2] * p.fact0n1;
    clamp_bd(p.bdmax, dx);
    clamp_bd(p.bdmax, dy);
    clamp_bd(p.bdmax, dz);
    double g[3];
    if (fl.fp32_noise)
      bd_noise3_f(seed, step, slot, g);
    else
      bd_noise3(seed, step, slot, g);
    double x = p.x[i] + dx + p.fact0n2 * g[0];
    double y = p.y[i] + dy + p.fact0n2 * g[1];
    double z = p.z[i] + dz + p.fact0n2 * g[2];
    if (!p.qdnafree) fixcoor(p, x, y, z);
    p.x[i] = x;
    p.y[i] = y;
    p.z[i] = z;
    return;
  }
  if (i < m0) return;  // fixed ions do not move
  const int itype = abs(p.typei[i]);
  double fact1, fact2, dDx = 0.0, dDy = 0.0, dDz = 0.0;
  const double zold = p.z[i];
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
    dDz = didif * p.dt;
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
    dDz = D * dsw * p.dt;
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
      dDx = didif * p.dt * dd[2] * idist;
      dDy = didif * p.dt * dd[3] * idist;
      dDz = didif * p.dt * dd[4] * idist;
    } else {
      fact1 = p.fact1a[itype];
      fact2 = p.fact2a[itype];
    }
  } else {  // dynamics0.mono.f90:31-46
    fact1 = p.fact1a[itype];
    fact2 = p.fact2a[itype];
  }
  double dx = f[0] * fact1, dy = f[1] * fact1, dz = f[2] * fact1;
  clamp_bd(p.bdmax, dx);
  clamp_bd(p.bdmax, dy);
  clamp_bd(p.bdmax, dz);
  double g[3];
  if (fl.fp32_noise)
    bd_noise3_f(seed, step, slot, g);
  else
    bd_noise3(seed, step, slot, g);
  double x = p.x[i] + dx + fact2 * g[0] + dDx;
  double y = p.y[i] + dy + fact2 * g[1] + dDy;
  double z = zold + dz + fact2 * g[2] + dDz;
  if (p.qcountion) {  // countions.f90:25-31
    const int it = itype - p.nold - 1;
    for (int j = 0; j < p.cntpts; ++j) {
      const double zc = p.zcont[j];
      if (zold < zc && z >= zc)
        atomicAdd(&p.nforward[it * p.cntpts + j], 1);
      else if (zold >= zc && z < zc)
        atomicAdd(&p.nbackward[it * p.cntpts + j], 1);
    }
  }
  fixcoor(p, x, y, z);
  p.x[i] = x;
  p.y[i] = y;
  p.z[i] = z;
}

void launch_assemble(const KP &p, int ntot_ub, const AssembleFlags &fl,
                     int do_bd, int variant, uint64_t seed, uint64_t step,
                     cudaStream_t stream) {
  if (ntot_ub <= 0) return;
  const int nb = (ntot_ub + kBdThreads - 1) / kBdThreads;
  k_assemble<<<nb, kBdThreads, 0, stream>>>(p, fl, do_bd, variant, seed, step);
}

}  // namespace bgpu
