// Single-particle terms of ENERGY with one warp per particle: static field
// (staticf1.f90), repulsion map (vdwgd1trln.f90 / vdwgd1spln.f90), RFPAR
// gathers and self term (rfpar.f90:75-176) and the membrane (membrane.f90).
//
// Lane layout for the trilinear maps: lane = 8 g + corner, corner = 4a+2b+c
// selects the grid node (ix+a, iy+b, iz+c); g = 0 static field, 1 repulsion,
// 2 gsrfen (srfe), 3 greff (reff).  Each lane gathers one node and forms its
// weight and derivative terms; eight-lane shuffle trees give the sums.  The
// 27-point B-spline repulsion takes lanes 0..26 in a second pass.  The FP64
// kernel forms every weight as the reference does; the FP32 kernel works on
// float-float positions and single-precision weights throughout.
#include "batch.cuh"
#include "ff.cuh"
#include "launch.h"
#include "physics.cuh"
#include "fields32.cuh"

namespace bgpu {

constexpr int kFieldWarps = 4;

// Trilinear node weight of one lane along one axis: the reference forms
// w = 1 - |x - n dcel| / dcel and its sign (staticf1.f90:78-88).
template <class R>
__device__ __forceinline__ void axis_weight(double xi, int n0, int off,
                                            const Grid3 &g, R &w, R &sgn) {
  const double d = xi - (n0 + off) * g.dcel;
  sgn = d >= 0.0 ? R(1) : R(-1);
  w = (R)(1.0 - fabs(d) * g.idcel);
}

template <class R>
__global__ void __launch_bounds__(32 * kFieldWarps)
    k_fields_warp(KP p, uint32_t mask, int qforces, int slot0) {
  __shared__ double red[kFieldWarps * 4];
  __shared__ double tot[4];
  const int lane = threadIdx.x & 31;
  const int i = blockIdx.x * kFieldWarps + (threadIdx.x >> 5);
  const int ntot = p.st->ntot;
  double eo[4] = {0.0, 0.0, 0.0, 0.0};  // lane 0: ememb, egsbpa, evdwgd, erfpar
  if (i < ntot) {  // warp-uniform
    const bool site = i < p.nsites;
    const bool fixed = !site && i < p.nsites + p.nfix;
    const double x = p.x[i], y = p.y[i], z = p.z[i];
    const int iontype = site ? 0 : abs(p.typei[i]);
    const int itype2 = site ? p.typtyp[i] : p.nwtype[iontype];
    const double charge = site ? p.sitecharge[i] : p.cg[iontype];
    const bool qf = qforces != 0;
    const int g = lane >> 3, c = lane & 7;
    const int ca = (c >> 2) & 1, cb = (c >> 1) & 1, cc = c & 1;

    const bool do_phix = (mask & 4u) && p.qphix && !fixed &&
                         (!site || charge != 0.0) && in_grid(p.g1, x, y, z);
    const Grid3 &g2 = p.g2;
    bool phiv_ok = false;
    if ((mask & 8u) && p.qphiv && !fixed) {
      const double m = p.qtrln ? 0.0 : g2.dcel;
      phiv_ok = x <= g2.xbcen + g2.tranx - m && x >= g2.xbcen - g2.tranx + m &&
                y <= g2.ybcen + g2.trany - m && y >= g2.ybcen - g2.trany + m &&
                z <= p.vzmax && z >= p.vzmin;
    }
    const bool do_rf = (mask & 16u) && p.qrfpar && !site && in_grid(p.g3, x, y, z);
    size_t vifir = 0;
    double esvdw = 0.0;
    int vit2 = 0;
    if (phiv_ok) phiv_select(p, i, iontype, vifir, esvdw, vit2);

    // ---- pass A: trilinear maps, one node per lane ------------------------
    R le = 0, lf0 = 0, lf1 = 0, lf2 = 0, lsum = 0;
    R gs_own = 0;  // gsrfen at this lane's node (rf lanes)
    bool active = false;
    R ai = 0, as = 0, bi = 0, bs = 0, ci = 0, cs = 0, val = 0, vforce = 0;
    if (g == 0 && do_phix) {
      const Grid3 &gg = p.g1;
      const double xi = x + gg.tranx - gg.xbcen, yi = y + gg.trany - gg.ybcen,
                   zi = z + gg.tranz - gg.zbcen;
      int ix, iy, iz;
      cell_of(gg, xi, yi, zi, ix, iy, iz);
      axis_weight<R>(xi, ix, ca, gg, ai, as);
      axis_weight<R>(yi, iy, cb, gg, bi, bs);
      axis_weight<R>(zi, iz, cc, gg, ci, cs);
      const size_t node = (size_t)(ix + ca) * gg.ncly * gg.nclz + (size_t)(iy + cb) * gg.nclz + iz + cc;
      const R phi = (R)__ldg(p.phix + node);
      val = phi * (R)(p.celec * charge);
      vforce = val * (R)gg.idcel;
      active = true;
    } else if (g == 1 && phiv_ok && p.qtrln) {
      const double xi = x + g2.tranx - g2.xbcen, yi = y + g2.trany - g2.ybcen,
                   zi = z + g2.tranz - g2.zbcen;
      int ix, iy, iz;
      cell_of(g2, xi, yi, zi, ix, iy, iz);
      axis_weight<R>(xi, ix, ca, g2, ai, as);
      axis_weight<R>(yi, iy, cb, g2, bi, bs);
      axis_weight<R>(zi, iz, cc, g2, ci, cs);
      const size_t node = vifir + (size_t)(ix + ca) * g2.ncly * g2.nclz +
                          (size_t)(iy + cb) * g2.nclz + iz + cc;
      const R phis = (R)__ldg(p.phiv + node);
      lsum = phis;
      val = phis * (R)esvdw;
      vforce = val * (R)g2.idcel;
      active = true;
    } else if (g >= 2 && do_rf) {
      const Grid3 &gg = p.g3;
      const double xi = x + gg.tranx - gg.xbcen, yi = y + gg.trany - gg.ybcen,
                   zi = z + gg.tranz - gg.zbcen;
      int ix, iy, iz;
      cell_of(gg, xi, yi, zi, ix, iy, iz);
      axis_weight<R>(xi, ix, ca, gg, ai, as);
      axis_weight<R>(yi, iy, cb, gg, bi, bs);
      axis_weight<R>(zi, iz, cc, gg, ci, cs);
      const size_t node = rfpar_ifir(p, iontype) + (size_t)(ix + ca) * gg.ncly * gg.nclz +
                          (size_t)(iy + cb) * gg.nclz + iz + cc;
      gs_own = (R)__ldg(p.gsrfen + node);
      val = g == 2 ? gs_own : (R)(p.sqrfac * (double)__ldg(p.greff + node));
      vforce = -val * (R)gg.idcel;  // rfpar.f90:131-144 accumulates -sign...
      active = true;
    }
    // the reference leaves the innermost (z) loop at a zero gsrfen node:
    // node (a,b,1) counts only if (a,b,0) and (a,b,1) are nonzero, node
    // (a,b,0) only if it is nonzero (rfpar.f90:121)
    const R gs_c0 = __shfl_sync(0xffffffffu, gs_own, lane & ~1);
    if (g >= 2 && active && !(gs_c0 != R(0) && (cc == 0 || gs_own != R(0)))) active = false;
    if (active) {
      const R fi = ai * bi * ci;
      le = fi * val;
      if (qf) {
        const R lo = (R)kRsmall, hi = R(1) - (R)kRsmall;
        if (ai < hi && ai > lo) lf0 = as * bi * ci * vforce;
        if (bi < hi && bi > lo) lf1 = bs * ai * ci * vforce;
        if (ci < hi && ci > lo) lf2 = cs * ai * bi * vforce;
      }
    }
    le = seg8_sum(le);
    lf0 = seg8_sum(lf0);
    lf1 = seg8_sum(lf1);
    lf2 = seg8_sum(lf2);
    lsum = seg8_sum(lsum);

    // ---- pass B: 27-point B-spline repulsion (lanes 0..26) ---------------
    R be = 0, bf0 = 0, bf1 = 0, bf2 = 0, bsum = 0;
    if (phiv_ok && !p.qtrln) {  // warp-uniform
      R e1 = 0, f0 = 0, f1 = 0, f2 = 0, s1 = 0;
      if (lane < 27) {
        const double xi = x + g2.tranx - g2.xbcen, yi = y + g2.trany - g2.ybcen,
                     zi = z + g2.tranz - g2.zbcen;
        int ix, iy, iz;
        spln_cell(g2, xi, yi, zi, ix, iy, iz);
        const int k = ix - 1 + lane / 9, l = iy - 1 + (lane / 3) % 3, m = iz - 1 + lane % 3;
        const double ua = 1.5 - (xi - k * g2.dcel) * g2.idcel;
        const double ub = 1.5 - (yi - l * g2.dcel) * g2.idcel;
        const double uc = 1.5 - (zi - m * g2.dcel) * g2.idcel;
        const R a = (R)m3(ua), da = (R)dm3(ua), b = (R)m3(ub), db = (R)dm3(ub),
                cz = (R)m3(uc), dc = (R)dm3(uc);
        // a node is visited when none of its axes is cut off
        // (vdwgd1spln.f90:118,125,132)
        if ((a != R(0) || da != R(0)) && (b != R(0) || db != R(0)) &&
            (cz != R(0) || dc != R(0))) {
          const R phivi = (R)__ldg(p.phiv + vifir + (size_t)k * g2.ncly * g2.nclz +
                                   (size_t)l * g2.nclz + m);
          const R phivsv = phivi * (R)esvdw;
          s1 = phivi;
          e1 = a * b * cz * phivsv;
          if (qf) {
            const R pre = phivsv * (R)g2.idcel;
            f0 = da * b * cz * pre;
            f1 = a * db * cz * pre;
            f2 = a * b * dc * pre;
          }
        }
      }
      be = warp_sum(e1);
      bf0 = warp_sum(f0);
      bf1 = warp_sum(f1);
      bf2 = warp_sum(f2);
      bsum = warp_sum(s1);
    }

    // ---- gather the group sums in lane 0 ----------------------------------
    const R e_v = __shfl_sync(0xffffffffu, le, 8), f0_v = __shfl_sync(0xffffffffu, lf0, 8),
            f1_v = __shfl_sync(0xffffffffu, lf1, 8), f2_v = __shfl_sync(0xffffffffu, lf2, 8),
            s_v = __shfl_sync(0xffffffffu, lsum, 8);
    const R srfe = __shfl_sync(0xffffffffu, le, 16), d10 = __shfl_sync(0xffffffffu, lf0, 16),
            d11 = __shfl_sync(0xffffffffu, lf1, 16), d12 = __shfl_sync(0xffffffffu, lf2, 16);
    const R reff = __shfl_sync(0xffffffffu, le, 24), d20 = __shfl_sync(0xffffffffu, lf0, 24),
            d21 = __shfl_sync(0xffffffffu, lf1, 24), d22 = __shfl_sync(0xffffffffu, lf2, 24);
    if (lane == 0) {
      double f[3] = {0.0, 0.0, 0.0};
      if ((mask & 2u) && p.qmemb) {
        if (membrane_one(p, itype2, charge, x, y, z, !fixed && qf, false, eo[0], f))
          atomicAdd(&p.warn[itype2], 1);
      }
      if (do_phix) {
        eo[1] = (double)le;
        f[0] += (double)lf0;
        f[1] += (double)lf1;
        f[2] += (double)lf2;
      }
      if (phiv_ok) {
        double phisum;
        if (p.qtrln) {
          eo[2] = (double)e_v;
          f[0] += (double)f0_v;
          f[1] += (double)f1_v;
          f[2] += (double)f2_v;
          phisum = (double)s_v;
          if (phisum >= p.thold8) atomicAdd(&p.warn[vit2], 1);
        } else {
          eo[2] = (double)be;
          f[0] += (double)bf0;
          f[1] += (double)bf1;
          f[2] += (double)bf2;
          phisum = (double)bsum;
          if (phisum >= p.thold27) atomicAdd(&p.warn[vit2], 1);
        }
      }
      if ((mask & 16u) && p.qrfpar && !site) {
        const double a1 = do_rf ? (double)srfe : 0.0, a2 = do_rf ? (double)reff : 0.0;
        p.rf_in[i] = do_rf ? 1 : 0;
        p.rf_srfe[i] = a1;
        p.rf_reff[i] = a2;
        const double d1[3] = {do_rf ? (double)d10 : 0.0, do_rf ? (double)d11 : 0.0,
                              do_rf ? (double)d12 : 0.0};
        const double d2[3] = {do_rf ? (double)d20 : 0.0, do_rf ? (double)d21 : 0.0,
                              do_rf ? (double)d22 : 0.0};
        for (int k = 0; k < 3; ++k) {
          p.rf_d1[3 * i + k] = d1[k];
          p.rf_d2[3 * i + k] = d2[k];
        }
        if (do_rf && !fixed) {  // self term, rfpar.f90:161-176
          const double tau = p.celec * charge;
          const double aux = tau * charge * a1;
          eo[3] = 0.5 * aux * a1;
          if (qf) {
            f[0] -= aux * d1[0];
            f[1] -= aux * d1[1];
            f[2] -= aux * d1[2];
          }
        }
      }
      if (p.qproxdiff && !site)  // dids is rebuilt by the ion-site pass
        for (int m = 0; m < 5; ++m) p.dids[5 * (size_t)i + m] = 0.0;
      p.ffield[i] = f[0];
      p.ffield[p.cap + i] = f[1];
      p.ffield[2 * p.cap + i] = f[2];
    }
  }
  block_sum<4>(eo, red, tot);
  if (threadIdx.x == 0) {
    double *dst = p.epart + (size_t)(slot0 + blockIdx.x) * kNTerms;
    for (int k = 0; k < kNTerms; ++k) dst[k] = 0.0;
    dst[9] = tot[0];   // EMEMB
    dst[10] = tot[1];  // EGSBPA
    dst[12] = tot[2];  // EVDWGD
    dst[13] = tot[3];  // ERFPAR (self)
  }
}

__global__ void __launch_bounds__(32 * kFieldWarps)
    k_fields_warp_f32(const __grid_constant__ KP p, uint32_t mask, int qforces, int slot0) {
  __shared__ float red[kFieldWarps * 4];
  __shared__ float tot[4];
  __shared__ AxisF ax[12];
  stage_axes(p, ax);
  const int i = blockIdx.x * kFieldWarps + (threadIdx.x >> 5);
  const int ntot = p.st->ntot;
  float eo[4] = {0.0f, 0.0f, 0.0f, 0.0f};  // lane 0: ememb, egsbpa, evdwgd, erfpar
  if (i < ntot) {  // warp-uniform
    const bool site = i < p.nsites;
    fields_one_f32(p, i, site, !site && i < p.nsites + p.nfix, mask, qforces, eo, ax);
  }
  block_sum_f<4>(eo, red, tot);
  if (threadIdx.x == 0) {
    double *dst = p.epart + (size_t)(slot0 + blockIdx.x) * kNTerms;
    for (int k = 0; k < kNTerms; ++k) dst[k] = 0.0;
    dst[9] = tot[0];
    dst[10] = tot[1];
    dst[12] = tot[2];
    dst[13] = tot[3];
  }
}

// ---------------------------------------------------------------------------
// FP32 mode: FP64 coordinates -> float-float records (also the pair-law type
// code, mobility and charge), and back.
// ---------------------------------------------------------------------------
__global__ void k_pack(KP p) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= p.st->ntot) return;
  const bool site = i < p.nsites;
  const int iontype = site ? 0 : abs(p.typei[i]);
  const int it2 = site ? p.typtyp[i] : p.nwtype[iontype];
  const double q = site ? p.sitecharge[i] : p.cg[iontype];
  const int mobile = i >= p.nsites + p.nfix;
  const double x = p.x[i], y = p.y[i], z = p.z[i];
  const float xh = (float)x, yh = (float)y, zh = (float)z;
  p.pk1[i] = make_float4(xh, yh, zh, __int_as_float((it2 - 1) | (mobile << 16)));
  p.pk2[i] = make_float4((float)(x - (double)xh), (float)(y - (double)yh),
                         (float)(z - (double)zh), 0.0f);
  p.pk3[i] = make_float4(0.0f, (float)q, __int_as_float(mobile << 1), 0.0f);
}

__global__ void k_unpack(KP p) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= p.st->ntot) return;
  const float4 h = p.pk1[i], l = p.pk2[i];
  p.x[i] = (double)h.x + (double)l.x;
  p.y[i] = (double)h.y + (double)l.y;
  p.z[i] = (double)h.z + (double)l.z;
}

void launch_pack(const KP &p, int ntot_ub, bool to_records, cudaStream_t stream) {
  if (ntot_ub <= 0) return;
  const int nb = (ntot_ub + 127) / 128;
  if (to_records)
    k_pack<<<nb, 128, 0, stream>>>(p);
  else
    k_unpack<<<nb, 128, 0, stream>>>(p);
}

// Replica batches: one thread per slot of the batch arrays (one warp per
// slot with a B-spline repulsion map); slots past their replica's live count
// return at once.
constexpr int kBatchFieldThreads = 128;
__global__ void __launch_bounds__(kBatchFieldThreads)
    k_batch_fields_t(const __grid_constant__ KP p, const int *rep_of, const RepDev *rep,
                     float4 *pe, int nslots, uint32_t mask, int qforces) {
  __shared__ AxisF ax[12];
  stage_axes(p, ax);
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nslots) return;
  const RepDev &R = rep[rep_of[i]];
  if (i - R.off >= R.n) return;
  float eo[4] = {0.0f, 0.0f, 0.0f, 0.0f};
  fields_one_thread(p, i, mask, qforces, eo, ax);
  pe[i] = make_float4(eo[0], eo[1], eo[2], eo[3]);
}

__global__ void __launch_bounds__(32 * kFieldWarps)
    k_batch_fields(const __grid_constant__ KP p, const int *rep_of, const RepDev *rep,
                   float4 *pe, int nslots, uint32_t mask, int qforces) {
  __shared__ AxisF ax[12];
  stage_axes(p, ax);
  const int i = blockIdx.x * kFieldWarps + (threadIdx.x >> 5);
  if (i >= nslots) return;  // warp-uniform from here on
  const RepDev &R = rep[rep_of[i]];
  if (i - R.off >= R.n) return;
  float eo[4] = {0.0f, 0.0f, 0.0f, 0.0f};
  fields_one_f32(p, i, false, false, mask, qforces, eo, ax);
  if ((threadIdx.x & 31) == 0) pe[i] = make_float4(eo[0], eo[1], eo[2], eo[3]);
}

void launch_batch_fields(const KP &p, const int *rep_of, const RepDev *rep, float4 *pe,
                         int nslots, uint32_t mask, int qforces, cudaStream_t stream) {
  if (nslots <= 0) return;
  if ((mask & 8u) && p.qphiv && !p.qtrln) {
    const int nb = (nslots + kFieldWarps - 1) / kFieldWarps;
    k_batch_fields<<<nb, 32 * kFieldWarps, 0, stream>>>(p, rep_of, rep, pe, nslots, mask,
                                                         qforces);
  } else {
    const int nb = (nslots + kBatchFieldThreads - 1) / kBatchFieldThreads;
    k_batch_fields_t<<<nb, kBatchFieldThreads, 0, stream>>>(p, rep_of, rep, pe, nslots, mask,
                                                            qforces);
  }
}

int fields_blocks(int ntot_ub) { return (ntot_ub + kFieldWarps - 1) / kFieldWarps; }

void launch_fields(const KP &p, int ntot_ub, uint32_t mask, int qforces, bool fp32,
                   int slot0, cudaStream_t stream) {
  const int nb = fields_blocks(ntot_ub);
  if (nb == 0) return;
  if (fp32)
    k_fields_warp_f32<<<nb, 32 * kFieldWarps, 0, stream>>>(p, mask, qforces, slot0);
  else
    k_fields_warp<double><<<nb, 32 * kFieldWarps, 0, stream>>>(p, mask, qforces, slot0);
}

}  // namespace bgpu
