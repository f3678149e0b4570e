// Warp-level single-particle terms of the FP32 path (one warp per particle),
// shared by the field kernel and the fused BD loop kernel.
#pragma once
#include "ff.cuh"
#include "physics.cuh"

namespace bgpu {

template <class R>
__device__ __forceinline__ R seg8_sum(R v) {
  v += __shfl_xor_sync(0xffffffffu, v, 4);
  v += __shfl_xor_sync(0xffffffffu, v, 2);
  v += __shfl_xor_sync(0xffffffffu, v, 1);
  return v;
}

template <class R>
__device__ __forceinline__ R warp_sum(R v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// quadratic B-spline and derivative in single precision (m3.f90, dm3.f90)
__device__ __forceinline__ float m3f(float x) {
  const float m2m = (x >= 0.0f && x <= 2.0f) ? 1.0f - fabsf(x - 1.0f) : 0.0f;
  const float m2 = (x >= 1.0f && x <= 3.0f) ? 1.0f - fabsf(x - 2.0f) : 0.0f;
  return (x >= 0.0f && x <= 3.0f) ? x * 0.5f * m2m + (3.0f - x) * 0.5f * m2 : 0.0f;
}
__device__ __forceinline__ float dm3f(float x) {
  const float m2m = (x >= 0.0f && x <= 2.0f) ? 1.0f - fabsf(x - 1.0f) : 0.0f;
  const float m2 = (x >= 1.0f && x <= 3.0f) ? 1.0f - fabsf(x - 2.0f) : 0.0f;
  return m2m - m2;
}

// ---------------------------------------------------------------------------
// FP32 variant: no double-precision instruction.  Positions come from the
// float-float particle records (pk1 hi, pk2 lo); lanes 0..11 find, for axis a
// of grid m (lane 3m+a; m = 0 static field, 1 repulsion, 2 RFPAR), the
// trilinear cell, the offset u - ix and the in-map test, and lanes 9..11 the
// nint cell of the B-spline stencil (ff_cell).  Every other lane reads them by
// shuffle: w = 1 - |u - ix - a|, sign(u - ix - a).  Outputs: ffield_f, the
// RFPAR gradients (rfd), srfe into pk2.w and reff/flags into pk3 for the
// pair kernels.
// ---------------------------------------------------------------------------
__device__ __forceinline__ size_t phiv_ifir(const KP &p, int i, int iontype) {
  const size_t ncel3 = (size_t)p.g2.nclx * p.g2.ncly * p.g2.nclz;
  if (!p.qnmcden) return 0;
  if (i < p.nsites) return p.site_map ? (size_t)p.site_map[i] * ncel3 : 0;
  if (i >= p.nsites + p.nfix) return (size_t)p.phiv_map_of_type[iontype] * ncel3;
  return 0;
}

// The FP32 field terms of particle i, one warp (lane 0 holds eo: ememb,
// egsbpa, evdwgd, erfpar).  site / fixed: the particle's role.
// The 12 axis records of the cell search, copied from the parameter block
// into shared memory: every lane reads its own record, and divergent indexing
// of the parameter block serialises.  Every thread of the block calls it.
__device__ __forceinline__ void stage_axes(const KP &p, AxisF *ax) {
  if (threadIdx.x < 12) ax[threadIdx.x] = p.f.ax[threadIdx.x];
  __syncthreads();
}

// ax: the block's staged copy of p.f.ax (stage_axes); pos: when given, the
// particle's position records {hi, lo} and {charge, ion type bits} (else
// read from pk1 / pk2 / pk3 / typei).
__device__ __forceinline__ void fields_one_f32(const KP &p, int i, bool site, bool fixed,
                                               uint32_t mask, int qforces, float eo[4],
                                               const AxisF *ax, const float4 *pos = nullptr) {
  const int lane = threadIdx.x & 31;
  const float4 h4 = pos ? pos[0] : p.pk1[i], l4 = pos ? pos[1] : p.pk2[i];
  const float charge = pos ? pos[2].x : p.pk3[i].y;
  const int code = __float_as_int(h4.w);
  const int itype2 = (code & 0xffff) + 1;
  const int mobile = (code >> 16) & 1;
  const int iontype = site ? 0 : (pos ? __float_as_int(pos[2].y) : abs(p.typei[i]));
  const bool qf = qforces != 0;
  // ---- per-(grid, axis) cells, float-float, lanes 0..11 -----------------
  int cix = 0, cin = 0;
  float cfr = 0.0f;
  if (lane < 12) {
    const AxisF &A = ax[lane];
    const int a = lane % 3;
    const float ph = a == 0 ? h4.x : (a == 1 ? h4.y : h4.z);
    const float pl = a == 0 ? l4.x : (a == 1 ? l4.y : l4.z);
    cfr = ff_cell(A, ph, pl, lane >= 9, cix);
    cin = lane < 9 && ff_inside(A, ph, pl);
  }
  const unsigned full = 0xffffffffu;
  const int in1 = __shfl_sync(full, cin, 0) & __shfl_sync(full, cin, 1) & __shfl_sync(full, cin, 2);
  const int in2 = __shfl_sync(full, cin, 3) & __shfl_sync(full, cin, 4) & __shfl_sync(full, cin, 5);
  const int in3 = __shfl_sync(full, cin, 6) & __shfl_sync(full, cin, 7) & __shfl_sync(full, cin, 8);
  const bool do_phix = (mask & 4u) && p.qphix && !fixed && (!site || charge != 0.0f) && in1;
  const bool phiv_ok = (mask & 8u) && p.qphiv && !fixed && in2;
  const bool do_rf = (mask & 16u) && p.qrfpar && !site && in3;
  const size_t vifir = phiv_ok ? phiv_ifir(p, i, iontype) : 0;
  const float esvdw = phiv_ok ? p.esvdw_f[itype2] : 0.0f;

  // ---- pass A: trilinear maps, lane = 8 g + corner ------------------------
  const int g = lane >> 3, c = lane & 7;
  const int ca = (c >> 2) & 1, cb = (c >> 1) & 1, cc = c & 1;
  const int src = 3 * (g < 2 ? g : 2);  // grid of this lane's group
  const int ix = __shfl_sync(full, cix, src), iy = __shfl_sync(full, cix, src + 1),
            iz = __shfl_sync(full, cix, src + 2);
  const float fx = __shfl_sync(full, cfr, src), fy = __shfl_sync(full, cfr, src + 1),
              fz = __shfl_sync(full, cfr, src + 2);
  const float dxa = fx - (float)ca, dyb = fy - (float)cb, dzc = fz - (float)cc;
  const float ai = 1.0f - fabsf(dxa), bi = 1.0f - fabsf(dyb), ci = 1.0f - fabsf(dzc);
  const float as = dxa >= 0.0f ? 1.0f : -1.0f, bs = dyb >= 0.0f ? 1.0f : -1.0f,
              cs = dzc >= 0.0f ? 1.0f : -1.0f;
  float val = 0.0f, vforce = 0.0f, lsum = 0.0f, gs_own = 0.0f;
  bool active = false;
  if (g == 0 && do_phix) {
    const Grid3 &gg = p.g1;
    const size_t node = (size_t)(ix + ca) * gg.ncly * gg.nclz + (size_t)(iy + cb) * gg.nclz + iz + cc;
    val = __ldg(p.phix + node) * (p.f.celec * charge);
    vforce = val * p.f.ax[0].idc;
    active = true;
  } else if (g == 1 && phiv_ok && p.qtrln) {
    const Grid3 &gg = p.g2;
    const size_t node = vifir + (size_t)(ix + ca) * gg.ncly * gg.nclz +
                        (size_t)(iy + cb) * gg.nclz + iz + cc;
    lsum = (float)__ldg(p.phiv + node);
    val = lsum * esvdw;
    vforce = val * p.f.ax[3].idc;
    active = true;
  } else if (g >= 2 && do_rf) {
    const Grid3 &gg = p.g3;
    const size_t node = rfpar_ifir(p, iontype) + (size_t)(ix + ca) * gg.ncly * gg.nclz +
                        (size_t)(iy + cb) * gg.nclz + iz + cc;
    gs_own = __ldg(p.gsrfen + node);
    val = g == 2 ? gs_own : p.f.sqrfac * __ldg(p.greff + node);
    vforce = -val * p.f.ax[6].idc;
    active = true;
  }
  const float gs_c0 = __shfl_sync(full, gs_own, lane & ~1);  // rfpar.f90:121
  if (g >= 2 && active && !(gs_c0 != 0.0f && (cc == 0 || gs_own != 0.0f))) active = false;
  float le = 0.0f, lf0 = 0.0f, lf1 = 0.0f, lf2 = 0.0f;
  if (active) {
    le = ai * bi * ci * val;
    if (qf) {
      const float lo = (float)kRsmall, hi = 1.0f - (float)kRsmall;
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

  // ---- pass B: 27-point B-spline repulsion ------------------------------
  float be = 0.0f, bf0 = 0.0f, bf1 = 0.0f, bf2 = 0.0f, bsum = 0.0f;
  if (phiv_ok && !p.qtrln) {  // warp-uniform
    const int sx = __shfl_sync(full, cix, 9), sy = __shfl_sync(full, cix, 10),
              sz = __shfl_sync(full, cix, 11);
    const float ux = __shfl_sync(full, cfr, 9), uy = __shfl_sync(full, cfr, 10),
                uz = __shfl_sync(full, cfr, 11);
    float e1 = 0.0f, f0 = 0.0f, f1 = 0.0f, f2 = 0.0f, s1 = 0.0f;
    if (lane < 27) {
      const int dk = lane / 9 - 1, dl = (lane / 3) % 3 - 1, dm = lane % 3 - 1;
      // 1.5 - (xi - k dcel)/dcel with k = ix + dk
      const float ua = 1.5f - ux + (float)dk, ub = 1.5f - uy + (float)dl,
                  uc = 1.5f - uz + (float)dm;
      const float a = m3f(ua), da = dm3f(ua), b = m3f(ub), db = dm3f(ub),
                  cz = m3f(uc), dc = dm3f(uc);
      if ((a != 0.0f || da != 0.0f) && (b != 0.0f || db != 0.0f) &&
          (cz != 0.0f || dc != 0.0f)) {
        const Grid3 &gg = p.g2;
        const float phivi = (float)__ldg(p.phiv + vifir +
                                        (size_t)(sx + dk) * gg.ncly * gg.nclz +
                                        (size_t)(sy + dl) * gg.nclz + sz + dm);
        const float phivsv = phivi * esvdw;
        s1 = phivi;
        e1 = a * b * cz * phivsv;
        if (qf) {
          const float pre = phivsv * p.f.ax[9].idc;
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
  const float e_v = __shfl_sync(full, le, 8), f0_v = __shfl_sync(full, lf0, 8),
              f1_v = __shfl_sync(full, lf1, 8), f2_v = __shfl_sync(full, lf2, 8),
              s_v = __shfl_sync(full, lsum, 8);
  const float srfe = __shfl_sync(full, le, 16), d10 = __shfl_sync(full, lf0, 16),
              d11 = __shfl_sync(full, lf1, 16), d12 = __shfl_sync(full, lf2, 16);
  const float reff = __shfl_sync(full, le, 24), d20 = __shfl_sync(full, lf0, 24),
              d21 = __shfl_sync(full, lf1, 24), d22 = __shfl_sync(full, lf2, 24);
  if (lane == 0) {
    float ff0 = 0.0f, ff1 = 0.0f, ff2 = 0.0f;
    if ((mask & 2u) && p.qmemb) {  // membrane in FP64 (an option off the hot path)
      double f[3] = {0.0, 0.0, 0.0}, em = 0.0;
      const double dq = site ? p.sitecharge[i] : p.cg[iontype];
      if (membrane_one(p, itype2, dq, (double)h4.x + (double)l4.x,
                       (double)h4.y + (double)l4.y, (double)h4.z + (double)l4.z,
                       !fixed && qf, false, em, f))
        atomicAdd(&p.warn[itype2], 1);
      eo[0] = (float)em;
      ff0 = (float)f[0];
      ff1 = (float)f[1];
      ff2 = (float)f[2];
    }
    if (do_phix) {
      eo[1] = le;
      ff0 += lf0;
      ff1 += lf1;
      ff2 += lf2;
    }
    if (phiv_ok) {
      if (p.qtrln) {
        eo[2] = e_v;
        ff0 += f0_v;
        ff1 += f1_v;
        ff2 += f2_v;
        if (s_v >= p.f.thold8) atomicAdd(&p.warn[itype2], 1);
      } else {
        eo[2] = be;
        ff0 += bf0;
        ff1 += bf1;
        ff2 += bf2;
        if (bsum >= p.f.thold27) atomicAdd(&p.warn[itype2], 1);
      }
    }
    if ((mask & 16u) && p.qrfpar && !site) {
      p.rfd[2 * (size_t)i] = do_rf ? make_float4(d10, d11, d12, 0.0f) : make_float4(0.f, 0.f, 0.f, 0.f);
      p.rfd[2 * (size_t)i + 1] = do_rf ? make_float4(d20, d21, d22, 0.0f) : make_float4(0.f, 0.f, 0.f, 0.f);
      if (do_rf && !fixed) {  // self term, rfpar.f90:161-176
        const float aux = p.f.celec * charge * charge * srfe;
        eo[3] = 0.5f * aux * srfe;
        if (qf) {
          ff0 -= aux * d10;
          ff1 -= aux * d11;
          ff2 -= aux * d12;
        }
      }
    }
    if (p.qproxdiff && !site)
      for (int m = 0; m < 5; ++m) p.dids[5 * (size_t)i + m] = 0.0;
    p.ffield_f[i] = ff0;
    p.ffield_f[p.cap + i] = ff1;
    p.ffield_f[2 * p.cap + i] = ff2;
    p.pk2[i].w = do_rf ? srfe : 0.0f;
    // flags: 1 in the RFPAR map, 2 mobile, 4 may play i of an RFPAR cross
    // pair (in map and mobile), 8 may play j (in map, srfe != 0)
    const int rfl = (do_rf ? 1 : 0) | (mobile << 1) | ((do_rf && mobile) ? 4 : 0) |
                    ((do_rf && srfe != 0.0f) ? 8 : 0);
    p.pk3[i] = make_float4(do_rf ? reff : 0.0f, charge, __int_as_float(rfl), 0.0f);
  }
}

// ---------------------------------------------------------------------------
// The same terms with one thread per particle, for ions that are neither
// sites nor fixed, with a trilinear repulsion map (replica batches, where a
// warp per slot leaves most lanes idle in the cell search and the sums).  The thread does every lane's
// arithmetic of fields_one_f32 with the same expressions, and forms each
// shuffle-tree sum in the tree's order -- IEEE addition commutes, so every
// lane of an xor butterfly holds the same fixed-order sum -- so the results
// are the warp version's bit for bit (a batch replica's step equals a single
// context's).
// ---------------------------------------------------------------------------
// seg8_sum's value: levels xor 4, 2, 1
__device__ __forceinline__ float tree8(const float v[8]) {
  const float w0 = v[0] + v[4], w1 = v[1] + v[5], w2 = v[2] + v[6], w3 = v[3] + v[7];
  return (w0 + w2) + (w1 + w3);
}
__device__ __forceinline__ void fields_one_thread(const KP &p, int i, uint32_t mask, int qforces,
                                                  float eo[4], const AxisF *ax) {
  const float4 h4 = p.pk1[i], l4 = p.pk2[i];
  const float charge = p.pk3[i].y;
  const int code = __float_as_int(h4.w);
  const int itype2 = (code & 0xffff) + 1;
  const int mobile = (code >> 16) & 1;
  const int iontype = abs(p.typei[i]);
  const bool qf = qforces != 0;
  // the cells of lanes 0..11
  int cix[12], cin[12];
  float cfr[12];
#pragma unroll
  for (int k = 0; k < 12; ++k) {
    const AxisF &A = ax[k];
    const int a = k % 3;
    const float ph = a == 0 ? h4.x : (a == 1 ? h4.y : h4.z);
    const float pl = a == 0 ? l4.x : (a == 1 ? l4.y : l4.z);
    cfr[k] = ff_cell(A, ph, pl, k >= 9, cix[k]);
    cin[k] = k < 9 && ff_inside(A, ph, pl);
  }
  const int in1 = cin[0] & cin[1] & cin[2], in2 = cin[3] & cin[4] & cin[5],
            in3 = cin[6] & cin[7] & cin[8];
  const bool do_phix = (mask & 4u) && p.qphix && in1;
  const bool phiv_ok = (mask & 8u) && p.qphiv && in2;
  const bool do_rf = (mask & 16u) && p.qrfpar && in3;
  const size_t vifir = phiv_ok ? phiv_ifir(p, i, iontype) : 0;
  const float esvdw = phiv_ok ? p.esvdw_f[itype2] : 0.0f;
  // pass A: group g = 0 static field, 1 repulsion, 2 gsrfen, 3 greff; corner c
  float se[4], sf0[4], sf1[4], sf2[4], ssum[4];
#pragma unroll
  for (int g = 0; g < 4; ++g) {
    const int src = 3 * (g < 2 ? g : 2);
    const int ix = cix[src], iy = cix[src + 1], iz = cix[src + 2];
    const float fx = cfr[src], fy = cfr[src + 1], fz = cfr[src + 2];
    float le[8], lf0[8], lf1[8], lf2[8], ls[8], gs[8];
    bool act[8];
    float val[8], vf[8];
#pragma unroll
    for (int c = 0; c < 8; ++c) {
      const int ca = (c >> 2) & 1, cb = (c >> 1) & 1, cc = c & 1;
      val[c] = 0.0f;
      vf[c] = 0.0f;
      ls[c] = 0.0f;
      gs[c] = 0.0f;
      act[c] = false;
      if (g == 0 && do_phix) {
        const Grid3 &gg = p.g1;
        const size_t node = (size_t)(ix + ca) * gg.ncly * gg.nclz + (size_t)(iy + cb) * gg.nclz +
                            iz + cc;
        val[c] = __ldg(p.phix + node) * (p.f.celec * charge);
        vf[c] = val[c] * p.f.ax[0].idc;
        act[c] = true;
      } else if (g == 1 && phiv_ok && p.qtrln) {
        const Grid3 &gg = p.g2;
        const size_t node = vifir + (size_t)(ix + ca) * gg.ncly * gg.nclz +
                            (size_t)(iy + cb) * gg.nclz + iz + cc;
        ls[c] = (float)__ldg(p.phiv + node);
        val[c] = ls[c] * esvdw;
        vf[c] = val[c] * p.f.ax[3].idc;
        act[c] = true;
      } else if (g >= 2 && do_rf) {
        const Grid3 &gg = p.g3;
        const size_t node = rfpar_ifir(p, iontype) + (size_t)(ix + ca) * gg.ncly * gg.nclz +
                            (size_t)(iy + cb) * gg.nclz + iz + cc;
        gs[c] = __ldg(p.gsrfen + node);
        val[c] = g == 2 ? gs[c] : p.f.sqrfac * __ldg(p.greff + node);
        vf[c] = -val[c] * p.f.ax[6].idc;
        act[c] = true;
      }
    }
#pragma unroll
    for (int c = 0; c < 8; ++c) {
      const int ca = (c >> 2) & 1, cb = (c >> 1) & 1, cc = c & 1;
      const float dxa = fx - (float)ca, dyb = fy - (float)cb, dzc = fz - (float)cc;
      const float ai = 1.0f - fabsf(dxa), bi = 1.0f - fabsf(dyb), ci = 1.0f - fabsf(dzc);
      const float as = dxa >= 0.0f ? 1.0f : -1.0f, bs = dyb >= 0.0f ? 1.0f : -1.0f,
                  cs = dzc >= 0.0f ? 1.0f : -1.0f;
      bool a = act[c];
      const float gs_c0 = gs[c & ~1];  // rfpar.f90:121
      if (g >= 2 && a && !(gs_c0 != 0.0f && (cc == 0 || gs[c] != 0.0f))) a = false;
      le[c] = lf0[c] = lf1[c] = lf2[c] = 0.0f;
      if (a) {
        le[c] = ai * bi * ci * val[c];
        if (qf) {
          const float lo = (float)kRsmall, hi = 1.0f - (float)kRsmall;
          if (ai < hi && ai > lo) lf0[c] = as * bi * ci * vf[c];
          if (bi < hi && bi > lo) lf1[c] = bs * ai * ci * vf[c];
          if (ci < hi && ci > lo) lf2[c] = cs * ai * bi * vf[c];
        }
      }
    }
    se[g] = tree8(le);
    sf0[g] = tree8(lf0);
    sf1[g] = tree8(lf1);
    sf2[g] = tree8(lf2);
    ssum[g] = tree8(ls);
  }
  float ff0 = 0.0f, ff1 = 0.0f, ff2 = 0.0f;
  if ((mask & 2u) && p.qmemb) {  // membrane in FP64 (an option off the hot path)
    double f[3] = {0.0, 0.0, 0.0}, em = 0.0;
    if (membrane_one(p, itype2, p.cg[iontype], (double)h4.x + (double)l4.x,
                     (double)h4.y + (double)l4.y, (double)h4.z + (double)l4.z, qf, false, em,
                     f))
      atomicAdd(&p.warn[itype2], 1);
    eo[0] = (float)em;
    ff0 = (float)f[0];
    ff1 = (float)f[1];
    ff2 = (float)f[2];
  }
  if (do_phix) {
    eo[1] = se[0];
    ff0 += sf0[0];
    ff1 += sf1[0];
    ff2 += sf2[0];
  }
  if (phiv_ok) {  // trilinear (the caller keeps B-spline maps on the warp version)
    eo[2] = se[1];
    ff0 += sf0[1];
    ff1 += sf1[1];
    ff2 += sf2[1];
    if (ssum[1] >= p.f.thold8) atomicAdd(&p.warn[itype2], 1);
  }
  const float srfe = se[2], reff = se[3];
  if ((mask & 16u) && p.qrfpar) {
    p.rfd[2 * (size_t)i] = do_rf ? make_float4(sf0[2], sf1[2], sf2[2], 0.0f)
                                 : make_float4(0.f, 0.f, 0.f, 0.f);
    p.rfd[2 * (size_t)i + 1] = do_rf ? make_float4(sf0[3], sf1[3], sf2[3], 0.0f)
                                     : make_float4(0.f, 0.f, 0.f, 0.f);
    if (do_rf) {  // self term, rfpar.f90:161-176
      const float aux = p.f.celec * charge * charge * srfe;
      eo[3] = 0.5f * aux * srfe;
      if (qf) {
        ff0 -= aux * sf0[2];
        ff1 -= aux * sf1[2];
        ff2 -= aux * sf2[2];
      }
    }
  }
  if (p.qproxdiff)
    for (int m = 0; m < 5; ++m) p.dids[5 * (size_t)i + m] = 0.0;
  p.ffield_f[i] = ff0;
  p.ffield_f[p.cap + i] = ff1;
  p.ffield_f[2 * p.cap + i] = ff2;
  p.pk2[i].w = do_rf ? srfe : 0.0f;
  const int rfl = (do_rf ? 1 : 0) | (mobile << 1) | ((do_rf && mobile) ? 4 : 0) |
                  ((do_rf && srfe != 0.0f) ? 8 : 0);
  p.pk3[i] = make_float4(do_rf ? reff : 0.0f, charge, __int_as_float(rfl), 0.0f);
}

}  // namespace bgpu
