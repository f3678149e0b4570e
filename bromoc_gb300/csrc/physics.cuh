// Device physics of the cg-gcmc-bd hot path: pair laws, effective-potential
// table lookup, grid-map gathers, membrane.  FP64 routines keep the
// reference's expression order; FP32 routines are the fast path.
#pragma once
#include "kparams.cuh"

namespace bgpu {

__device__ __forceinline__ double pow3d(double v) { return v * v * v; }
__device__ __forceinline__ double pow6d(double v) {
  double v2 = v * v;
  return v2 * v2 * v2;
}
// 1/sqrt(x) for a positive normal float: the hardware approximation (PTX
// rsqrt.approx.ftz.f32, relative error below 2^-22.9 by the PTX ISA).
// rsqrtf() wraps the same operation in a denormal-input path that pair
// distances and RFPAR denominators never take.
__device__ __forceinline__ float rsqrt_nz(float x) {
  float y;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ float pow3f(float v) { return v * v * v; }
__device__ __forceinline__ float pow6f(float v) {
  float v2 = v * v;
  return v2 * v2 * v2;
}

// ---- tabulated effective potential, FP64 (polynom.f90:197-230) ---------
// Returns U; yp = -(dU/dr)/r; x = r inside the table, else 0.
__device__ __forceinline__ double efp64(const KP &p, const PairParam &q,
                                        double x2, double &yp, double &x,
                                        int &err) {
  x = 0.0;
  if (x2 < q.dm2lo) {
    double ix2 = 1.0 / x2;
    double c = q.sc0 * pow6d(ix2);
    yp = 12.0 * c * ix2;
    return c + q.sc1;
  }
  if (x2 > q.dm2hi) {
    double ix2 = 1.0 / x2;
    double c = q.sc2 * pow3d(ix2);
    if (q.flags & kChr) {
      double f = q.fct * sqrt(ix2);
      yp = (6.0 * c + f) * ix2;
      return c + f;
    }
    yp = 6.0 * c * ix2;
    return c;
  }
  x = sqrt(x2);
  int i = (int)((x - q.dmi) * p.ires) + q.nxi;
  if (i < q.nxi || i >= q.nxi + q.npieces) {
    err |= kErrTableIndex;
    i = min(max(i, q.nxi), q.nxi + q.npieces - 1);
  }
  const double p1 = p.ep[3 * i], p2 = p.ep[3 * i + 1], p3 = p.ep[3 * i + 2];
  yp = -p2 / x - 2.0 * p3;
  return p1 + x * (p2 + x * p3);
}

// ---- tabulated effective potential, FP32 local form ----------------------
// Piece k stored as (a, b, c, x_k): U = a + t (b + t c), t = r - x_k, which
// is the reference's p1 + r (p2 + r p3) re-expanded about the piece's knot so
// that single precision does not lose the cancellation in p1 + r p2 + r^2 p3.
__device__ __forceinline__ float efp32(const KP &p, const PairParamF &q,
                                       float x2, float &yp, int &err) {
  if (x2 < q.dm2lo) {
    float ix2 = 1.0f / x2;
    float c = q.sc0 * pow6f(ix2);
    yp = 12.0f * c * ix2;
    return c + q.sc1;
  }
  if (x2 > q.dm2hi) {
    float ix2 = 1.0f / x2;
    float c = q.sc2 * pow3f(ix2);
    if (q.flags & kChr) {
      float f = q.fct * sqrtf(ix2);
      yp = (6.0f * c + f) * ix2;
      return c + f;
    }
    yp = 6.0f * c * ix2;
    return c;
  }
  float ir = rsqrtf(x2);
  float r = x2 * ir;
  int i = (int)((r - q.dmi) * p.iresf) + q.nxi;
  const int last = q.nxi + (q.flags >> 8) - 1;  // npieces packed in flags
  if (i < q.nxi || i > last) i = min(max(i, q.nxi), last);
  const float4 c = p.ep32[i];
  const float t = r - c.w;
  yp = -(c.y + 2.0f * c.z * t) * ir;
  return c.x + t * (c.y + t * c.z);
}

// ---- analytic pair law, FP64 (energy.mono.f90:135-178) -------------------
// e[0..3] += w * (Coulomb, LJ, SRPMF, table); returns de = -(dU/dr)/r.
// dist (r inside the table, else 0) feeds the PROXDIFF record.
__device__ __forceinline__ double law64(const KP &p, const PairParam &q,
                                        double dist2, double w, double e[4],
                                        double &dist, int &err) {
  dist = 0.0;
  if (q.flags & kEfp) {
    double yp;
    e[3] += w * efp64(p, q, dist2, yp, dist, err);
    return yp;
  }
  double idist2 = 1.0 / dist2, idist = 0.0, de = 0.0;
  if (q.flags & (kChr | kSrp)) idist = sqrt(idist2);
  if (q.flags & kChr) {
    double cofo = q.fct * idist;
    e[0] += w * cofo;
    de = cofo * idist2;
  }
  if (q.flags & kLj) {
    double dist6 = pow3d(q.sgp2 * idist2);
    double dist12 = dist6 * dist6;
    e[1] += w * q.epp4 * (dist12 - dist6);
    de += q.epp4 * (2.0 * dist12 - dist6) * 6.0 * idist2;
  }
  if ((q.flags & kSrp) && dist2 <= p.rth) {
    double r = 1.0 / idist;
    double a = q.c3 * kPi * (q.c1 - r);
    double s, c;
    sincos(a, &s, &c);
    double e1 = exp((q.c1 - r) * q.c2);
    double e3 = pow6d(q.c1 * idist);
    double e0 = q.c0 * e1 * c + q.c4 * e3;
    double dc = (-q.c2 * c + q.c3 * kPi * s) * q.c0 * e1 - 6.0 * q.c4 * e3 * idist;
    if (r >= p.srpx) {
      double fdf = exp(-p.srpk * (r - p.srpx)) - p.srpy;
      dc = dc * fdf - e0 * p.srpk * (fdf + p.srpy);
      e0 = e0 * fdf;
    }
    e[2] += w * e0;
    de -= dc * idist;
  }
  return de;
}

// ---- which SRPMF branch a pair takes, FP32 path --------------------------
// The reference's SRPMF law (energy.mono.f90:147-175) is not continuous at
// its two boundaries: energy and force jump where the taper starts (r =
// srpx), and the force where the law ends (r^2 = rth).  An FP32 r^2 carries a
// relative error of a few 1e-7, so a pair that close to a boundary could take
// the other branch than in FP64 and be off by the whole jump.  Outside a
// window of kSrpWin (relative) around either boundary the FP32 r^2 decides;
// inside it r2d() -- the pair's r^2 in FP64 from its float-float position
// records -- decides, as the FP64 path would.
// Returns 0 beyond rth, 1 inside rth before the taper, 2 in the taper.
// The window's bounds are kernel-parameter constants (srpx2lo/hi, rthlo/hi),
// which the comparisons read directly.
template <class R2D>
__device__ __forceinline__ int srp_branch(const KP &p, float r2, R2D r2d) {
  if (r2 > p.rthhi) return 0;
  if (r2 < p.rthlo) {
    if (r2 >= p.srpx2hi) return 2;
    if (r2 <= p.srpx2lo) return 1;
  }
  const double d = r2d();
  return d > p.rth ? 0 : (d >= p.srpx * p.srpx ? 2 : 1);
}

// r^2 in FP64 of a pair from its float-float records (hi, lo) of the target
// (th, tl) and the source (h, l): every difference of two floats is exact in
// FP64.  s: whole box lengths to take off each component (the periodic
// extension mode's nearest image), zero otherwise.
__device__ __forceinline__ double r2_ff64(const float4 &th, const float4 &tl, const float4 &h,
                                          const float4 &l, double sx = 0.0, double sy = 0.0,
                                          double sz = 0.0) {
  const double dx = ((double)th.x - (double)h.x) + ((double)tl.x - (double)l.x) - sx;
  const double dy = ((double)th.y - (double)h.y) + ((double)tl.y - (double)l.y) - sy;
  const double dz = ((double)th.z - (double)h.z) + ((double)tl.z - (double)l.z) - sz;
  return dx * dx + dy * dy + dz * dz;
}

// ---- analytic pair law, FP32 ---------------------------------------------
template <class R2D>
__device__ __forceinline__ float law32(const KP &p, const PairParamF &q,
                                       float r2, float w, float e[4],
                                       int &err, R2D r2d) {
  if (q.flags & kEfp) {
    float yp;
    e[3] += w * efp32(p, q, r2, yp, err);
    return yp;
  }
  const float ir = rsqrtf(r2);
  const float ir2 = ir * ir;
  float de = 0.0f;
  if (q.flags & kChr) {
    float cofo = q.fct * ir;
    e[0] += w * cofo;
    de = cofo * ir2;
  }
  if (q.flags & kLj) {
    float d6 = pow3f(q.sgp2 * ir2);
    float d12 = d6 * d6;
    e[1] += w * q.epp4 * (d12 - d6);
    de += q.epp4 * 6.0f * ir2 * (2.0f * d12 - d6);
  }
  const int branch = (q.flags & kSrp) && r2 <= p.rthhi ? srp_branch(p, r2, r2d) : 0;
  if (branch) {
    float r = r2 * ir;
    float s, c;
    sincospif(q.c3 * (q.c1 - r), &s, &c);  // cos(c3 pi (c1 - r))
    float e1 = expf((q.c1 - r) * q.c2);
    float e3 = pow6f(q.c1 * ir);
    float e0 = q.c0 * e1 * c + q.c4 * e3;
    float dc = (-q.c2 * c + q.c3 * (float)kPi * s) * q.c0 * e1 - 6.0f * q.c4 * e3 * ir;
    if (branch == 2) {
      float fdf = expf(-p.srpkf * (r - p.srpxf)) - p.srpyf;
      dc = dc * fdf - e0 * p.srpkf * (fdf + p.srpyf);
      e0 = e0 * fdf;
    }
    e[2] += w * e0;
    de -= dc * ir;
  }
  return de;
}

// ---- SRPMF of a pair inside rth, FP32 (energy.mono.f90:147-175):
// c0 exp((c1 - r) c2) cos(c3 pi (c1 - r)) + c4 (c1 / r)^6, tapered when
// branch == 2 (srp_branch), nothing when branch == 0; adds w E to e[2] and
// returns its -(dE/dr)/r term.
__device__ __forceinline__ float srpmf32(const KP &p, int is, float r2, float ir, float w,
                                         float e[4], int branch) {
  if (branch == 0) return 0.0f;
  const float4 *q = p.ppk + 4 * is;
  const float4 q1 = __ldg(q + 1);
  const float c4 = __ldg(q + 2).x;
  const float r = r2 * ir;
  float s, c;
  sincospif(q1.w * (q1.y - r), &s, &c);
  const float e1 = expf((q1.y - r) * q1.z);
  const float e3 = pow6f(q1.y * ir);
  float e0 = q1.x * e1 * c + c4 * e3;
  float dc = (-q1.z * c + q1.w * (float)kPi * s) * q1.x * e1 - 6.0f * c4 * e3 * ir;
  if (branch == 2) {
    const float fdf = expf(-p.srpkf * (r - p.srpxf)) - p.srpyf;
    dc = dc * fdf - e0 * p.srpkf * (fdf + p.srpyf);
    e0 = e0 * fdf;
  }
  e[2] = fmaf(w, e0, e[2]);
  return -dc * ir;
}

// ---- analytic pair law, FP32, packed table (p.ppk) ----------------------
// The common Coulomb + LJ path needs one 16-byte load per pair; SRPMF
// coefficients and the table constants are fetched only when used.
template <class R2D>
__device__ __forceinline__ float law32k(const KP &p, int is, float r2, float w,
                                        float e[4], R2D r2d) {
  const float4 *q = p.ppk + 4 * is;
  const float4 q0 = __ldg(q);
  const int fl = __float_as_int(q0.w);
  if (fl & kEfp) {
    const float4 q2 = __ldg(q + 2), q3 = __ldg(q + 3);
    float y, yp;
    if (r2 < q3.x) {
      const float ix2 = 1.0f / r2;
      const float c = q2.y * pow6f(ix2);
      yp = 12.0f * c * ix2;
      y = c + q2.z;
    } else if (r2 > q3.y) {
      const float ix2 = 1.0f / r2;
      const float c = q2.w * pow3f(ix2);
      if (fl & kChr) {
        const float f = q0.x * sqrtf(ix2);
        yp = (6.0f * c + f) * ix2;
        y = c + f;
      } else {
        yp = 6.0f * c * ix2;
        y = c;
      }
    } else {
      const float ir = rsqrtf(r2), r = r2 * ir;
      const int nxi = __float_as_int(q3.w), last = nxi + (fl >> 8) - 1;
      int i = (int)((r - q3.z) * p.iresf) + nxi;
      i = min(max(i, nxi), last);
      const float4 c = __ldg(p.ep32 + i);
      const float t = r - c.w;
      yp = -(c.y + 2.0f * c.z * t) * ir;
      y = c.x + t * (c.y + t * c.z);
    }
    e[3] = fmaf(w, y, e[3]);
    return yp;
  }
  const float ir = rsqrtf(r2), ir2 = ir * ir;
  float de = 0.0f;
  if (fl & kChr) {
    const float cofo = q0.x * ir;
    e[0] = fmaf(w, cofo, e[0]);
    de = cofo * ir2;
  }
  if (fl & kLj) {
    const float d6 = pow3f(q0.z * ir2), d12 = d6 * d6;
    e[1] = fmaf(w, q0.y * (d12 - d6), e[1]);
    de = fmaf(q0.y * 6.0f * ir2, 2.0f * d12 - d6, de);
  }
  if ((fl & kSrp) && r2 <= p.rthhi)
    de += srpmf32(p, is, r2, ir, w, e, srp_branch(p, r2, r2d));
  return de;
}

// ---- pair energy as INTERACT computes it (interact.f90:181-205) ----------
// Note the SRPMF taper differs from ENERGY: e*exp(-k(r-x)) - y.
__device__ __forceinline__ double law_interact64(const KP &p,
                                                 const PairParam &q,
                                                 double dist2, int &err) {
  if (q.flags & kEfp) {
    double yp, x;
    return efp64(p, q, dist2, yp, x, err);
  }
  double idist2 = 1.0 / dist2, idist = 0.0, u = 0.0;
  if (q.flags & (kChr | kSrp)) idist = sqrt(idist2);
  if (q.flags & kChr) u += q.fct * idist;
  if (q.flags & kLj) {
    double dist6 = pow3d(q.sgp2 * idist2);
    u += q.epp4 * dist6 * (dist6 - 1.0);
  }
  if ((q.flags & kSrp) && dist2 <= p.rth) {
    double r = 1.0 / idist;
    double es = q.c0 * exp((q.c1 - r) * q.c2) * cos(q.c3 * kPi * (q.c1 - r)) +
                q.c4 * pow6d(q.c1 * idist);
    if (r >= p.srpx) es = es * exp(-p.srpk * (r - p.srpx)) - p.srpy;
    u += es;
  }
  return u;
}

// ---- switching functions (switch1.f90, switch2.f90) ----------------------
__device__ __forceinline__ void switch1(double &sw, double &dsw, double z,
                                        double p1, double ip1, double zm1,
                                        double zm2) {
  if (z >= zm2 + p1 || z <= zm1 - p1) {
    sw = 0.0;
    dsw = 0.0;
  } else if (z > zm2) {
    double d = (z - zm2) * ip1;
    sw = 1.0 + (2.0 * d - 3.0) * d * d;
    dsw = -6.0 * (d - 1.0) * ip1 * d;
  } else if (z < zm1) {
    double d = (zm1 - z) * ip1;
    sw = 1.0 + (2.0 * d - 3.0) * d * d;
    dsw = 6.0 * (d - 1.0) * ip1 * d;
  } else {
    sw = 1.0;
    dsw = 0.0;
  }
}

__device__ __forceinline__ void switch2(double &sw, double &dsw, double r2,
                                        double radius, double p2, double ip2,
                                        double &r) {
  if (r2 <= radius * radius) {
    sw = 0.0;
    dsw = 0.0;
  } else if (r2 < (radius + p2) * (radius + p2)) {
    r = sqrt(r2);
    double d = (radius + p2 - r) * ip2;
    sw = 1.0 + (2.0 * d - 3.0) * d * d;
    dsw = 6.0 * (d - 1.0) * d * ip2;
  } else {
    sw = 1.0;
    dsw = 0.0;
  }
}

// ---- membrane, one particle (membrane.f90:36-107) -------------------------
// Adds to e and f; returns 1 when the particle sits inside the membrane
// (the reference's warning counter).  With `single` the INTERACT variant
// (interact.f90:59-119) is used: no forces, 1e10 inside the membrane.
__device__ __forceinline__ int membrane_one(const KP &p, int itype,
                                            double charge, double x, double y,
                                            double z, bool lgiat, bool single,
                                            double &e, double f[3]) {
  int warn = 0;
  if (p.voltage != 0.0 && charge != 0.0) {
    if (z < p.zmemb1) {
      double ex = exp(p.ikappa * (z - p.zmemb1));
      e += charge * p.afact * ex;
      if (lgiat) f[2] -= charge * p.afact * p.ikappa * ex;
    } else if (z >= p.zmemb1 && z <= p.zmemb2) {
      e += charge * p.afact * (p.ceps * p.ikappa * (z - p.zmemb1) + 1.0);
      if (lgiat) f[2] -= charge * p.afact * p.ceps * p.ikappa;
    } else if (z > p.zmemb2) {
      double ex = exp(-p.ikappa * (z - p.zmemb2));
      e += charge * (p.voltage - p.afact * ex);
      if (lgiat) f[2] -= charge * p.afact * p.ikappa * ex;
    }
  }
  const double a1 = p.ampl1[itype];
  if (a1 > 0.0) {
    double sw1, dsw1;
    switch1(sw1, dsw1, z, p.p1a[itype], p.p1b[itype], p.zmemb1, p.zmemb2);
    if (sw1 != 0.0) {
      const double a2 = p.ampl2[itype];
      if (p.qpore) {
        double sw2, dsw2, r = 0.0;
        switch2(sw2, dsw2, x * x + y * y, p.rcyl[itype], p.p2a[itype],
                p.p2b[itype], r);
        if (sw2 != 0.0) {
          if (sw1 == 1.0) {
            if (sw2 == 1.0) {
              warn = 1;
              e += single ? 1.0e10 : a2;
            } else {
              if (lgiat) {
                double ir = 1.0 / r;
                f[0] += a2 * dsw2 * x * ir;
                f[1] += a2 * dsw2 * y * ir;
              }
              e += a2 * sw2;
            }
          } else {
            if (sw2 == 1.0) {
              if (lgiat) f[2] += a1 * dsw1;
              e += a1 * sw1;
            } else {
              if (lgiat) {
                double ir = 1.0 / r;
                f[0] += 0.5 * a2 * dsw2 * x * ir;
                f[1] += 0.5 * a2 * dsw2 * y * ir;
                f[2] += 0.5 * a1 * dsw1;
              }
              e += 0.5 * (a2 * sw2 + a1 * sw1);
            }
          }
        }
      } else {
        if (sw1 == 1.0) {
          warn = 1;
          e += single ? 1.0e10 : a1 * sw1;
        } else {
          e += a1 * sw1;
        }
      }
    }
  }
  return warn;
}

__device__ __forceinline__ bool in_grid(const Grid3 &g, double x, double y,
                                        double z) {
  return x <= g.xbcen + g.tranx && x >= g.xbcen - g.tranx &&
         y <= g.ybcen + g.trany && y >= g.ybcen - g.trany &&
         z <= g.zbcen + g.tranz && z >= g.zbcen - g.tranz;
}

__device__ __forceinline__ void cell_of(const Grid3 &g, double xi, double yi,
                                        double zi, int &ix, int &iy, int &iz) {
  ix = (int)(xi * g.idcel);
  iy = (int)(yi * g.idcel);
  iz = (int)(zi * g.idcel);
  if (ix == g.nclx - 1) ix = g.nclx - 2;
  if (iy == g.ncly - 1) iy = g.ncly - 2;
  if (iz == g.nclz - 1) iz = g.nclz - 2;
}

// ---- static field, one particle (staticf1.f90:66-115) ---------------------
__device__ __forceinline__ void staticf_one(const KP &p, double x, double y,
                                            double z, double chi, bool qf,
                                            double &e, double f[3]) {
  const Grid3 &g = p.g1;
  if (!in_grid(g, x, y, z)) return;
  const int ncyz = g.ncly * g.nclz;
  const double xi = x + g.tranx - g.xbcen, yi = y + g.trany - g.ybcen,
               zi = z + g.tranz - g.zbcen;
  int ix, iy, iz;
  cell_of(g, xi, yi, zi, ix, iy, iz);
  const double pre = p.celec * chi;
#pragma unroll
  for (int a = 0; a < 2; ++a) {
    double ai = xi - (ix + a) * g.dcel;
    const double as = fsign(1.0, ai);
    ai = 1.0 - fabs(ai) * g.idcel;
#pragma unroll
    for (int b = 0; b < 2; ++b) {
      double bi = yi - (iy + b) * g.dcel;
      const double bs = fsign(1.0, bi);
      bi = 1.0 - fabs(bi) * g.idcel;
      const size_t row = (size_t)(ix + a) * ncyz + (size_t)(iy + b) * g.nclz + iz;
      const float2 ph = make_float2(__ldg(p.phix + row), __ldg(p.phix + row + 1));
#pragma unroll
      for (int c = 0; c < 2; ++c) {
        double ci = zi - (iz + c) * g.dcel;
        const double cs = fsign(1.0, ci);
        ci = 1.0 - fabs(ci) * g.idcel;
        const double phi = (double)(c ? ph.y : ph.x);
        if (qf) {
          const double prefac = phi * pre * g.idcel;
          if (ai < 1.0 - kRsmall && ai > kRsmall) f[0] += as * bi * ci * prefac;
          if (bi < 1.0 - kRsmall && bi > kRsmall) f[1] += bs * ai * ci * prefac;
          if (ci < 1.0 - kRsmall && ci > kRsmall) f[2] += cs * ai * bi * prefac;
        }
        e += ai * bi * ci * chi * phi * p.celec;
      }
    }
  }
}

// ---- repulsion map, trilinear (vdwgd1trln.f90:57-158) --------------------
// Returns the corner sum (phisum) for the warning threshold.
__device__ __forceinline__ double vdwgd_trln_one(const KP &p, double xi,
                                                 double yi, double zi,
                                                 size_t ifir, double esvdw,
                                                 bool qf, double &e,
                                                 double f[3]) {
  const Grid3 &g = p.g2;
  const int ncyz = g.ncly * g.nclz;
  int ix, iy, iz;
  cell_of(g, xi, yi, zi, ix, iy, iz);
  double phisum = 0.0;
#pragma unroll
  for (int a = 0; a < 2; ++a) {
    double ai = xi - (ix + a) * g.dcel;
    const double as = fsign(1.0, ai);
    ai = 1.0 - fabs(ai) * g.idcel;
#pragma unroll
    for (int b = 0; b < 2; ++b) {
      double bi = yi - (iy + b) * g.dcel;
      const double bs = fsign(1.0, bi);
      bi = 1.0 - fabs(bi) * g.idcel;
      const size_t row = ifir + (size_t)(ix + a) * ncyz + (size_t)(iy + b) * g.nclz + iz;
#pragma unroll
      for (int c = 0; c < 2; ++c) {
        double ci = zi - (iz + c) * g.dcel;
        const double cs = fsign(1.0, ci);
        ci = 1.0 - fabs(ci) * g.idcel;
        const double phis = (double)__ldg(p.phiv + row + c);
        phisum += phis;
        if (qf) {
          const double prefac = phis * esvdw * g.idcel;
          if (ai < 1.0 - kRsmall && ai > kRsmall) f[0] += as * bi * ci * prefac;
          if (bi < 1.0 - kRsmall && bi > kRsmall) f[1] += bs * ai * ci * prefac;
          if (ci < 1.0 - kRsmall && ci > kRsmall) f[2] += cs * ai * bi * prefac;
        }
        e += ai * bi * ci * esvdw * phis;
      }
    }
  }
  return phisum;
}

// quadratic B-spline and derivative (m3.f90, dm3.f90)
__device__ __forceinline__ double m3(double x) {
  double m2m = (x >= 0.0 && x <= 2.0) ? 1.0 - fabs(x - 1.0) : 0.0;
  double m2 = (x >= 1.0 && x <= 3.0) ? 1.0 - fabs(x - 2.0) : 0.0;
  return (x >= 0.0 && x <= 3.0) ? x * 0.5 * m2m + (3.0 - x) * 0.5 * m2 : 0.0;
}
__device__ __forceinline__ double dm3(double x) {
  double m2m = (x >= 0.0 && x <= 2.0) ? 1.0 - fabs(x - 1.0) : 0.0;
  double m2 = (x >= 1.0 && x <= 3.0) ? 1.0 - fabs(x - 2.0) : 0.0;
  return m2m - m2;
}

__device__ __forceinline__ void spln_cell(const Grid3 &g, double xi, double yi,
                                          double zi, int &ix, int &iy,
                                          int &iz) {
  ix = (int)llround(xi * g.idcel);  // nint: half away from zero
  iy = (int)llround(yi * g.idcel);
  iz = (int)llround(zi * g.idcel);
  if (ix == 0) ix = 1;
  if (iy == 0) iy = 1;
  if (iz == 0) iz = 1;
  if (ix == g.nclx - 1) ix = g.nclx - 2;
  if (iy == g.ncly - 1) iy = g.ncly - 2;
  if (iz == g.nclz - 1) iz = g.nclz - 2;
}

// ---- repulsion map, 27-point B-spline (vdwgd1spln.f90:57-167) ------------
__device__ __forceinline__ double vdwgd_spln_one(const KP &p, double xi,
                                                 double yi, double zi,
                                                 size_t ifir, double esvdw,
                                                 bool qf, double &e,
                                                 double f[3]) {
  const Grid3 &g = p.g2;
  const int ncyz = g.ncly * g.nclz;
  int ix, iy, iz;
  spln_cell(g, xi, yi, zi, ix, iy, iz);
  double phisum = 0.0;
  for (int k = ix - 1; k <= ix + 1; ++k) {
    double ai = 1.5 - (xi - k * g.dcel) * g.idcel;
    const double dai = dm3(ai);
    ai = m3(ai);
    if (!(ai != 0.0 || dai != 0.0)) continue;
    for (int l = iy - 1; l <= iy + 1; ++l) {
      double bi = 1.5 - (yi - l * g.dcel) * g.idcel;
      const double dbi = dm3(bi);
      bi = m3(bi);
      if (!(bi != 0.0 || dbi != 0.0)) continue;
      for (int m = iz - 1; m <= iz + 1; ++m) {
        double ci = 1.5 - (zi - m * g.dcel) * g.idcel;
        const double dci = dm3(ci);
        ci = m3(ci);
        if (!(ci != 0.0 || dci != 0.0)) continue;
        const double phivi =
            (double)__ldg(p.phiv + ifir + (size_t)k * ncyz + (size_t)l * g.nclz + m);
        const double phivsv = phivi * esvdw;
        phisum += phivi;
        if (qf) {
          const double prefac = phivsv * g.idcel;
          f[0] += dai * bi * ci * prefac;
          f[1] += ai * dbi * ci * prefac;
          f[2] += ai * bi * dci * prefac;
        }
        e += ai * bi * ci * phivsv;
      }
    }
  }
  return phisum;
}

// ---- single-particle B-spline repulsion energy (vdwgd0spln.f90:83-128) ---
__device__ __forceinline__ double vdwgd_spln0(const KP &p, double xi,
                                              double yi, double zi,
                                              size_t ifir, double esvdw,
                                              double &e) {
  const Grid3 &g = p.g2;
  const int ncyz = g.ncly * g.nclz;
  int ix, iy, iz;
  spln_cell(g, xi, yi, zi, ix, iy, iz);
  double phisum = 0.0;
  for (int k = ix - 1; k <= ix + 1; ++k) {
    const double ai = m3(1.5 - (xi - k * g.dcel) * g.idcel);
    if (ai == 0.0) continue;
    for (int l = iy - 1; l <= iy + 1; ++l) {
      const double bi = m3(1.5 - (yi - l * g.dcel) * g.idcel);
      if (bi == 0.0) continue;
      for (int m = iz - 1; m <= iz + 1; ++m) {
        const double fi = ai * bi * m3(1.5 - (zi - m * g.dcel) * g.idcel);
        if (fi != 0.0) {
          const double phis =
              (double)__ldg(p.phiv + ifir + (size_t)k * ncyz + (size_t)l * g.nclz + m);
          phisum += phis;
          e += fi * esvdw * phis;
        }
      }
    }
  }
  return phisum;
}

// Map offset, scale and combined type of particle i (0-based) for the
// repulsion map (vdwgd1trln.f90:61-92); iontype = |typei| for ions.
__device__ __forceinline__ void phiv_select(const KP &p, int i, int iontype,
                                            size_t &ifir, double &esvdw,
                                            int &itype2) {
  const size_t ncel3 = (size_t)p.g2.nclx * p.g2.ncly * p.g2.nclz;
  itype2 = i < p.nsites ? p.typtyp[i] : p.nwtype[iontype];
  esvdw = p.svdw;
  ifir = 0;
  if (p.qnmcden) {
    if (i < p.nsites)
      ifir = p.site_map ? (size_t)p.site_map[i] * ncel3 : 0;
    else if (i >= p.nsites + p.nfix)
      ifir = (size_t)p.phiv_map_of_type[iontype] * ncel3;
  } else if (p.qsvdw) {
    esvdw = p.svdw * p.scal[itype2];
  }
}

// ---- RFPAR gather (rfpar.f90:94-150) with the reference's early exit of
// the innermost loop on a zero gsrfen value ---------------------------------
__device__ __forceinline__ void rfpar_gather(const KP &p, double x, double y,
                                             double z, size_t ifir, bool qf,
                                             double &aux1, double &aux2,
                                             double d1[3], double d2[3]) {
  const Grid3 &g = p.g3;
  const int ncyz = g.ncly * g.nclz;
  aux1 = aux2 = 0.0;
  d1[0] = d1[1] = d1[2] = d2[0] = d2[1] = d2[2] = 0.0;
  const double xi = x + g.tranx - g.xbcen, yi = y + g.trany - g.ybcen,
               zi = z + g.tranz - g.zbcen;
  int ix, iy, iz;
  cell_of(g, xi, yi, zi, ix, iy, iz);
#pragma unroll
  for (int a = 0; a < 2; ++a) {
    double ai = xi - (ix + a) * g.dcel;
    const double as = fsign(1.0, ai);
    ai = 1.0 - fabs(ai) * g.idcel;
#pragma unroll
    for (int b = 0; b < 2; ++b) {
      double bi = yi - (iy + b) * g.dcel;
      const double bs = fsign(1.0, bi);
      bi = 1.0 - fabs(bi) * g.idcel;
      const size_t row = ifir + (size_t)(ix + a) * ncyz + (size_t)(iy + b) * g.nclz + iz;
#pragma unroll
      for (int c = 0; c < 2; ++c) {
        double ci = zi - (iz + c) * g.dcel;
        const double cs = fsign(1.0, ci);
        ci = 1.0 - fabs(ci) * g.idcel;
        const double gaux1 = (double)__ldg(p.gsrfen + row + c);
        if (gaux1 == 0.0) break;
        const double gaux2 = p.sqrfac * (double)__ldg(p.greff + row + c);
        const double fi = ai * bi * ci;
        aux1 += fi * gaux1;
        aux2 += fi * gaux2;
        if (qf) {
          const double pa1 = gaux1 * g.idcel, pa2 = gaux2 * g.idcel;
          if (ai < 1.0 - kRsmall && ai > kRsmall) {
            const double t = as * bi * ci;
            d1[0] -= t * pa1;
            d2[0] -= t * pa2;
          }
          if (bi < 1.0 - kRsmall && bi > kRsmall) {
            const double t = bs * ai * ci;
            d1[1] -= t * pa1;
            d2[1] -= t * pa2;
          }
          if (ci < 1.0 - kRsmall && ci > kRsmall) {
            const double t = cs * ai * bi;
            d1[2] -= t * pa1;
            d2[2] -= t * pa2;
          }
        }
      }
    }
  }
}

__device__ __forceinline__ size_t rfpar_ifir(const KP &p, int itype) {
  const size_t ncel3 = (size_t)p.g3.nclx * p.g3.ncly * p.g3.nclz;
  return p.qrfpsin ? 0 : (size_t)p.rfpar_map_of_type[itype] * ncel3;
}

// ---- block reductions (fixed tree: deterministic for a fixed blockDim) --
// Sums v[0..N) over the block; the totals land in the SHARED array out[N],
// visible to every thread on return.  smem: (blockDim.x/32) * N doubles.
template <int N>
__device__ __forceinline__ void block_sum(const double v[N], double *smem,
                                          double *out) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int nw = (blockDim.x + 31) >> 5;
#pragma unroll
  for (int k = 0; k < N; ++k) {
    double x = v[k];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if (lane == 0) smem[wid * N + k] = x;
  }
  __syncthreads();
  if (threadIdx.x < N) {
    double s = 0.0;
    for (int w = 0; w < nw; ++w) s += smem[w * N + threadIdx.x];
    out[threadIdx.x] = s;
  }
  __syncthreads();
}

// Bounds guard of the GCMC/INTERACT kernels: records the first violation
// (site code, index, bound) in DevState and tells the caller to skip.
__device__ __forceinline__ bool guard_bad(DevState *st, long long idx,
                                          long long bound, int site) {
  if (idx >= 0 && idx < bound) return false;
  if (atomicCAS(&st->bad_site, 0, site) == 0) {
    st->bad_index = (int)idx;
    st->bad_bound = (int)bound;
  }
  atomicOr(&st->err, kErrBounds);
  return true;
}

}  // namespace bgpu
