// ORACLE -- test infrastructure only (see ref_state.h).
// Grid-map gathers, membrane, reaction-field parameters and INTERACT.
#include <cmath>

#include "ref_state.h"

namespace bref {

static inline double fsign(double a, double b) {  // Fortran SIGN(a, b)
  return b >= 0.0 ? std::fabs(a) : -std::fabs(a);
}

// switch1.f90:19-48
void switch1(double &sw, double &dsw, double z, double p1, double ip1,
             double zmemb1, double zmemb2) {
  if (z >= zmemb2 + p1 || z <= zmemb1 - p1) {
    sw = 0.0;
    dsw = 0.0;
  } else if (z > zmemb2) {
    double delzp1 = (z - zmemb2) * ip1;
    sw = 1.0 + (2.0 * delzp1 - 3.0) * delzp1 * delzp1;
    dsw = -6.0 * (delzp1 - 1.0) * ip1 * delzp1;
  } else if (z < zmemb1) {
    double delzp1 = (zmemb1 - z) * ip1;
    sw = 1.0 + (2.0 * delzp1 - 3.0) * delzp1 * delzp1;
    dsw = 6.0 * (delzp1 - 1.0) * ip1 * delzp1;
  } else {
    sw = 1.0;
    dsw = 0.0;
  }
}

// switch2.f90:19-39
void switch2(double &sw, double &dsw, double r2, double radius, double p2,
             double ip2, double &r) {
  if (r2 <= radius * radius) {
    sw = 0.0;
    dsw = 0.0;
  } else if (r2 < (radius + p2) * (radius + p2)) {
    r = std::sqrt(r2);
    double delrp2 = (radius + p2 - r) * ip2;
    sw = 1.0 + (2.0 * delrp2 - 3.0) * delrp2 * delrp2;
    dsw = 6.0 * (delrp2 - 1.0) * delrp2 * ip2;
  } else {
    sw = 1.0;
    dsw = 0.0;
  }
}

// membrane.f90:19-110
void membrane(State &s, bool qforces) {
  s.ememb = 0.0;
  for (int iat = 1; iat <= s.ntot; ++iat) {
    bool lgiat = (iat <= s.nsites || iat >= s.nsites + s.nfix + 1) && qforces;
    int itype;
    double charge;
    if (iat <= s.nsites) {
      itype = s.typtyp[iat];
      charge = s.sitecharge[iat];
    } else {
      int itype2 = std::abs(s.typei[iat]);
      charge = s.cg[itype2];
      itype = s.nwtype[itype2];
    }
    const double zi = s.z[iat];
    if (s.voltage != 0.0 && charge != 0.0) {
      if (zi < s.zmemb1) {
        double e = std::exp(s.ikappa * (zi - s.zmemb1));
        s.ememb += charge * s.afact * e;
        if (lgiat) s.fz[iat] -= charge * s.afact * s.ikappa * e;
      } else if (zi >= s.zmemb1 && zi <= s.zmemb2) {
        s.ememb += charge * s.afact * (s.ceps * s.ikappa * (zi - s.zmemb1) + 1.0);
        if (lgiat) s.fz[iat] -= charge * s.afact * s.ceps * s.ikappa;
      } else if (zi > s.zmemb2) {
        double e = std::exp(-s.ikappa * (zi - s.zmemb2));
        s.ememb += charge * (s.voltage - s.afact * e);
        if (lgiat) s.fz[iat] -= charge * s.afact * s.ikappa * e;
      }
    }
    if (s.ampl1[itype] > 0.0) {
      double sw1, dsw1;
      switch1(sw1, dsw1, zi, s.p1a[itype], s.p1b[itype], s.zmemb1, s.zmemb2);
      if (sw1 != 0.0) {
        if (s.qpore) {
          double r2 = s.x[iat] * s.x[iat] + s.y[iat] * s.y[iat];
          double sw2, dsw2, r = 0.0;
          switch2(sw2, dsw2, r2, s.rcylinder[itype], s.p2a[itype],
                  s.p2b[itype], r);
          if (sw2 != 0.0) {
            if (sw1 == 1.0) {
              if (sw2 == 1.0) {
                s.warn[itype] += 1;
                s.ememb += s.ampl2[itype];
              } else {
                if (lgiat) {
                  double ir = 1.0 / r;
                  s.fx[iat] += s.ampl2[itype] * dsw2 * s.x[iat] * ir;
                  s.fy[iat] += s.ampl2[itype] * dsw2 * s.y[iat] * ir;
                }
                s.ememb += s.ampl2[itype] * sw2;
              }
            } else {
              if (sw2 == 1.0) {
                if (lgiat) s.fz[iat] += s.ampl1[itype] * dsw1;
                s.ememb += s.ampl1[itype] * sw1;
              } else {
                if (lgiat) {
                  double ir = 1.0 / r;
                  s.fx[iat] += 0.5 * s.ampl2[itype] * dsw2 * s.x[iat] * ir;
                  s.fy[iat] += 0.5 * s.ampl2[itype] * dsw2 * s.y[iat] * ir;
                  s.fz[iat] += 0.5 * s.ampl1[itype] * dsw1;
                }
                s.ememb += 0.5 * (s.ampl2[itype] * sw2 + s.ampl1[itype] * sw1);
              }
            }
          }
        } else {
          if (sw1 == 1.0) s.warn[itype] += 1;
          s.ememb += s.ampl1[itype] * sw1;
        }
      }
    }
  }
}

// staticf1.f90:19-121
void staticf1(State &s, bool qforces) {
  const Grid &g = s.g1;
  const int ncyz = g.ncly * g.nclz;
  s.egsbpa = 0.0;
  for (int i = 1; i <= s.ntot; ++i) {
    if (!(i <= s.nsites || i > s.nsites + s.nfix)) continue;
    bool ok = false;
    double chi = 0.0;
    if (i <= s.nsites) {
      if (s.sitecharge[i] != 0.0) {  // namsite(i) == 'P '
        chi = s.sitecharge[i];
        ok = true;
      }
    } else {
      chi = s.cg[std::abs(s.typei[i])];
      ok = true;
    }
    if (ok)
      ok = s.x[i] <= g.xbcen + g.tranx && s.x[i] >= g.xbcen - g.tranx &&
           s.y[i] <= g.ybcen + g.trany && s.y[i] >= g.ybcen - g.trany &&
           s.z[i] <= g.zbcen + g.tranz && s.z[i] >= g.zbcen - g.tranz;
    if (!ok) continue;
    double rxnfx = 0.0, rxnfy = 0.0, rxnfz = 0.0;
    double xi = s.x[i] + g.tranx - g.xbcen;
    double yi = s.y[i] + g.trany - g.ybcen;
    double zi = s.z[i] + g.tranz - g.zbcen;
    int ix = (int)(xi * g.idcel), iy = (int)(yi * g.idcel),
        iz = (int)(zi * g.idcel);
    if (ix == g.nclx - 1) ix = g.nclx - 2;
    if (iy == g.ncly - 1) iy = g.ncly - 2;
    if (iz == g.nclz - 1) iz = g.nclz - 2;
    for (int n1 = ix; n1 <= ix + 1; ++n1) {
      double ai = xi - n1 * g.dcel;
      double aisign = fsign(1.0, ai);
      ai = 1.0 - std::fabs(ai) * g.idcel;
      for (int n2 = iy; n2 <= iy + 1; ++n2) {
        double bi = yi - n2 * g.dcel;
        double bisign = fsign(1.0, bi);
        bi = 1.0 - std::fabs(bi) * g.idcel;
        for (int n3 = iz; n3 <= iz + 1; ++n3) {
          double ci = zi - n3 * g.dcel;
          double cisign = fsign(1.0, ci);
          ci = 1.0 - std::fabs(ci) * g.idcel;
          double fi = ai * bi * ci;
          double phi = (double)s.phix[(size_t)n1 * ncyz + n2 * g.nclz + n3];
          if (qforces) {
            double prefac = phi * s.celec * chi * g.idcel;
            if (ai < 1.0 - rsmall && ai > rsmall) rxnfx += aisign * bi * ci * prefac;
            if (bi < 1.0 - rsmall && bi > rsmall) rxnfy += bisign * ai * ci * prefac;
            if (ci < 1.0 - rsmall && ci > rsmall) rxnfz += cisign * ai * bi * prefac;
          }
          s.egsbpa += fi * chi * phi * s.celec;
        }
      }
    }
    if (qforces) {
      s.fx[i] += rxnfx;
      s.fy[i] += rxnfy;
      s.fz[i] += rxnfz;
    }
  }
}

// staticf0.f90:19-85
void staticf0(State &s, double xj, double yj, double zj, int j, int jtype) {
  const Grid &g = s.g1;
  s.egsbpa = 0.0;
  bool beion = s.qpar() && j > s.nsites;
  bool besite = s.qnucl() && j <= s.nsites && s.sitecharge[j] != 0.0;
  bool ok = beion || besite;
  double chi = 0.0;
  if (beion) chi = s.cg[jtype];
  if (besite) chi = s.sitecharge[j];
  if (ok)
    ok = xj <= g.xbcen + g.tranx && xj >= g.xbcen - g.tranx &&
         yj <= g.ybcen + g.trany && yj >= g.ybcen - g.trany &&
         zj <= g.zbcen + g.tranz && zj >= g.zbcen - g.tranz;
  if (!ok) return;
  const int ncyz = g.ncly * g.nclz;
  double xi = xj + g.tranx - g.xbcen, yi = yj + g.trany - g.ybcen,
         zi = zj + g.tranz - g.zbcen;
  int ix = (int)(xi * g.idcel), iy = (int)(yi * g.idcel), iz = (int)(zi * g.idcel);
  if (ix == g.nclx - 1) ix = g.nclx - 2;
  if (iy == g.ncly - 1) iy = g.ncly - 2;
  if (iz == g.nclz - 1) iz = g.nclz - 2;
  for (int n1 = ix; n1 <= ix + 1; ++n1) {
    double ai = 1.0 - std::fabs(xi - n1 * g.dcel) * g.idcel;
    for (int n2 = iy; n2 <= iy + 1; ++n2) {
      double bi = 1.0 - std::fabs(yi - n2 * g.dcel) * g.idcel;
      for (int n3 = iz; n3 <= iz + 1; ++n3) {
        double ci = 1.0 - std::fabs(zi - n3 * g.dcel) * g.idcel;
        double fi = ai * bi * ci;
        s.egsbpa += fi * chi *
                    (double)s.phix[(size_t)n1 * ncyz + n2 * g.nclz + n3] *
                    s.celec;
      }
    }
  }
}

// Map offset and scale of one particle for the repulsion map
// (vdwgd1trln.f90:61-92 / vdwgd0trln.f90:55-80).
static void phiv_select(const State &s, int i, int iontype, int &ifir,
                        double &esvdw, int &itype2) {
  const int ncel3 = s.g2.nclx * s.g2.ncly * s.g2.nclz;
  if (i <= s.nsites)
    itype2 = s.typtyp[i];
  else
    itype2 = s.nwtype[iontype];
  esvdw = s.svdw;
  if (s.qnmcden) {
    // fixed ions keep ifir = 0 (no branch of vdwgd0trln.f90:56-77 matches)
    if (i <= s.nsites)
      ifir = s.site_phiv_map[i] * ncel3;
    else if (i > s.nsites + s.nfix)
      ifir = s.phiv_map_of_type[iontype] * ncel3;
  } else if (s.qsvdw) {
    esvdw = s.svdw * s.scal[itype2];
  }
}

// m3.f90 / dm3.f90: quadratic B-spline and its derivative
static double m3(double x) {
  double m2m = (x >= 0.0 && x <= 2.0) ? 1.0 - std::fabs(x - 1.0) : 0.0;
  double m2 = (x >= 1.0 && x <= 3.0) ? 1.0 - std::fabs(x - 2.0) : 0.0;
  if (x >= 0.0 && x <= 3.0) return x * 0.5 * m2m + (3.0 - x) * 0.5 * m2;
  return 0.0;
}
static double dm3(double x) {
  double m2m = (x >= 0.0 && x <= 2.0) ? 1.0 - std::fabs(x - 1.0) : 0.0;
  double m2 = (x >= 1.0 && x <= 3.0) ? 1.0 - std::fabs(x - 2.0) : 0.0;
  return m2m - m2;
}

// vdwgd1trln.f90:19-164
void vdwgd1trln(State &s, bool qforces) {
  const Grid &g = s.g2;
  const int ncyz = g.ncly * g.nclz;
  s.evdwgd = 0.0;
  for (int i = 1; i <= s.ntot; ++i) {
    if (!(i <= s.nsites || i > s.nsites + s.nfix)) continue;
    bool ok = s.x[i] <= g.xbcen + g.tranx && s.x[i] >= g.xbcen - g.tranx &&
              s.y[i] <= g.ybcen + g.trany && s.y[i] >= g.ybcen - g.trany &&
              s.z[i] <= s.vzmax && s.z[i] >= s.vzmin;
    if (!ok) continue;
    double xi = s.x[i] + g.tranx - g.xbcen, yi = s.y[i] + g.trany - g.ybcen,
           zi = s.z[i] + g.tranz - g.zbcen;
    int ifir = 0, itype2 = 0;
    double esvdw;
    phiv_select(s, i, i > s.nsites ? std::abs(s.typei[i]) : 0, ifir, esvdw,
                itype2);
    double vdwfx = 0.0, vdwfy = 0.0, vdwfz = 0.0;
    int ix = (int)(xi * g.idcel), iy = (int)(yi * g.idcel), iz = (int)(zi * g.idcel);
    if (ix == g.nclx - 1) ix = g.nclx - 2;
    if (iy == g.ncly - 1) iy = g.ncly - 2;
    if (iz == g.nclz - 1) iz = g.nclz - 2;
    double phisum = 0.0;
    for (int n1 = ix; n1 <= ix + 1; ++n1) {
      double ai = xi - n1 * g.dcel;
      double aisign = fsign(1.0, ai);
      ai = 1.0 - std::fabs(ai) * g.idcel;
      for (int n2 = iy; n2 <= iy + 1; ++n2) {
        double bi = yi - n2 * g.dcel;
        double bisign = fsign(1.0, bi);
        bi = 1.0 - std::fabs(bi) * g.idcel;
        for (int n3 = iz; n3 <= iz + 1; ++n3) {
          double ci = zi - n3 * g.dcel;
          double cisign = fsign(1.0, ci);
          ci = 1.0 - std::fabs(ci) * g.idcel;
          double fi = ai * bi * ci;
          double phis =
              (double)s.phiv[(size_t)ifir + (size_t)n1 * ncyz + n2 * g.nclz + n3];
          phisum += phis;
          if (qforces) {
            double prefac = phis * esvdw * g.idcel;
            if (ai < 1.0 - rsmall && ai > rsmall) vdwfx += aisign * bi * ci * prefac;
            if (bi < 1.0 - rsmall && bi > rsmall) vdwfy += bisign * ai * ci * prefac;
            if (ci < 1.0 - rsmall && ci > rsmall) vdwfz += cisign * ai * bi * prefac;
          }
          s.evdwgd += fi * esvdw * phis;
        }
      }
    }
    if (phisum >= s.thold8) s.warn[itype2] += 1;
    if (qforces) {
      s.fx[i] += vdwfx;
      s.fy[i] += vdwfy;
      s.fz[i] += vdwfz;
    }
  }
}

// vdwgd1spln.f90:19-173
void vdwgd1spln(State &s, bool qforces) {
  const Grid &g = s.g2;
  const int ncyz = g.ncly * g.nclz;
  s.evdwgd = 0.0;
  for (int i = 1; i <= s.ntot; ++i) {
    if (!(i <= s.nsites || i > s.nsites + s.nfix)) continue;
    bool ok = s.x[i] <= g.xbcen + g.tranx - g.dcel &&
              s.x[i] >= g.xbcen - g.tranx + g.dcel &&
              s.y[i] <= g.ybcen + g.trany - g.dcel &&
              s.y[i] >= g.ybcen - g.trany + g.dcel && s.z[i] <= s.vzmax &&
              s.z[i] >= s.vzmin;
    if (!ok) continue;
    double xi = s.x[i] + g.tranx - g.xbcen, yi = s.y[i] + g.trany - g.ybcen,
           zi = s.z[i] + g.tranz - g.zbcen;
    int ifir = 0, itype2 = 0;
    double esvdw;
    phiv_select(s, i, i > s.nsites ? std::abs(s.typei[i]) : 0, ifir, esvdw,
                itype2);
    double vdwfx = 0.0, vdwfy = 0.0, vdwfz = 0.0;
    int ix = (int)std::lround(xi * g.idcel), iy = (int)std::lround(yi * g.idcel),
        iz = (int)std::lround(zi * g.idcel);  // nint
    if (ix == 0) ix = 1;
    if (iy == 0) iy = 1;
    if (iz == 0) iz = 1;
    if (ix == g.nclx - 1) ix = g.nclx - 2;
    if (iy == g.ncly - 1) iy = g.ncly - 2;
    if (iz == g.nclz - 1) iz = g.nclz - 2;
    double phisum = 0.0;
    for (int k = ix - 1; k <= ix + 1; ++k) {
      size_t ipx = (size_t)k * ncyz;
      double ai = 1.5 - (xi - k * g.dcel) * g.idcel;
      double dai = dm3(ai);
      ai = m3(ai);
      if (!(ai != 0.0 || dai != 0.0)) continue;
      for (int l = iy - 1; l <= iy + 1; ++l) {
        size_t ipy = (size_t)l * g.nclz + ipx;
        double bi = 1.5 - (yi - l * g.dcel) * g.idcel;
        double dbi = dm3(bi);
        bi = m3(bi);
        if (!(bi != 0.0 || dbi != 0.0)) continue;
        for (int m = iz - 1; m <= iz + 1; ++m) {
          size_t ipz = m + ipy;
          double ci = 1.5 - (zi - m * g.dcel) * g.idcel;
          double dci = dm3(ci);
          ci = m3(ci);
          if (!(ci != 0.0 || dci != 0.0)) continue;
          double fi = ai * bi * ci;
          double phivi = (double)s.phiv[ifir + ipz];
          double phivsv = phivi * esvdw;
          phisum += phivi;
          if (qforces) {
            double prefac = phivsv * g.idcel;
            vdwfx += dai * bi * ci * prefac;
            vdwfy += ai * dbi * ci * prefac;
            vdwfz += ai * bi * dci * prefac;
          }
          s.evdwgd += fi * phivsv;
        }
      }
    }
    if (phisum >= s.thold27) s.warn[itype2] += 1;
    if (qforces) {
      s.fx[i] += vdwfx;
      s.fy[i] += vdwfy;
      s.fz[i] += vdwfz;
    }
  }
}

// vdwgd0trln.f90:19-118
void vdwgd0trln(State &s, double xj, double yj, double zj, int j, int jtype,
                int jtype2, bool qalert) {
  const Grid &g = s.g2;
  const int ncyz = g.ncly * g.nclz;
  s.evdwgd = 0.0;
  bool ok = xj <= g.xbcen + g.tranx && xj >= g.xbcen - g.tranx &&
            yj <= g.ybcen + g.trany && yj >= g.ybcen - g.trany &&
            zj <= s.vzmax && zj >= s.vzmin;
  if (!ok) return;
  double xi = xj + g.tranx - g.xbcen, yi = yj + g.trany - g.ybcen,
         zi = zj + g.tranz - g.zbcen;
  int ifir = 0, it2 = 0;
  double esvdw;
  phiv_select(s, j, j > s.nsites ? jtype : 0, ifir, esvdw, it2);
  if (!s.qnmcden && s.qsvdw) esvdw = s.svdw * s.scal[jtype2];
  int ix = (int)(xi * g.idcel), iy = (int)(yi * g.idcel), iz = (int)(zi * g.idcel);
  if (ix == g.nclx - 1) ix = g.nclx - 2;
  if (iy == g.ncly - 1) iy = g.ncly - 2;
  if (iz == g.nclz - 1) iz = g.nclz - 2;
  double phisum = 0.0;
  for (int n1 = ix; n1 <= ix + 1; ++n1) {
    double ai = 1.0 - std::fabs(xi - n1 * g.dcel) * g.idcel;
    for (int n2 = iy; n2 <= iy + 1; ++n2) {
      double bi = 1.0 - std::fabs(yi - n2 * g.dcel) * g.idcel;
      for (int n3 = iz; n3 <= iz + 1; ++n3) {
        double ci = 1.0 - std::fabs(zi - n3 * g.dcel) * g.idcel;
        double fi = ai * bi * ci;
        double phis =
            (double)s.phiv[(size_t)ifir + (size_t)n1 * ncyz + n2 * g.nclz + n3];
        phisum += phis;
        s.evdwgd += fi * esvdw * phis;
      }
    }
  }
  if (phisum >= s.thold8) {
    s.evdwgd = 1.0e10;
    if (qalert) s.warn[jtype2] += 1;
  }
}

// vdwgd0spln.f90:19-131 (its acceptance box has no -dcel margin)
void vdwgd0spln(State &s, double xj, double yj, double zj, int j, int jtype,
                int jtype2, bool qalert) {
  const Grid &g = s.g2;
  const int ncyz = g.ncly * g.nclz;
  s.evdwgd = 0.0;
  bool ok = xj <= g.xbcen + g.tranx && xj >= g.xbcen - g.tranx &&
            yj <= g.ybcen + g.trany && yj >= g.ybcen - g.trany &&
            zj <= s.vzmax && zj >= s.vzmin;
  if (!ok) return;
  double xi = xj + g.tranx - g.xbcen, yi = yj + g.trany - g.ybcen,
         zi = zj + g.tranz - g.zbcen;
  int ifir = 0, it2 = 0;
  double esvdw;
  phiv_select(s, j, j > s.nsites ? jtype : 0, ifir, esvdw, it2);
  if (!s.qnmcden && s.qsvdw) esvdw = s.svdw * s.scal[jtype2];
  int ix = (int)std::lround(xi * g.idcel), iy = (int)std::lround(yi * g.idcel),
      iz = (int)std::lround(zi * g.idcel);
  if (ix == 0) ix = 1;
  if (iy == 0) iy = 1;
  if (iz == 0) iz = 1;
  if (ix == g.nclx - 1) ix = g.nclx - 2;
  if (iy == g.ncly - 1) iy = g.ncly - 2;
  if (iz == g.nclz - 1) iz = g.nclz - 2;
  double phisum = 0.0;
  for (int k = ix - 1; k <= ix + 1; ++k) {
    size_t ipx = (size_t)k * ncyz;
    double ai = m3(1.5 - (xi - k * g.dcel) * g.idcel);
    if (ai == 0.0) continue;
    for (int l = iy - 1; l <= iy + 1; ++l) {
      size_t ipy = (size_t)l * g.nclz + ipx;
      double bi = m3(1.5 - (yi - l * g.dcel) * g.idcel);
      if (bi == 0.0) continue;
      for (int m = iz - 1; m <= iz + 1; ++m) {
        size_t ipz = m + ipy;
        double fi = ai * bi * m3(1.5 - (zi - m * g.dcel) * g.idcel);
        if (fi != 0.0) {
          double phis = (double)s.phiv[ifir + ipz];
          phisum += phis;
          s.evdwgd += fi * esvdw * phis;
        }
      }
    }
  }
  if (phisum >= s.thold27) {
    s.evdwgd = 1.0e10;
    if (qalert) s.warn[jtype2] += 1;
  }
}

// One trilinear gather of gsrfen/greff with derivatives (rfpar.f90:97-150);
// the early exit of the n3 loop on a zero gsrfen value is kept.
static void rfpar_gather(const State &s, double xin, double yin, double zin,
                         int ifir, bool qforces, double &aux1, double &aux2,
                         double d1[3], double d2[3]) {
  const Grid &g = s.g3;
  const int ncyz = g.ncly * g.nclz;
  aux1 = aux2 = 0.0;
  d1[0] = d1[1] = d1[2] = d2[0] = d2[1] = d2[2] = 0.0;
  double xi = xin + g.tranx - g.xbcen, yi = yin + g.trany - g.ybcen,
         zi = zin + g.tranz - g.zbcen;
  int ix = (int)(xi * g.idcel), iy = (int)(yi * g.idcel), iz = (int)(zi * g.idcel);
  if (ix == g.nclx - 1) ix = g.nclx - 2;
  if (iy == g.ncly - 1) iy = g.ncly - 2;
  if (iz == g.nclz - 1) iz = g.nclz - 2;
  for (int n1 = ix; n1 <= ix + 1; ++n1) {
    double ai = xi - n1 * g.dcel;
    double aisign = fsign(1.0, ai);
    ai = 1.0 - std::fabs(ai) * g.idcel;
    for (int n2 = iy; n2 <= iy + 1; ++n2) {
      double bi = yi - n2 * g.dcel;
      double bisign = fsign(1.0, bi);
      bi = 1.0 - std::fabs(bi) * g.idcel;
      for (int n3 = iz; n3 <= iz + 1; ++n3) {
        double ci = zi - n3 * g.dcel;
        double cisign = fsign(1.0, ci);
        ci = 1.0 - std::fabs(ci) * g.idcel;
        double fi = ai * bi * ci;
        size_t in3 = (size_t)ifir + (size_t)n1 * ncyz + n2 * g.nclz + n3;
        double gaux1 = (double)s.gsrfen[in3];
        double gaux2 = s.sqrfac * (double)s.greff[in3];
        if (gaux1 == 0.0) break;
        double prefa1 = gaux1 * g.idcel, prefa2 = gaux2 * g.idcel;
        aux1 += fi * gaux1;
        aux2 += fi * gaux2;
        if (qforces) {
          if (ai < 1.0 - rsmall && ai > rsmall) {
            double aux = aisign * bi * ci;
            d1[0] -= aux * prefa1;
            d2[0] -= aux * prefa2;
          }
          if (bi < 1.0 - rsmall && bi > rsmall) {
            double aux = bisign * ai * ci;
            d1[1] -= aux * prefa1;
            d2[1] -= aux * prefa2;
          }
          if (ci < 1.0 - rsmall && ci > rsmall) {
            double aux = cisign * ai * bi;
            d1[2] -= aux * prefa1;
            d2[2] -= aux * prefa2;
          }
        }
      }
    }
  }
}

static inline bool in_g3(const State &s, double x, double y, double z) {
  const Grid &g = s.g3;
  return x <= g.xbcen + g.tranx && x >= g.xbcen - g.tranx &&
         y <= g.ybcen + g.trany && y >= g.ybcen - g.trany &&
         z <= g.zbcen + g.tranz && z >= g.zbcen - g.tranz;
}

static inline int rfpar_ifir(const State &s, int itype) {
  const Grid &g = s.g3;
  const int ncel3 = g.nclx * g.ncly * g.nclz;
  return s.qrfpsin ? 0 : s.rfpar_map_of_type[itype] * ncel3;
}

// rfpar.f90:20-228
void rfparion(State &s, bool qforces) {
  const int nion = s.ntot - s.nsites;
  std::vector<double> srfe(nion + 1, 0.0), reff(nion + 1, 0.0),
      sd1(3 * (nion + 1), 0.0), sd2(3 * (nion + 1), 0.0);
  s.erfpar = 0.0;
  for (int i = s.nsites + 1; i <= s.ntot; ++i) {
    if (!in_g3(s, s.x[i], s.y[i], s.z[i])) continue;
    int ik = i - s.nsites;
    int itype = std::abs(s.typei[i]);
    double aux1, aux2;
    rfpar_gather(s, s.x[i], s.y[i], s.z[i], rfpar_ifir(s, itype), qforces,
                 aux1, aux2, &sd1[3 * ik], &sd2[3 * ik]);
    srfe[ik] = aux1;
    reff[ik] = aux2;
    if (ik <= s.nfix) continue;
    double tau = s.celec * s.cg[itype];
    double aux = tau * s.cg[itype] * srfe[ik];
    s.erfpar += 0.5 * aux * srfe[ik];
    if (qforces) {
      double de = -aux;
      s.fx[i] += de * sd1[3 * ik + 0];
      s.fy[i] += de * sd1[3 * ik + 1];
      s.fz[i] += de * sd1[3 * ik + 2];
    }
    for (int j = 1 + s.nsites; j <= i - 1; ++j) {
      int jk = j - s.nsites;
      if (srfe[jk] == 0.0) continue;
      int jtype = std::abs(s.typei[j]);
      double dxj = s.x[j] - s.x[i], dyj = s.y[j] - s.y[i], dzj = s.z[j] - s.z[i];
      double dist2 = dxj * dxj + dyj * dyj + dzj * dzj;
      double srfeij = srfe[jk] * srfe[ik];
      double reffij = reff[jk] * reff[ik];
      double rfdn = 1.0 / std::sqrt(reffij * reffij + dist2);
      double rfcf = reffij * rfdn;
      double aux0 = tau * s.cg[jtype];
      double a1 = aux0 * rfcf;
      s.erfpar += a1 * srfeij;
      if (qforces) {
        double a2 = aux0 * srfeij * rfdn * rfdn * rfdn;
        double de = -a1 * srfe[ik];
        s.fx[j] += de * sd1[3 * jk + 0];
        s.fy[j] += de * sd1[3 * jk + 1];
        s.fz[j] += de * sd1[3 * jk + 2];
        de = -a1 * srfe[jk];
        s.fx[i] += de * sd1[3 * ik + 0];
        s.fy[i] += de * sd1[3 * ik + 1];
        s.fz[i] += de * sd1[3 * ik + 2];
        double aux3 = -a2 * (dist2 + reff[jk] * reff[ik] * 0.5);
        de = aux3 * reff[ik];
        s.fx[j] += de * sd2[3 * jk + 0];
        s.fy[j] += de * sd2[3 * jk + 1];
        s.fz[j] += de * sd2[3 * jk + 2];
        de = aux3 * reff[jk];
        s.fx[i] += de * sd2[3 * ik + 0];
        s.fy[i] += de * sd2[3 * ik + 1];
        s.fz[i] += de * sd2[3 * ik + 2];
        de = a2 * reffij;
        s.fx[j] += de * dxj;
        s.fy[j] += de * dyj;
        s.fz[j] += de * dzj;
        s.fx[i] -= de * dxj;
        s.fy[i] -= de * dyj;
        s.fz[i] -= de * dzj;
      }
    }
  }
}

// rfpar.f90:232-369
void rfparionj(State &s, double xj, double yj, double zj, int j, int jtype) {
  s.erfpar = 0.0;
  if (!in_g3(s, xj, yj, zj)) return;
  const int ntot = s.ntot;  // includes the trial slot on insertion
  const int nion = ntot - s.nsites;
  std::vector<double> srfe(nion + 1, 0.0), reff(nion + 1, 0.0);
  double dd1[3], dd2[3];
  for (int i = s.nsites + 1; i <= ntot; ++i) {
    int ik = i - s.nsites;
    double aux1 = 0.0, aux2 = 0.0;
    int itype;
    double px, py, pz;
    bool ok;
    if (i == j) {
      itype = jtype;
      px = xj;
      py = yj;
      pz = zj;
      ok = true;
    } else {
      itype = std::abs(s.typei[i]);
      px = s.x[i];
      py = s.y[i];
      pz = s.z[i];
      ok = in_g3(s, px, py, pz);
    }
    if (ok)
      rfpar_gather(s, px, py, pz, rfpar_ifir(s, itype), false, aux1, aux2, dd1,
                   dd2);
    srfe[ik] = aux1;
    reff[ik] = aux2;
  }
  double tau = s.celec * s.cg[jtype];
  int jk = j - s.nsites;
  s.erfpar += 0.5 * tau * s.cg[jtype] * srfe[jk] * srfe[jk];
  for (int i = s.nsites + 1; i <= ntot; ++i) {
    if (i == j) continue;
    int ik = i - s.nsites;
    if (srfe[ik] == 0.0) continue;
    int itype = std::abs(s.typei[i]);
    double dist2 = (s.x[i] - xj) * (s.x[i] - xj) + (s.y[i] - yj) * (s.y[i] - yj) +
                   (s.z[i] - zj) * (s.z[i] - zj);
    double reffij = reff[jk] * reff[ik];
    s.erfpar += tau * s.cg[itype] * reffij * srfe[jk] * srfe[ik] /
                std::sqrt(reffij * reffij + dist2);
  }
}

// interact.f90:19-419
void interact(State &s, uint32_t mask, double &dener, double xj, double yj,
              double zj, int jtype, int j, bool qalert) {
  dener = 0.0;
  const bool beion = s.qpar() && j > s.nsites;
  const int jtype2 = beion ? s.nwtype[jtype] : s.typtyp[j];
  const bool Qmemb = (mask & BROMOC_M_MEMB) && s.qmemb;
  const bool Qphix = (mask & BROMOC_M_PHIX) && s.qphix;
  const bool Qphiv = (mask & BROMOC_M_PHIV) && s.qphiv;
  const bool Qrfpar = (mask & BROMOC_M_RFPAR) && s.qrfpar;
  const bool Qnonbond = (mask & BROMOC_M_NONBOND) != 0;
  if (Qmemb) {
    s.ememb = 0.0;
    if (s.voltage != 0.0) {
      double charge = 0.0;
      if (beion)
        charge = s.cg[jtype];
      else if (s.qnucl())
        charge = s.sitecharge[j];
      if (charge != 0.0) {
        if (zj < s.zmemb1)
          s.ememb += charge * s.afact * std::exp(s.ikappa * (zj - s.zmemb1));
        else if (zj >= s.zmemb1 && zj <= s.zmemb2)
          s.ememb += charge * s.afact * (s.ceps * s.ikappa * (zj - s.zmemb1) + 1.0);
        else if (zj > s.zmemb2)
          s.ememb += charge * (s.voltage - s.afact * std::exp(-s.ikappa * (zj - s.zmemb2)));
      }
    }
    if (s.ampl1[jtype2] > 0.0) {
      double sw1, dsw1;
      switch1(sw1, dsw1, zj, s.p1a[jtype2], s.p1b[jtype2], s.zmemb1, s.zmemb2);
      if (sw1 != 0.0) {
        if (s.qpore) {
          double r2 = xj * xj + yj * yj, sw2, dsw2, r = 0.0;
          switch2(sw2, dsw2, r2, s.rcylinder[jtype2], s.p2a[jtype2],
                  s.p2b[jtype2], r);
          if (sw2 != 0.0) {
            if (sw1 == 1.0) {
              if (sw2 == 1.0) {
                if (qalert) s.warn[jtype2] += 1;
                s.ememb += 1.0e10;
              } else {
                s.ememb += s.ampl2[jtype2] * sw2;
              }
            } else {
              if (sw2 == 1.0)
                s.ememb += s.ampl1[jtype2] * sw1;
              else
                s.ememb += 0.5 * (s.ampl2[jtype2] * sw2 + s.ampl1[jtype2] * sw1);
            }
          }
        } else {
          if (sw1 == 1.0) {
            if (qalert) s.warn[jtype2] += 1;
            s.ememb += 1.0e10;
          } else {
            s.ememb += s.ampl1[jtype2] * sw1;
          }
        }
      }
    }
    dener = s.ememb;
  }
  // interact.f90:121-141 (the ntot bump of an insertion trial is the
  // j == ntot + 1 case of mmij_interact)
  if ((mask & BROMOC_M_MMIJ) && s.mm.on) {
    s.egsbpb = mmij_interact(s, xj, yj, zj, j, jtype);
    dener += s.egsbpb;
  }
  if (Qrfpar) {
    if (j == s.ntot + 1) {
      s.ntot += 1;
      rfparionj(s, xj, yj, zj, j, jtype);
      s.ntot -= 1;
    } else {
      rfparionj(s, xj, yj, zj, j, jtype);
    }
    dener += s.erfpar;
    s.egsbpb = s.erfpar;
  }
  if (Qphix) {
    staticf0(s, xj, yj, zj, j, jtype);
    dener += s.egsbpa;
  }
  if (Qphiv) {
    if (s.qtrln)
      vdwgd0trln(s, xj, yj, zj, j, jtype, jtype2, qalert);
    else
      vdwgd0spln(s, xj, yj, zj, j, jtype, jtype2, qalert);
    dener += s.evdwgd;
  }
  if (beion && Qnonbond) {
    for (int i = s.nsites + 1; i <= s.ntot; ++i) {
      if (i == j) continue;
      int itype2 = s.nwtype[std::abs(s.typei[i])];
      int is = nindex(s, itype2, jtype2);
      double ddx = s.x[i] - xj, ddy = s.y[i] - yj, ddz = s.z[i] - zj;
      s.min_image(ddx, ddy, ddz);  // extension mode only
      double dist2 = ddx * ddx + ddy * ddy + ddz * ddz;
      if (s.periodic && dist2 >= s.rcut2) continue;
      if (s.qefpot[is]) {
        double eefp, dist;
        gety(s, is, dist2, eefp, dist);
        dener += eefp;
      } else {
        double idist2 = 1.0 / dist2, idist = 0.0;
        if (s.qchr[is] || s.qsrpmfi[is]) idist = std::sqrt(idist2);
        if (s.qchr[is]) dener += s.fct[is] * idist;
        if (s.qlj[is]) {
          double dist6 = pow3(s.sgp2[is] * idist2);
          dener += s.epp4[is] * dist6 * (dist6 - 1.0);
        }
        if (s.qsrpmfi[is] && dist2 <= s.rth) {
          double dist = 1.0 / idist;
          double e = s.c0[is] * std::exp((s.c1[is] - dist) * s.c2[is]) *
                         std::cos(s.c3[is] * pi * (s.c1[is] - dist)) +
                     s.c4[is] * pow6(s.c1[is] * idist);
          // interact.f90:200 tapers as e*exp(-k(r-x)) - y (energy.mono.f90
          // multiplies by (exp(-k(r-x)) - y)); kept as in the reference.
          if (dist >= s.srpx) e = e * std::exp(-s.srpk * (dist - s.srpx)) - s.srpy;
          dener += e;
        }
      }
    }
  }
  // DNA bonded and Go-like terms of site j: interact.f90:211-334
  if (s.qnucl() && !beion) nucl_interact(s, mask, j, dener);
  if (s.qpar() && s.qnucl() && Qnonbond) {
    auto pairlaw = [&](int is, double dist2) {
      if (s.qefpot[is]) {
        double eefp, dist;
        gety(s, is, dist2, eefp, dist);
        dener += eefp;
        return;
      }
      double idist2 = 1.0 / dist2, idist = 0.0;
      if (s.qchr[is] || s.qsrpmfi[is]) idist = std::sqrt(idist2);
      if (s.qchr[is]) dener += s.fct[is] * idist;
      if (s.qlj[is]) {
        double dist6 = pow3(s.sgp2[is] * idist2);
        dener += s.epp4[is] * dist6 * (dist6 - 1.0);
      }
      if (s.qsrpmfi[is] && dist2 <= s.rth) {
        double dist = 1.0 / idist;
        double e = s.c0[is] * std::exp((s.c1[is] - dist) * s.c2[is]) *
                       std::cos(s.c3[is] * pi * (s.c1[is] - dist)) +
                   s.c4[is] * pow6(s.c1[is] * idist);
        if (dist >= s.srpx) e = e * std::exp(-s.srpk * (dist - s.srpx)) - s.srpy;
        dener += e;
      }
    };
    if (beion) {
      for (int i = 1; i <= s.nsites; ++i) {
        int is = nindex(s, s.typtyp[i], jtype2);
        double dist2 = (s.x[i] - xj) * (s.x[i] - xj) +
                       (s.y[i] - yj) * (s.y[i] - yj) +
                       (s.z[i] - zj) * (s.z[i] - zj);
        pairlaw(is, dist2);
      }
    } else {
      for (int i = s.nsites + 1; i <= s.ntot; ++i) {
        int is = nindex(s, s.nwtype[std::abs(s.typei[i])], jtype2);
        double dist2 = (s.x[i] - xj) * (s.x[i] - xj) +
                       (s.y[i] - yj) * (s.y[i] - yj) +
                       (s.z[i] - zj) * (s.z[i] - zj);
        pairlaw(is, dist2);
      }
    }
  }
}

}  // namespace bref
